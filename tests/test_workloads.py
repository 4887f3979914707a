"""The benchmark configurations as specified (neurons, slots, inputs, rates, LUT mapping), and the
algorithmic-bytes formula the roofline figures use."""
import math

import numpy as np

import bench
from axicor_gb300 import workloads as W


def rate(q32):
    return float(q32) / 4294967296.0


def test_config0_config1_config4_shapes():
    c0, c1, c4 = W.config0(), W.config1(), W.config4()
    assert (c0.num_neurons, c0.slots, c0.num_inputs, c0.ticks) == (16384, 128, 256, 1000)
    assert (c1.num_neurons, c1.slots, c1.num_inputs, c1.ticks) == (1507328, 100, 4096, 10000)
    assert (c4.num_neurons, c4.slots, c4.num_inputs, c4.ticks) == (8000000, 128, 8192, 5000)
    assert c1.num_neurons % 64 == 0 and c4.num_neurons % 64 == 0
    for w in (c0, c1):
        assert abs(rate(w.rate_q32[0]) - 0.05) < 1e-9 and w.rate_q32.size == 1
    # config 4: sinusoidal 0.01..0.2 over a 100-tick period
    r = np.array([rate(x) for x in c4.rate_q32])
    assert r.size == 100 and abs(r.min() - 0.01) < 1e-6 and abs(r.max() - 0.2) < 1e-3
    assert abs(r[50] - 0.2) < 1e-6 and abs(r[0] - 0.01) < 1e-6


def test_lut_mapping():
    """threshold 2000, linear leak threshold >> 4, refractory 3, length 4, GSOP +8/-4 with the
    +-2047 clamp as inertia_curve[1..15] = 0, variant 1 inhibitory."""
    lut = W.config1().lut
    for v in (0, 1):
        p = lut[v]
        assert p["threshold"] == 2000 and p["leak_rate"] == 125 and p["refractory_period"] == 3
        assert p["signal_propagation_length"] == 4
        assert p["gsop_potentiation"] == 8 and p["gsop_depression"] == 4
        assert p["inertia_curve"][0] == 128 and not p["inertia_curve"][1:].any()
    assert lut[0]["is_inhibitory"] == 0 and lut[1]["is_inhibitory"] == 1


def test_population_ranges_and_prefix_stability():
    ws = W.population(count=512)
    assert len(ws) == 512
    n = np.array([w.num_neurons for w in ws])
    assert n.min() >= 900 and n.max() <= 110000
    assert {w.slots for w in ws} <= {32, 64, 96, 128}
    for w in ws:
        p = w.lut[0]
        assert 1500 <= p["threshold"] <= 2500
        assert p["leak_rate"] in {p["threshold"] >> s for s in (3, 4, 5)}
        assert 4 <= p["gsop_potentiation"] <= 16 and 2 <= p["gsop_depression"] <= 8
        assert 0.01 - 1e-9 <= rate(w.rate_q32[0]) <= 0.1 + 1e-9
        assert w.num_inputs == max(32, w.num_neurons // 64)
    # a smaller population is the first brains of the larger one (same seeded draws)
    small = W.population(count=64)
    for a, b in zip(small, ws[:64]):
        assert a.dims == b.dims and a.slots == b.slots and a.seed == b.seed
        assert np.array_equal(a.lut, b.lut) and np.array_equal(a.rate_q32, b.rate_q32)


def test_algorithmic_bytes_formula():
    """6 B per evaluated slot, 64 B per axon, 20 B per neuron, 4 B per spike, 8 B per GSOP slot,
    4 B per input word and 6 B per output, per tick."""
    N, A, I, outs = 1507328, 1511424, 4096, 4096
    ticks, ev, spk, gs = 10, 376832 * 100 * 10, 376832 * 10, 376832 * 100 * 10
    got = bench.algorithmic_bytes(ticks, ev, spk, gs, N, A, I, outs)
    want = 6 * ev + ticks * (64 * A + 20 * N + 4 * math.ceil(I / 32) + 6 * outs) + 4 * spk + 8 * gs
    assert got == want
    per_tick = got / ticks
    assert 6.5e8 < per_tick < 6.6e8      # 656 MB per tick in the saturated steady state
    assert bench.rows_update_kernel_bytes(37683200, 376832, 376832) == 6 * 37683200 + 24 * 376832 + 4 * 376832
