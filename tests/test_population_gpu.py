"""The batched population: every brain bit-exact against the same brain run
alone through the batch entry point, and against the oracle."""
import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import population as Pop
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView

pytestmark = pytest.mark.gpu


def mixed_population(count=10, seed=3):
    ws = W.population(seed=seed, count=count, ticks=40)
    for i, w in enumerate(ws):               # keep the test small: 1k .. 6k neurons
        n = int(1000 + (i * 613) % 5000)
        w.dims = W.cube_dims(n)
        w.num_inputs = max(32, n // 64)
    ws[1].lut[0]["adaptive_mode"] = 1
    ws[1].lut[0]["adaptive_leak_gain"] = 200
    ws[1].lut[0]["adaptive_leak_max"] = 300
    ws[1].lut[0]["homeostasis_penalty"] = 30
    ws[2].lut[1]["spontaneous_firing_period_ticks"] = 5
    ws[3].lut[0]["signal_propagation_length"] = 6          # mixed lengths: exact head tests
    ws[-1].dopamine = 120
    for v in (0, 1):
        ws[-1].lut[v]["d1_affinity"] = 60
        ws[-1].lut[v]["d2_affinity"] = 90
    return ws


def snapshot(b):
    return b.vram.download_state(), b.vram.download_heads()


@pytest.mark.parametrize("lanes", [8, 16])
def test_population_matches_each_brain_alone(gpu, lanes):
    ticks, tpg = 40, 10
    ws = mixed_population()
    brains = [Pop.Brain(w, ticks) for w in ws]
    pop = Pop.Population(brains)
    try:
        pop.set_schedule(lanes, 3, 2)
        pop.run(0, ticks, tpg)
        N.lib().gpu_device_synchronize()
        got = [snapshot(b) for b in brains]
        c = pop.counters()
        assert c[0] == ticks and c[3] > 0 and c[6] == 0
        for b, (gs, gh) in zip(brains, got):
            b.reset()
            b.run_alone(0, ticks, batch=10)
            rs, rh = snapshot(b)
            assert np.array_equal(gh, rh), f"{b.w.name}: heads differ"
            if not np.array_equal(gs, rs):
                a, o = StateView(gs, b.lay.padded_n), StateView(rs, b.lay.padded_n)
                bad = [f for f in ("voltage", "flags", "threshold_offset", "timers", "weights") if
                       not np.array_equal(getattr(a, f), getattr(o, f))]
                raise AssertionError(f"{b.w.name}: state differs in {bad}")
    finally:
        pop.close()
        for b in brains:
            b.free()


def test_population_against_oracle_and_tuner(gpu):
    ticks = 24
    ws = mixed_population(count=5, seed=11)
    brains = [Pop.Brain(w, ticks) for w in ws]
    pop = Pop.Population(brains)
    try:
        sc, ms = pop.tune(0, 2, None)          # 12 candidates x 2 ticks = 24 ticks, states advance exactly
        assert sc.lanes_per_neuron in (8, 16) and min(ms) > 0
        N.lib().gpu_device_synchronize()
        for b in brains:
            gs, gh = snapshot(b)
            hs, hh = b.state0.copy(), b.heads0.copy()
            oracle.run_ticks(hs, hh, b.w.lut, b.lay.padded_n, b.lay.total_axons, b.w.v_seg, 0, ticks, b.bitmask,
                             b.words, b.lay.virtual_offset, b.w.num_inputs, dopamine=b.w.dopamine)
            assert np.array_equal(gh, hh), b.w.name
            assert np.array_equal(gs, hs), b.w.name
    finally:
        pop.close()
        for b in brains:
            b.free()


def test_population_fixup_rescan(gpu):
    """A deferred-GSOP list of capacity 0 sends every deferred slot to the rescan path."""
    from test_row_engine_gpu import stress_brain
    ticks = 20
    ws = mixed_population(count=4, seed=5)
    brains = []
    for w in ws:
        b = Pop.Brain(w, ticks)
        b.lay, b.state0, b.heads0 = stress_brain(w, seed=7)
        b.reset()
        brains.append(b)
    prev = N.lib().axc_population_fix_capacity(0)
    pop = Pop.Population(brains)
    try:
        pop.run(0, ticks, 10)
        N.lib().gpu_device_synchronize()
        for b in brains:
            gs, gh = snapshot(b)
            hs, hh = b.state0.copy(), b.heads0.copy()
            oracle.run_ticks(hs, hh, b.w.lut, b.lay.padded_n, b.lay.total_axons, b.w.v_seg, 0, ticks, b.bitmask,
                             b.words, b.lay.virtual_offset, b.w.num_inputs, dopamine=b.w.dopamine)
            assert np.array_equal(gh, hh) and np.array_equal(gs, hs), b.w.name
    finally:
        N.lib().axc_population_fix_capacity(prev)
        pop.close()
        for b in brains:
            b.free()


def test_population_refuses_ticks_past_the_bitmask(gpu):
    """A run or a tuning past a brain's input bitmask is refused on the host, before any launch."""
    ticks = 20
    ws = mixed_population(count=4, seed=9)
    brains = [Pop.Brain(w, ticks) for w in ws]
    pop = Pop.Population(brains)
    try:
        with pytest.raises(RuntimeError):
            pop.run(10, 20, 10)                 # rows 10..29 of a 20-row bitmask
        with pytest.raises(RuntimeError):
            pop.tune(0, 2, None)                # 12 candidates x 2 ticks = 24 rows
        with pytest.raises(ValueError):
            brains[0].run_alone(10, 20, 10)
        pop.run(0, ticks, 10)                   # the whole bitmask: accepted
        N.lib().gpu_device_synchronize()
        assert pop.counters()[0] == ticks
    finally:
        pop.close()
        for b in brains:
            b.free()
