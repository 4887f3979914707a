"""The row engine's lit-sum form, bit-exact against the oracle.

Once most weights are frozen (GSOP cannot move them) and most axons are fully
lit, the row copy puts each row's frozen slots on fully-lit axons (segments
1..30, variant length = the LUT maximum) last and sums their weights once per
row; a tick whose every such axon is still fully lit adds that sum and tests
only the other slots, one thread per evaluated neuron.  Any tick with an axon
that has left the fully-lit set takes the full 8-lane pass.  These brains start
with frozen weights so the form is reached within a few ticks, and carry the
slots the form must leave to the per-tick test: movable weights, segment 0, a
second variant length, axons owned by two somas.  (Segments >= 31 are left
out: a fully-lit axon must cover segments 1..min(largest segment, 30) with
seven 4-segment tails, which a brain whose slots reach segment 31 never does;
the full pass's handling of them is covered by the row-engine tests.)  A LUT
with a higher threshold then silences part of the brain mid-run, so axons leave
the fully-lit set inside a batch and ticks fall back to the full pass.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView
from helpers import Twin

pytestmark = pytest.mark.gpu


def frozen_brain(seed=3, mixed_lengths=False):
    w = W.small(dims=(24, 24, 12), slots=96, inputs=96, p=0.08, seed=seed)
    w.w_min, w.w_max = 2100, 2900           # rank >= 1: frozen under inertia_curve[1..15] = 0
    if mixed_lengths:   # inhibitory neurons (3 % here) test every slot: their length is not the LUT maximum
        w.lut[1]["signal_propagation_length"] = 3
        w.inhibitory_permille = 30
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    rng = np.random.default_rng(seed)
    live = sv.targets != 0
    small = live & (rng.random(live.shape) < 0.02)          # movable weights
    sv.weights[small] = (np.sign(sv.weights[small]) * rng.integers(50, 800, size=small.sum())).astype(np.int16)
    odd = live & (rng.random(live.shape) < 0.01)            # segment 0
    sv.targets[odd] = sv.targets[odd] & 0x00FFFFFF
    n = lay.num_neurons
    share = np.nonzero(rng.random(n) < 0.01)[0]              # axons owned by two somas
    sv.soma_to_axon[share] = rng.integers(0, n, size=share.size).astype(np.uint32)
    return w, lay, state, heads


def silencing_lut(lut):
    """Excitatory neurons never reach threshold: their axons leave the fully-lit set within ~28 ticks."""
    quiet = lut.copy()
    quiet[0]["threshold"] = 1 << 30
    return quiet


@pytest.mark.parametrize("mixed_lengths", [False, True])
def test_lit_sum_batches(gpu, mixed_lengths):
    lib = N.lib()
    w, lay, h_state, h_heads = frozen_brain(mixed_lengths=mixed_lengths)
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(h_state)
    vram.upload_axon_heads(h_heads)
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    ids = np.arange(lay.padded_n, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, ids.size, 16)
    tick, lit_ticks = 0, []
    try:
        for phase, lut in (("saturated", w.lut), ("silenced", silencing_lut(w.lut))):
            if phase == "silenced":
                S.upload_lut(lut)
            vram.counters(reset=True)
            for b in range(6):
                bm = S.input_bitmask(w.seed, tick, 16, w.num_inputs, w.rate_q32)
                out = np.zeros(16 * ids.size, np.uint8)
                eng.step_day_phase_batch(16, io, bm, None, None, lay.virtual_offset, w.num_inputs, d_ids, w.v_seg,
                                         0, tick, h_output_history=out)
                ref = np.zeros_like(out)
                oracle.run_ticks(h_state, h_heads, lut, lay.padded_n, lay.total_axons, w.v_seg, tick, 16, bm, words,
                                 lay.virtual_offset, w.num_inputs, mapped_soma_ids=ids, outputs=ref)
                assert np.array_equal(out, ref), f"{phase} batch {b}: raster differs"
                assert np.array_equal(vram.download_heads(), h_heads), f"{phase} batch {b}: heads differ"
                assert np.array_equal(vram.download_state(), h_state), f"{phase} batch {b}: state differs"
                tick += 16
            lit_ticks.append(int(vram.counters()[6]))
        assert lit_ticks[0] > 32, f"the saturated brain must reach the lit-sum form ({lit_ticks})"
        assert lit_ticks[1] < 96, f"silencing must send ticks to the full pass ({lit_ticks})"
    finally:
        S.upload_lut(w.lut)
        lib.gpu_free(d_ids)
        vram.free()


def test_lit_sum_per_tick_entry_point(gpu):
    """cu_step_day_phase with the lit-sum form: the row copy is laid out again every 64 calls."""
    lib = N.lib()
    prev = lib.axc_tick_engine_mode(1)
    w, lay, state, heads = frozen_brain(seed=5)
    tw = Twin(w, state=state, heads=heads, lay=lay)
    try:
        tw.vram.counters(reset=True)
        for k in range(150):
            g, o, err = tw.step_both()
            assert np.array_equal(g, o), f"raster differs at tick {k}"
            if k % 10 == 9:
                tw.compare(f"tick {k}")
        assert int(tw.vram.counters()[6]) > 40
        quiet = silencing_lut(w.lut)
        w.lut = quiet
        S.upload_lut(quiet)
        for k in range(150, 190):
            g, o, err = tw.step_both()
            assert np.array_equal(g, o), f"raster differs at tick {k}"
        tw.compare("end")
    finally:
        S.upload_lut(W.default_lut())
        tw.close()
        lib.axc_tick_engine_mode(prev)
