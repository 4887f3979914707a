"""The batch engine's neuron-major kernels, bit-exact against the oracle.

The brains are edited to reach every path of the fused GSOP: segment 0 (a
same-tick push can put a new head in the tail), segments >= 31 (exact head
test), variants whose length differs from the LUT maximum, axons owned by
two somas (two pushes per tick), and a deferred-GSOP list that is too short
(the fix-up stage rescans every spiker).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView

pytestmark = pytest.mark.gpu


def stress_brain(w, seed=1, seg_max=40, shared_axons=0.05):
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    rng = np.random.default_rng(seed)
    live = sv.targets != 0
    redo = live & (rng.random(sv.targets.shape) < 0.3)
    segs = rng.integers(0, seg_max + 1, size=redo.sum()).astype(np.uint32)
    sv.targets[redo] = (sv.targets[redo] & 0x00FFFFFF) | (segs << 24)
    n = lay.num_neurons
    share = np.nonzero(rng.random(n) < shared_axons)[0]
    sv.soma_to_axon[share] = rng.integers(0, n, size=share.size).astype(np.uint32)
    return lay, state, heads


def run_batches(w, lay, state, heads, nb=4, batch=16, dopamine=(0,), fix_cap=None, mode=1):
    lib = N.lib()
    prev_mode = lib.axc_batch_engine_mode(mode)
    prev_cap = lib.axc_row_engine_fix_capacity(fix_cap) if fix_cap is not None else None
    try:
        S.upload_lut(w.lut)
        vram = S.VramState(lay.padded_n, lay.total_axons)
        vram.upload_state(state)
        vram.upload_axon_heads(heads)
        eng = S.ShardEngine(vram)
        words = (w.num_inputs + 31) // 32
        ids = np.arange(lay.padded_n, dtype=np.uint32)
        d_ids = S.device_array(ids)
        io = S.IoDeviceBuffers(words, 0, ids.size, batch)
        h_state, h_heads = state.copy(), heads.copy()
        spikes = 0
        for b in range(nb):
            dop = dopamine[b % len(dopamine)]
            bm = S.input_bitmask(w.seed, b * batch, batch, w.num_inputs, w.rate_q32)
            out = np.zeros(batch * ids.size, np.uint8)
            eng.step_day_phase_batch(batch, io, bm, None, None, lay.virtual_offset, w.num_inputs, d_ids, w.v_seg,
                                     dop, b * batch, h_output_history=out)
            ref = np.zeros_like(out)
            err = oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, b * batch,
                                   batch, bm, words, lay.virtual_offset, w.num_inputs, mapped_soma_ids=ids,
                                   outputs=ref, dopamine=dop)
            assert np.array_equal(out, ref), f"batch {b}: raster differs at {np.nonzero(out != ref)[0][:8]}"
            gh = vram.download_heads()
            assert np.array_equal(gh, h_heads), f"batch {b}: heads differ"
            gs = vram.download_state()
            if not np.array_equal(gs, h_state):
                a, o = StateView(gs, lay.padded_n), StateView(h_state, lay.padded_n)
                bad = [f for f in ("voltage", "flags", "threshold_offset", "timers", "weights", "targets")
                       if not np.array_equal(getattr(a, f), getattr(o, f))]
                wd = np.argwhere(a.weights != o.weights)
                raise AssertionError(f"batch {b}: state differs in {bad}; weights first {wd[:4].tolist()}")
            assert vram.error_flags() == err
            spikes += int(ref.sum())
        lib.gpu_free(d_ids)
        return spikes, vram.counters()
    finally:
        lib.axc_batch_engine_mode(prev_mode)
        if prev_cap is not None:
            lib.axc_row_engine_fix_capacity(prev_cap)


@pytest.mark.parametrize("case", ["default", "adaptive_heartbeat", "mixed_lengths", "dopamine_inertia",
                                  "long_tail_cooling"])
def test_row_engine_stress(gpu, case):
    w = W.small(dims=(16, 16, 8), slots=96, inputs=64, p=0.1)
    dop = (0,)
    if case == "adaptive_heartbeat":
        w.lut[0]["adaptive_mode"] = 1
        w.lut[0]["adaptive_leak_gain"] = 250
        w.lut[0]["adaptive_leak_max"] = 350
        w.lut[0]["homeostasis_penalty"] = 40
        w.lut[0]["homeostasis_decay"] = 2
        w.lut[1]["spontaneous_firing_period_ticks"] = 6
        w.lut[1]["refractory_period"] = 0
    elif case == "mixed_lengths":
        w.lut[0]["signal_propagation_length"] = 6
        w.lut[1]["signal_propagation_length"] = 3
    elif case == "dopamine_inertia":
        for v in (0, 1):
            w.lut[v]["inertia_curve"] = np.array([128, 110, 90, 70, 60, 50, 40, 30, 20, 16, 12, 8, 6, 4, 2, 1],
                                                 np.uint8)
            w.lut[v]["d1_affinity"] = 80
            w.lut[v]["d2_affinity"] = 120
        w.w_max = 6000
        dop = (0, 150, -300, 90)
    elif case == "long_tail_cooling":
        # lengths > 16 make the cooling shift non-zero: the exact general path
        w.lut[0]["signal_propagation_length"] = 40
        w.lut[1]["signal_propagation_length"] = 40
    lay, state, heads = stress_brain(w)
    spikes, ctr = run_batches(w, lay, state, heads, dopamine=dop)
    assert spikes > 0 and ctr[4] > 0


@pytest.mark.parametrize("cap", [0, 7])
def test_row_engine_fixup_overflow_rescan(gpu, cap):
    w = W.small(dims=(16, 16, 8), slots=96, inputs=64, p=0.1)
    lay, state, heads = stress_brain(w, seed=3, seg_max=12)
    run_batches(w, lay, state, heads, fix_cap=cap)


def test_row_engine_matches_columnar_engine_and_counters(gpu):
    w = W.small(dims=(24, 24, 12), slots=100, inputs=96, p=0.05)
    lay, state, heads = S.generate_brain(w.spec())
    s_rows, c_rows = run_batches(w, lay, state, heads, nb=3, batch=20, mode=1)
    s_cols, c_cols = run_batches(w, lay, state, heads, nb=3, batch=20, mode=0)
    assert s_rows == s_cols
    assert list(c_rows[1:5]) == list(c_cols[1:5])


def test_engines_interleave_on_one_shard(gpu):
    """Batch (rows), per-tick calls, batch (columnar) on the same device state."""
    lib = N.lib()
    w = W.small(dims=(16, 16, 8), slots=64)
    lay, state, heads = stress_brain(w, seed=5)
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    io = S.IoDeviceBuffers(words, 0, 0, 10)
    h_state, h_heads = state.copy(), heads.copy()
    tick = 0
    prev = lib.axc_batch_engine_mode(1)
    try:
        for mode, use_graph in ((1, True), (1, False), (0, True), (1, True)):
            lib.axc_batch_engine_mode(mode)
            bm = S.input_bitmask(w.seed, tick, 10, w.num_inputs, w.rate_q32)
            eng.step_day_phase_batch(10, io, bm, None, None, lay.virtual_offset, w.num_inputs, None, 1, 0, tick,
                                     use_graph=use_graph)
            oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, 1, tick, 10, bm, words,
                             lay.virtual_offset, w.num_inputs)
            tick += 10
            eng.synchronize()
            assert np.array_equal(vram.download_heads(), h_heads), (mode, use_graph)
            assert np.array_equal(vram.download_state(), h_state), (mode, use_graph)
    finally:
        lib.axc_batch_engine_mode(prev)


@pytest.mark.parametrize("slots", [12, 40, 100, 110, 120])
def test_row_shapes(gpu, slots):
    """Rows that end inside a 32-slot round (single-slot tail rounds) and rows
    whose tail takes a full round."""
    w = W.small(dims=(16, 16, 8), slots=slots, inputs=64, p=0.1)
    lay, state, heads = stress_brain(w, seed=9)
    spikes, ctr = run_batches(w, lay, state, heads, nb=2, batch=16)
    assert spikes > 0 and ctr[4] > 0


@pytest.mark.parametrize("curve", ["rank0_only", "four_ranks"])
def test_frozen_weight_groups(gpu, curve):
    """Weights in ranks whose GSOP deltas are zero cannot move; the update
    pass skips such slot groups.  Weights are planted on both sides of the
    rank boundary, at +-32767 and at -32768 (which the clamp moves)."""
    w = W.small(dims=(16, 16, 8), slots=100, inputs=64, p=0.1)
    if curve == "four_ranks":
        for v in (0, 1):
            w.lut[v]["inertia_curve"] = np.array([128, 96, 64, 32] + [0] * 12, np.uint8)
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    rng = np.random.default_rng(4)
    live = sv.targets != 0
    edge = 2048 if curve == "rank0_only" else 8192
    pool = np.array([edge - 1, edge, edge + 1, edge + 300, 20000, 32767, 100, 700], np.int32)
    mag = rng.choice(pool, size=sv.weights.shape)
    sign = np.where(sv.weights < 0, -1, 1)
    neww = (sign * mag).astype(np.int16)
    neww[(rng.random(sv.weights.shape) < 0.01) & (sign < 0)] = -32768
    sv.weights[live] = neww[live]
    spikes, ctr = run_batches(w, lay, state, heads, nb=3, batch=16)
    assert spikes > 0 and ctr[4] > 0
