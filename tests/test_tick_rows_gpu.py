"""The per-tick entry point cu_step_day_phase on the row engine, bit-exact against the oracle.

cu_step_day_phase keeps a neuron-major copy of the shard's dendrites across
calls and writes GSOP's weight changes through to the .state blob, so the
shard's memory after every tick must equal the oracle's (physics.cu:441-495):
each tick here compares the readout of every neuron, the whole .state blob and
every axon head.  The copy must be rebuilt whenever the shard's memory or the
LUT changes between ticks by any route the reference uses
(shard_thread.rs:295-350: sort-and-prune, the sprouting upload through
gpu_memcpy_host_to_device; boot.rs: state uploads; node/mod.rs: LUT hot
reload), and after axc_shard_invalidate for writes this library cannot see.
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
from test_row_engine_gpu import stress_brain

pytestmark = pytest.mark.gpu


def ticks_both(tw, n, dopamine_fn=None, incoming_fn=None):
    spikes = 0
    for _ in range(n):
        k = tw.tick
        g, o, err = tw.step_both(incoming_fn(k) if incoming_fn else None, dopamine_fn(k) if dopamine_fn else None)
        assert np.array_equal(g, o), f"raster differs at tick {k}: {np.nonzero(g != o)[0][:10]}"
        tw.compare(f"tick {k}")
        spikes += int(o.sum())
    return spikes


@pytest.fixture
def tick_mode():
    lib = N.lib()
    prev = lib.axc_tick_engine_mode(1)
    yield lib
    lib.axc_tick_engine_mode(prev)


@pytest.mark.parametrize("case", ["default", "mixed_lengths", "dopamine_inertia", "long_tail_cooling"])
def test_per_tick_rows_stress(gpu, tick_mode, case):
    """Segment 0 and segments >= 31, axons owned by two somas, other variant lengths, dopamine every tick."""
    w = W.small(dims=(16, 16, 8), slots=96, inputs=64, p=0.1)
    dop = None
    if case == "mixed_lengths":
        w.lut[0]["signal_propagation_length"] = 6
        w.lut[1]["signal_propagation_length"] = 3
    elif case == "dopamine_inertia":
        for v in (0, 1):
            w.lut[v]["inertia_curve"] = np.array([128, 110, 90, 70, 60, 50, 40, 30, 20, 16, 12, 8, 6, 4, 2, 1],
                                                 np.uint8)
            w.lut[v]["d1_affinity"] = 80
            w.lut[v]["d2_affinity"] = 120
        w.w_max = 6000
        dop = lambda k: (k * 53 % 500) - 250
    elif case == "long_tail_cooling":
        w.lut[0]["signal_propagation_length"] = 40
        w.lut[1]["signal_propagation_length"] = 40
    lay, state, heads = stress_brain(w)
    tw = Twin(w, state=state, heads=heads, lay=lay)
    try:
        assert ticks_both(tw, 40, dopamine_fn=dop) > 0
        assert tw.vram.counters()[4] > 0
    finally:
        tw.close()


@pytest.mark.parametrize("cap", [0, 7])
def test_per_tick_rows_fixup_overflow(gpu, tick_mode, cap):
    """A deferred-GSOP list too short for the tick: the fix-up rescans every spiker (and writes through)."""
    lib = tick_mode
    prev = lib.axc_row_engine_fix_capacity(cap)
    w = W.small(dims=(16, 16, 8), slots=96, inputs=64, p=0.1)
    lay, state, heads = stress_brain(w, seed=3, seg_max=12)
    tw = Twin(w, state=state, heads=heads, lay=lay)
    try:
        ticks_both(tw, 30)
    finally:
        tw.close()
        lib.axc_row_engine_fix_capacity(prev)


@pytest.mark.parametrize("slots", [12, 110])
def test_per_tick_rows_shapes(gpu, tick_mode, slots):
    w = W.small(dims=(16, 16, 8), slots=slots, inputs=64, p=0.1)
    lay, state, heads = stress_brain(w, seed=9)
    tw = Twin(w, state=state, heads=heads, lay=lay)
    try:
        assert ticks_both(tw, 24) > 0
    finally:
        tw.close()


def test_per_tick_network_spikes(gpu, tick_mode):
    w = W.small()
    rng = np.random.default_rng(8)
    tw = Twin(w)
    try:
        inc = lambda k: rng.integers(0, tw.A + 40, size=int(rng.integers(0, 200))).astype(np.uint32)
        ticks_both(tw, 30, incoming_fn=inc)
    finally:
        tw.close()


def _raw_htod(dev_ptr, host):
    cu = C.CDLL("libcuda.so.1")
    cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
    host = np.ascontiguousarray(host)
    assert cu.cuMemcpyHtoD_v2(C.c_uint64(dev_ptr), C.c_void_p(host.ctypes.data), C.c_size_t(host.nbytes)) == 0


def test_per_tick_rows_follow_every_external_write(gpu, tick_mode):
    """Between ticks the shard's memory and the LUT change by every route the reference uses; after each,
    the per-tick ticks stay bit-exact (the row copy is rebuilt)."""
    lib = tick_mode
    w = W.small(dims=(16, 16, 8), slots=80, inputs=64, p=0.1)
    for v in (0, 1):   # several movable ranks, so GSOP keeps moving weights after the edits
        w.lut[v]["inertia_curve"] = np.array([128, 96, 64, 32] + [0] * 12, np.uint8)
    tw = Twin(w)
    rng = np.random.default_rng(12)
    N_ = tw.N
    try:
        ticks_both(tw, 12)
        # 1. cu_upload_state_blob with edited weights (boot / checkpoint restore)
        sv = StateView(tw.h_state, N_)
        live = sv.targets != 0
        pick = live & (rng.random(live.shape) < 0.2)
        sv.weights[pick] = (np.sign(sv.weights[pick]) * rng.integers(1, 1500, size=pick.sum())).astype(np.int16)
        tw.vram.upload_state(tw.h_state)
        ticks_both(tw, 8)
        # 2. the sprouting upload: targets and weights through gpu_memcpy_host_to_device (shard_thread.rs:339-350)
        sv = StateView(tw.h_state, N_)
        cut = rng.random(N_) < 0.1
        sv.targets[60:, cut] = 0
        sv.weights[60:, cut] = 0
        grow = np.nonzero((sv.targets[40] != 0) & (rng.random(N_) < 0.1))[0]
        sv.targets[40, grow] = (sv.targets[40, grow] & 0xFF000000) | rng.integers(1, tw.A, size=grow.size).astype(
            np.uint32)
        sv.weights[40, grow] = 300
        p = tw.vram.ptrs
        assert lib.gpu_memcpy_host_to_device(p.dendrite_targets, N.ptr(np.ascontiguousarray(sv.targets)),
                                             sv.targets.nbytes)
        assert lib.gpu_memcpy_host_to_device(p.dendrite_weights, N.ptr(np.ascontiguousarray(sv.weights)),
                                             sv.weights.nbytes)
        ticks_both(tw, 8)
        # 3. Night Phase sort-and-prune (bindings.cu:450-515)
        lib.launch_sort_and_prune(C.byref(tw.vram.ptrs), N_, 120)
        lib.gpu_device_synchronize()
        oracle.sort_and_prune(tw.h_state, tw.h_heads, N_, 120)
        tw.compare("after sort_and_prune")
        ticks_both(tw, 8)
        # 4. a new LUT (other frozen ranks, other lengths)
        lut = tw.w.lut.copy()
        for v in (0, 1):
            lut[v]["inertia_curve"] = np.array([128, 128, 100, 80, 60, 40] + [0] * 10, np.uint8)
        lut[1]["signal_propagation_length"] = 3
        tw.w.lut = lut
        S.upload_lut(lut)
        ticks_both(tw, 8)
        # 5. hot reload on the shard's stream (node/mod.rs:233, bindings.cu:275-282)
        lut = tw.w.lut.copy()
        lut[0]["gsop_potentiation"] = 20
        lut[1]["signal_propagation_length"] = 4
        tw.w.lut = lut
        lib.update_constant_memory_hot_reload(N.ptr(np.ascontiguousarray(lut)), None)
        ticks_both(tw, 8)
        # 6. a write this library cannot see (the driver API), announced with axc_shard_invalidate
        sv = StateView(tw.h_state, N_)
        live = sv.targets != 0
        pick = live & (rng.random(live.shape) < 0.2)
        sv.weights[pick] = (np.sign(sv.weights[pick]) * rng.integers(1, 900, size=pick.sum())).astype(np.int16)
        _raw_htod(p.dendrite_weights, np.ascontiguousarray(sv.weights))
        assert lib.axc_shard_invalidate(C.byref(tw.vram.ptrs)) == 0
        ticks_both(tw, 8)
    finally:
        tw.close()


def test_per_tick_interleaves_with_batches(gpu, tick_mode):
    """Per-tick calls, a graph batch, per-tick calls again on one shard, against the oracle."""
    w = W.small(dims=(16, 16, 8), slots=64)
    lay, state, heads = stress_brain(w, seed=5)
    tw = Twin(w, state=state, heads=heads, lay=lay)
    eng = S.ShardEngine(tw.vram)
    io = S.IoDeviceBuffers(tw.words, 0, 0, 20)
    try:
        ticks_both(tw, 10)
        bm = tw.bitmask(20)
        eng.step_day_phase_batch(20, io, bm, None, None, tw.voff, tw.nv, None, w.v_seg, 0, tw.tick)
        eng.synchronize()
        oracle.run_ticks(tw.h_state, tw.h_heads, w.lut, tw.N, tw.A, w.v_seg, tw.tick, 20, bm, tw.words, tw.voff,
                         tw.nv)
        tw.tick += 20
        tw.compare("after the batch")
        ticks_both(tw, 10)
    finally:
        tw.close()


@pytest.mark.parametrize("case", ["default", "dopamine_inertia"])
def test_per_tick_columnar_kernels(gpu, tick_mode, case):
    """axc_tick_engine_mode(0): the columnar per-tick kernels stay bit-exact too."""
    lib = tick_mode
    lib.axc_tick_engine_mode(0)
    w = W.small()
    dop = None
    if case == "dopamine_inertia":
        for v in (0, 1):
            w.lut[v]["inertia_curve"] = np.array([128, 120, 100, 90, 80, 70, 60, 50, 40, 30, 20, 10, 8, 6, 4, 2],
                                                 np.uint8)
            w.lut[v]["d1_affinity"] = 64
            w.lut[v]["d2_affinity"] = 96
        w.w_max = 5000
        dop = lambda k: (k * 37 % 400) - 200
    tw = Twin(w)
    try:
        assert ticks_both(tw, 30, dopamine_fn=dop) > 0
    finally:
        tw.close()
