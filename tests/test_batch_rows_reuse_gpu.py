"""The batch path keeps its neuron-major row copy from one batch to the next.

axc_step_day_phase_batch keeps its rows from one batch to the next (written
back to the .state blob at every batch end); the device lays them out anew at
every batch while the layout misses the lit-sum criterion, then after 100,
200, 400, ... ticks (up to 1,600).
The copy must be laid out anew whenever the shard's memory or the LUT changed
between batches by any route the reference uses (shard_thread.rs:295-350:
sort-and-prune, the sprouting upload through gpu_memcpy_host_to_device;
boot.rs: state uploads; node/mod.rs: LUT hot reload), after per-tick calls,
and after axc_shard_invalidate for writes this library cannot see.  Every
batch here is compared with the oracle (physics.cu:441-495): the whole .state
blob and every axon head.
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


def mostly_frozen(w, state, N, seed=5, movable=0.04):
    """Weights at a zero-inertia rank (|w| >= 2048 with inertia_curve[1..] = 0) but for a few percent, so that
    the layouts meet the lit-sum criterion early and the device keeps the copy between layouts."""
    for v in (0, 1):
        w.lut[v]["inertia_curve"] = np.array([128] + [0] * 15, np.uint8)
    sv = StateView(state, N)
    rng = np.random.default_rng(seed)
    live = sv.targets != 0
    freeze = live & (rng.random(live.shape) >= movable)
    mag = rng.integers(2048, 3000, size=int(freeze.sum())).astype(np.int16)
    sv.weights[freeze] = np.where(sv.weights[freeze] < 0, -mag, mag).astype(np.int16)


class BatchTwin:
    def __init__(self, w, frozen=True):
        self.w = w
        self.lay, self.h_state, self.h_heads = S.generate_brain(w.spec())
        if frozen:
            mostly_frozen(w, self.h_state, self.lay.padded_n)
        self.N, self.A = self.lay.padded_n, self.lay.total_axons
        S.upload_lut(w.lut)
        self.vram = S.VramState(self.N, self.A)
        self.vram.upload_state(self.h_state)
        self.vram.upload_axon_heads(self.h_heads)
        self.eng = S.ShardEngine(self.vram)
        self.words = (w.num_inputs + 31) // 32
        self.io = S.IoDeviceBuffers(self.words, 0, 0, 20)
        self.tick = 0

    def batch(self, ticks=20):
        bm = S.input_bitmask(self.w.seed, self.tick, ticks, self.w.num_inputs, self.w.rate_q32)
        self.eng.step_day_phase_batch(ticks, self.io, bm, None, None, self.lay.virtual_offset, self.w.num_inputs,
                                      None, self.w.v_seg, 0, self.tick)
        oracle.run_ticks(self.h_state, self.h_heads, self.w.lut, self.N, self.A, self.w.v_seg, self.tick, ticks, bm,
                         self.words, self.lay.virtual_offset, self.w.num_inputs)
        self.tick += ticks
        self.eng.synchronize()
        self.compare(f"batch ending at tick {self.tick}")

    def per_tick(self, ticks):
        lib = N.lib()
        for _ in range(ticks):
            bm = S.input_bitmask(self.w.seed, self.tick, 1, self.w.num_inputs, self.w.rate_q32)
            d_bm = S.device_array(bm)
            assert lib.cu_step_day_phase(C.byref(self.vram.ptrs), self.N, self.A, self.w.v_seg, self.tick, d_bm,
                                         self.lay.virtual_offset, self.w.num_inputs, None, 0, None, None, 0, 0,
                                         None) == 0
            lib.gpu_device_synchronize()
            lib.gpu_free(d_bm)
            oracle.step(self.h_state, self.h_heads, self.w.lut, self.N, self.A, self.w.v_seg, self.tick, bm,
                        self.lay.virtual_offset, self.w.num_inputs)
            self.tick += 1
        self.compare(f"per-tick calls ending at tick {self.tick}")

    def compare(self, where):
        assert np.array_equal(self.vram.download_heads(), self.h_heads), f"{where}: heads differ"
        gs = self.vram.download_state()
        if not np.array_equal(gs, self.h_state):
            a, o = StateView(gs, self.N), StateView(self.h_state, self.N)
            bad = [f for f in ("voltage", "flags", "threshold_offset", "timers", "targets", "weights")
                   if not np.array_equal(getattr(a, f), getattr(o, f))]
            raise AssertionError(f"{where}: state differs in {bad}")

    def close(self):
        self.vram.free()


def _raw_htod(dev_ptr, host):
    cu = C.CDLL("libcuda.so.1")
    cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
    host = np.ascontiguousarray(host)
    assert cu.cuMemcpyHtoD_v2(C.c_uint64(dev_ptr), C.c_void_p(host.ctypes.data), C.c_size_t(host.nbytes)) == 0


def test_batches_on_kept_rows_through_relayouts(gpu):
    """40 batches of 20 ticks with nothing in between on a brain whose weights are frozen but for 4 %: the
    layouts meet the lit-sum criterion, so the device keeps the copy for 100 to 800 ticks between layouts,
    while GSOP keeps moving the movable weights; every batch bit-exact."""
    w = W.small(dims=(16, 16, 8), slots=80, inputs=64, p=0.1)
    t = BatchTwin(w)
    try:
        w0 = StateView(t.h_state, t.N).weights.copy()
        t.vram.counters(reset=True)
        for _ in range(40):
            t.batch()
        assert np.count_nonzero(StateView(t.h_state, t.N).weights != w0) > 100, "GSOP must move weights"
        assert t.vram.counters()[6] > 200, "the kept layouts must run the lit-sum form"
        assert t.vram.error_flags() == 0
    finally:
        t.close()


def test_batches_follow_every_external_write(gpu):
    """Between kept copies (a mostly frozen brain, so the device keeps the rows from batch to batch) the shard
    and the LUT are written by every route the reference uses; each write must send the next batch to a new
    layout."""
    lib = N.lib()
    w = W.small(dims=(16, 16, 8), slots=80, inputs=64, p=0.1)
    t = BatchTwin(w)
    rng = np.random.default_rng(17)
    try:
        t.vram.counters(reset=True)
        for _ in range(6):
            t.batch()
        assert t.vram.counters()[6] > 0, "the device must keep the copy (lit-sum ticks) before the writes"
        # 1. cu_upload_state_blob with edited weights (boot / checkpoint restore)
        sv = StateView(t.h_state, t.N)
        live = sv.targets != 0
        pick = live & (rng.random(live.shape) < 0.2)
        sv.weights[pick] = (np.sign(sv.weights[pick]) * rng.integers(1, 1500, size=pick.sum())).astype(np.int16)
        t.vram.upload_state(t.h_state)
        t.batch()
        t.batch()
        # 2. the sprouting upload: targets and weights through gpu_memcpy_host_to_device (shard_thread.rs:339-350)
        sv = StateView(t.h_state, t.N)
        cut = rng.random(t.N) < 0.1
        sv.targets[60:, cut] = 0
        sv.weights[60:, cut] = 0
        grow = np.nonzero((sv.targets[40] != 0) & (rng.random(t.N) < 0.1))[0]
        sv.targets[40, grow] = (sv.targets[40, grow] & 0xFF000000) | rng.integers(1, t.A, size=grow.size).astype(
            np.uint32)
        sv.weights[40, grow] = 300
        p = t.vram.ptrs
        assert lib.gpu_memcpy_host_to_device(p.dendrite_targets, N.ptr(np.ascontiguousarray(sv.targets)),
                                             sv.targets.nbytes)
        assert lib.gpu_memcpy_host_to_device(p.dendrite_weights, N.ptr(np.ascontiguousarray(sv.weights)),
                                             sv.weights.nbytes)
        t.batch()
        t.batch()
        # 3. Night Phase sort-and-prune (bindings.cu:450-515)
        lib.launch_sort_and_prune(C.byref(t.vram.ptrs), t.N, 120)
        lib.gpu_device_synchronize()
        oracle.sort_and_prune(t.h_state, t.h_heads, t.N, 120)
        t.compare("after sort_and_prune")
        t.batch()
        t.batch()
        # 4. a new LUT (other frozen ranks, other lengths)
        lut = t.w.lut.copy()
        for v in (0, 1):
            lut[v]["inertia_curve"] = np.array([128, 128] + [0] * 14, np.uint8)   # the 2048..4095 ranks move again
        lut[1]["signal_propagation_length"] = 3
        t.w.lut = lut
        S.upload_lut(lut)
        t.batch()
        t.batch()
        # 5. hot reload on the shard's stream (node/mod.rs:233, bindings.cu:275-282)
        lut = t.w.lut.copy()
        lut[0]["gsop_potentiation"] = 20
        lut[1]["signal_propagation_length"] = 4
        t.w.lut = lut
        lib.update_constant_memory_hot_reload(N.ptr(np.ascontiguousarray(lut)), t.eng.stream)
        t.batch()
        t.batch()
        # 6. per-tick calls between batches
        t.per_tick(6)
        t.batch()
        t.batch()
        # 7. a write this library cannot see (the driver API), announced with axc_shard_invalidate
        sv = StateView(t.h_state, t.N)
        live = sv.targets != 0
        pick = live & (rng.random(live.shape) < 0.2)
        sv.weights[pick] = (np.sign(sv.weights[pick]) * rng.integers(1, 900, size=pick.sum())).astype(np.int16)
        _raw_htod(p.dendrite_weights, np.ascontiguousarray(sv.weights))
        assert lib.axc_shard_invalidate(C.byref(t.vram.ptrs)) == 0
        t.batch()
        t.batch()
        assert t.vram.error_flags() == 0
    finally:
        S.upload_lut(w.lut)
        t.close()
