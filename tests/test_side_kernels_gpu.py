"""The per-batch side kernels of bindings.cu against the oracle, bit-exact:
sort-and-prune (bindings.cu:450-515), outgoing-spike extraction (:378-436),
ghost sync (:341-368) and spike telemetry (physics.cu:400-434)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView

pytestmark = pytest.mark.gpu
SENT = 0x80000000


@pytest.mark.parametrize("threshold", [0, 300, 700, 2000])
def test_sort_and_prune_matches_oracle(gpu, threshold):
    w = W.small(dims=(20, 10, 10), slots=100)
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    rng = np.random.default_rng(threshold)
    # ties, holes before the end (empty slots that sink), garbage after the first empty, burst bits
    sv.weights[:, :] = np.where(rng.random(sv.weights.shape) < 0.2, 400, sv.weights)
    holes = rng.random(sv.targets.shape) < 0.05
    sv.targets[holes] = 0
    sv.dendrite_timers[:] = rng.integers(0, 256, size=sv.dendrite_timers.shape, dtype=np.uint8)
    sv.flags[:] |= rng.integers(0, 16, size=sv.flags.shape, dtype=np.uint8)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    N.lib().launch_sort_and_prune(C.byref(vram.ptrs), lay.padded_n, threshold)
    N.lib().gpu_device_synchronize()
    h = state.copy()
    oracle.sort_and_prune(h, heads.copy(), lay.padded_n, threshold)
    g = vram.download_state()
    a, b = StateView(g, lay.padded_n), StateView(h, lay.padded_n)
    for f in ("flags", "targets", "weights", "dendrite_timers"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    # the Day Phase's early exit relies on this: no live slot after the first empty one
    t = b.targets
    first0 = np.argmax(t == 0, axis=0)
    assert all((t[first0[n]:, n] == 0).all() for n in range(0, lay.padded_n, 37) if (t[:, n] == 0).any())


@pytest.mark.parametrize("batch_ticks,v_seg", [(20, 1), (7, 2), (1, 3)])
def test_extract_outgoing_spikes_matches_oracle(gpu, batch_ticks, v_seg):
    rng = np.random.default_rng(batch_ticks)
    A, count = 5000, 3000
    heads = np.full((A, 8), SENT, np.uint32)
    m = rng.random((A, 8)) < 0.4
    heads[m] = rng.integers(0, 3 * batch_ticks * v_seg, size=m.sum())
    big = rng.random((A, 8)) < 0.05
    heads[big] = rng.integers(0x70000000, 0x80000000, size=big.sum())
    heads = heads.reshape(-1)
    src = rng.integers(0, A, size=count).astype(np.uint32)
    src[rng.random(count) < 0.05] = SENT
    src[rng.random(count) < 0.02] = 0xFFFFFFFF
    dst = rng.integers(0, 1 << 24, size=count).astype(np.uint32)
    lib = N.lib()
    d_h, d_s, d_d = S.device_array(heads), S.device_array(src), S.device_array(dst)
    d_out = lib.gpu_malloc(count * 8 * 8)
    d_cnt = lib.gpu_malloc(4)
    try:
        lib.launch_extract_outgoing_spikes(d_h, d_s, d_d, count, batch_ticks, v_seg, d_out, d_cnt, None)
        lib.gpu_device_synchronize()
        cnt = np.zeros(1, np.uint32)
        assert lib.gpu_memcpy_device_to_host(N.ptr(cnt), d_cnt, 4)
        ev = np.zeros(2 * int(cnt[0]), np.uint32)
        if cnt[0]:
            assert lib.gpu_memcpy_device_to_host(N.ptr(ev), d_out, ev.nbytes)
        ref = oracle.extract_outgoing_spikes(heads, src, dst, batch_ticks, v_seg, count * 8)
        assert int(cnt[0]) == len(ref) > 0
        assert np.array_equal(ev.reshape(-1, 2), ref)
    finally:
        for p in (d_h, d_s, d_d, d_out, d_cnt):
            lib.gpu_free(p)


def test_ghost_sync_matches_oracle(gpu):
    rng = np.random.default_rng(1)
    A = 4000
    src = rng.integers(0, 1 << 30, size=A * 8).astype(np.uint32)
    dst = rng.integers(0, 1 << 30, size=A * 8).astype(np.uint32)
    si = rng.integers(0, A, size=1500).astype(np.uint32)
    si[::17] = SENT
    si[::29] = 0xFFFFFFFF
    di = rng.permutation(A)[:1500].astype(np.uint32)
    lib = N.lib()
    d_src, d_dst, d_si, d_di = (S.device_array(x) for x in (src, dst, si, di))
    try:
        lib.launch_ghost_sync(d_src, d_dst, d_si, d_di, si.size, None)
        lib.gpu_device_synchronize()
        g = np.empty_like(dst)
        assert lib.gpu_memcpy_device_to_host(N.ptr(g), d_dst, g.nbytes)
        ref = dst.copy()
        oracle.ghost_sync(src, ref, si, di)
        assert np.array_equal(g, ref)
    finally:
        for p in (d_src, d_dst, d_si, d_di):
            lib.gpu_free(p)


def test_extract_telemetry_and_last_spikes(gpu):
    w = W.small()
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    rng = np.random.default_rng(4)
    sv.flags[:] = (sv.flags & 0xF0) | (rng.random(lay.padded_n) < 0.3)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    lib = N.lib()
    d_ids = lib.gpu_malloc(lay.padded_n * 4)
    cnt = S.PinnedBuffer(1, np.uint32)
    cnt.array[0] = 5                     # the count is appended to, as in the reference
    try:
        lib.launch_extract_telemetry(C.byref(vram.ptrs), lay.padded_n, d_ids, cnt.as_ptr(), None)
        lib.gpu_device_synchronize()
        ref = oracle.spiking_ids(sv.flags.copy())
        assert int(cnt.array[0]) == 5 + ref.size
        ids = np.empty(lay.padded_n, np.uint32)
        assert lib.gpu_memcpy_device_to_host(N.ptr(ids), d_ids, ids.nbytes)
        assert np.array_equal(ids[5:5 + ref.size], ref)
        assert np.array_equal(vram.last_spikes(), ref)
    finally:
        lib.gpu_free(d_ids)
