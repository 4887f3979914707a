"""The allocation-free outgoing-spike extraction against the allocating one.

axc_extract_outgoing_spikes_noalloc exists for callers that may not allocate
device memory when they extract spikes: a node loop that runs after every
batch while other shards' streams stay busy (cudaMalloc/cudaFree can
synchronize the whole device), or a deployment that reserves all of its
device memory at boot.  Its scratch is a fixed array inside the library,
shared by every call, so this test calls it twice in a row with different
sizes (the second call must not see the first call's leftovers) and checks
each result bit for bit against launch_extract_outgoing_spikes, through the
C-ABI.  It checks the property the entry point exists for: around a call,
the high-water mark of the device's current memory pool (the pool that
cudaMallocAsync draws from) stays at zero, while the allocating entry point,
run the same way as a control, moves it.  It also checks that a call beyond
the fixed limit is refused.
"""
import ctypes as C

import numpy as np
import pytest

from axicor_gb300 import _native as N
from axicor_gb300 import shard as S

pytestmark = pytest.mark.gpu

SENT = 0x80000000
CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8   # cuda.h CUmemPool_attribute


class _Pool:
    """The device's current memory pool, through the driver API (libcuda)."""

    def __init__(self, device=0):
        self.cu = C.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), device) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetMemPool(C.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, C.byref(zero)) == 0

    def used_high(self):
        v = C.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, C.byref(v)) == 0
        return v.value


def _heads(rng, A, batch_ticks, v_seg):
    h = np.full((A, 8), SENT, np.uint32)
    recent = rng.random((A, 8)) < 0.35
    h[recent] = rng.integers(0, 2 * batch_ticks * v_seg, size=recent.sum())
    stale = rng.random((A, 8)) < 0.05
    h[stale] = rng.integers(0x70000000, 0x7FFFFFFF, size=stale.sum())
    return h.reshape(-1)


def _extract(fn, d_heads, d_src, d_dst, count, batch_ticks, v_seg, capacity, pool=None):
    """Runs one extraction; with `pool`, also returns the pool's high-water mark over the call."""
    lib = N.lib()
    d_out = lib.gpu_malloc(max(capacity, 1) * 8)
    d_cnt = lib.gpu_malloc(4)
    try:
        poison = np.full(1, 0xDEADBEEF, np.uint32)
        assert lib.gpu_memcpy_host_to_device(d_cnt, N.ptr(poison), 4)
        lib.gpu_device_synchronize()
        if pool is not None:
            pool.reset_high()
        rc = fn(d_heads, d_src, d_dst, count, batch_ticks, v_seg, d_out, d_cnt, None)
        lib.gpu_device_synchronize()
        high = pool.used_high() if pool is not None else None
        cnt = np.zeros(1, np.uint32)
        assert lib.gpu_memcpy_device_to_host(N.ptr(cnt), d_cnt, 4)
        n = int(cnt[0])
        ev = np.zeros(2 * max(n, 1), np.uint32)
        if 0 < n <= capacity:
            assert lib.gpu_memcpy_device_to_host(N.ptr(ev), d_out, n * 8)
        return rc, n, ev[: 2 * n].reshape(-1, 2), high
    finally:
        lib.gpu_free(d_out)
        lib.gpu_free(d_cnt)


def test_noalloc_matches_allocating_entry_point_twice(engine_lib):
    lib = N.lib()
    pool = _Pool()
    rng = np.random.default_rng(2024)
    A = 60000
    calls = [(40000, 20, 1), (3000, 7, 2)]     # the second call uses fewer scratch blocks than the first
    for count, batch_ticks, v_seg in calls:
        heads = _heads(rng, A, batch_ticks, v_seg)
        src = rng.permutation(A)[:count].astype(np.uint32)
        src[rng.random(count) < 0.05] = SENT            # skipped entries (bindings.cu:397)
        src[rng.random(count) < 0.02] = 0xFFFFFFFF
        dst = rng.integers(0, 1 << 24, size=count).astype(np.uint32)
        d_heads, d_src, d_dst = S.device_array(heads), S.device_array(src), S.device_array(dst)
        try:
            cap = count * 8

            def allocating(*a):
                lib.launch_extract_outgoing_spikes(*a)
                return 0

            rc_a, n_a, ev_a, high_a = _extract(allocating, d_heads, d_src, d_dst, count, batch_ticks, v_seg, cap,
                                               pool)
            rc_b, n_b, ev_b, high_b = _extract(lib.axc_extract_outgoing_spikes_noalloc, d_heads, d_src, d_dst,
                                               count, batch_ticks, v_seg, cap, pool)
            assert rc_a == 0 and rc_b == 0
            assert n_a > 1000, "the inputs must produce events"
            assert n_b == n_a
            assert np.array_equal(ev_b, ev_a)
            assert high_a > 0, "control: the allocating entry point draws its scratch from the pool"
            assert high_b == 0, f"the allocation-free entry point took {high_b} bytes from the pool"
        finally:
            for p in (d_heads, d_src, d_dst):
                lib.gpu_free(p)


def test_noalloc_refuses_counts_beyond_its_fixed_scratch(engine_lib):
    lib = N.lib()
    d_cnt = lib.gpu_malloc(4)
    try:
        poison = np.full(1, 0xDEADBEEF, np.uint32)
        assert lib.gpu_memcpy_host_to_device(d_cnt, N.ptr(poison), 4)
        too_many = (1 << 20) + 1
        rc = lib.axc_extract_outgoing_spikes_noalloc(None, None, None, too_many, 20, 1, None, d_cnt, None)
        assert rc != 0
        lib.gpu_device_synchronize()
        cnt = np.zeros(1, np.uint32)
        assert lib.gpu_memcpy_device_to_host(N.ptr(cnt), d_cnt, 4)
        assert cnt[0] == 0xDEADBEEF, "a refused call must launch nothing"
    finally:
        lib.gpu_free(d_cnt)
