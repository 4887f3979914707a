"""A shard's first batch on a non-blocking stream while the legacy stream is busy.

The reference runs every shard on its own non-blocking stream
(genesis-compute/src/compute/shard.rs:28-36) while the node loop issues work
on the legacy stream (ghost sync, genesis-node/src/node/mod.rs:409-420).  The
engine's per-shard scratch (row copy, per-tick counts) is created on a
shard's first batch; it must be zeroed in the order of that batch's stream.
A memset on the legacy stream would wait behind the legacy stream's queue and
land in the middle of the batch when the allocator hands back cached memory
without synchronizing the device.  So the allocator is first given memory to
cache (a large buffer filled with non-zero bytes and freed), the legacy
stream is kept busy with another brain's per-tick steps, and a fresh shard's
first batches run on a non-blocking stream against the oracle.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_first_batch_on_nonblocking_stream_while_legacy_stream_busy(gpu):
    lib = N.lib()
    # memory for the allocator to hand back: non-zero bytes, freed
    junk_bytes = 1 << 30
    junk = lib.gpu_malloc(junk_bytes)
    assert junk
    pattern = np.full(1 << 26, 0xA5, np.uint8)
    for off in range(0, junk_bytes, pattern.nbytes):
        assert lib.gpu_memcpy_host_to_device(junk + off, N.ptr(pattern), pattern.nbytes)
    lib.gpu_free(junk)

    busy_w = W.small(dims=(64, 64, 32), slots=100, inputs=256, p=0.05, seed=71)
    blay, bstate, bheads = S.generate_brain(busy_w.spec())
    w = W.small(dims=(48, 48, 24), slots=96, inputs=128, p=0.08, seed=72)
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)                       # both brains use the default LUT
    busy = S.VramState(blay.padded_n, blay.total_axons)
    busy.upload_state(bstate)
    busy.upload_axon_heads(bheads)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    bwords = (busy_w.num_inputs + 31) // 32
    bbm = S.input_bitmask(busy_w.seed, 0, 60, busy_w.num_inputs, busy_w.rate_q32)
    d_bbm = S.device_array(bbm)
    io = S.IoDeviceBuffers(words, 0, 0, 50)
    try:
        for k in range(60):   # queued on the legacy stream, not waited for
            assert lib.cu_step_day_phase(C.byref(busy.ptrs), blay.padded_n, blay.total_axons, 1, k,
                                         d_bbm + k * bwords * 4, blay.virtual_offset, busy_w.num_inputs, None, 0,
                                         None, None, 0, 0, None) == 0
        for b in range(2):
            bm = S.input_bitmask(w.seed, b * 50, 50, w.num_inputs, w.rate_q32)
            eng.step_day_phase_batch(50, io, bm, None, None, lay.virtual_offset, w.num_inputs, None, w.v_seg, 0,
                                     b * 50)
            oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, b * 50, 50, bm, words,
                             lay.virtual_offset, w.num_inputs)
        eng.synchronize()
        lib.gpu_device_synchronize()
        assert np.array_equal(vram.download_heads(), heads)
        assert np.array_equal(vram.download_state(), state)
    finally:
        lib.gpu_free(d_bbm)
        busy.free()
        vram.free()
