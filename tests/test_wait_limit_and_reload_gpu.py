"""The update pass's bounded wait running out, and LUT hot reload between batches.

- The update pass stages the tick's fully-lit bitmap in shared memory by one
  bulk copy and waits for it on an mbarrier with a bounded number of tries.
  axc_row_engine_wait_limit(0) makes that first wait give up at once: the
  pass must set AXC_ERR_WAIT_LIMIT, run without the bitmap and leave a state
  bit-exact against the oracle (the drain wait before the block exits keeps
  its full limit, so the copy lands before the block ends).  Nothing hangs:
  the copy is a local bulk copy that completes whether or not it is waited
  for.
- update_constant_memory_hot_reload (bindings.cu:275-282, called between
  batches by node/mod.rs:233) replaces the LUT on the shard's stream between
  two batches of the batch path; the ticks after it follow the new LUT.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _shard(w):
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    return lay, state, heads, vram, S.ShardEngine(vram)


def test_bitmap_wait_gives_up_and_state_stays_exact(gpu):
    lib = N.lib()
    w = W.small(dims=(16, 16, 8), slots=64, inputs=64, p=0.1)
    lay, h_state, h_heads, vram, eng = _shard(w)
    words = (w.num_inputs + 31) // 32
    ids = np.arange(lay.padded_n, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, ids.size, 16)
    prev = lib.axc_row_engine_wait_limit(0)
    try:
        assert vram.error_flags() == 0
        tick = 0
        for b in range(3):
            bm = S.input_bitmask(w.seed, tick, 16, w.num_inputs, w.rate_q32)
            out = np.zeros(16 * ids.size, np.uint8)
            eng.step_day_phase_batch(16, io, bm, None, None, lay.virtual_offset, w.num_inputs, d_ids, w.v_seg, 0,
                                     tick, h_output_history=out)
            ref = np.zeros_like(out)
            oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick, 16, bm, words,
                             lay.virtual_offset, w.num_inputs, mapped_soma_ids=ids, outputs=ref)
            tick += 16
            assert np.array_equal(out, ref), f"batch {b}: raster differs"
            assert np.array_equal(vram.download_heads(), h_heads), f"batch {b}: heads differ"
            assert np.array_equal(vram.download_state(), h_state), f"batch {b}: state differs"
        assert vram.error_flags(clear=True) & N.ERR_WAIT_LIMIT, "the wait that gave up must say so"
        # the per-tick entry point takes the same pass
        for k in range(8):
            bm = S.input_bitmask(w.seed, tick, 1, w.num_inputs, w.rate_q32)
            d_bm = S.device_array(bm)
            assert lib.cu_step_day_phase(C.byref(vram.ptrs), lay.padded_n, lay.total_axons, w.v_seg, tick, d_bm,
                                         lay.virtual_offset, w.num_inputs, None, 0, None, None, 0, 0, None) == 0
            lib.gpu_device_synchronize()
            lib.gpu_free(d_bm)
            oracle.step(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick, bm,
                        lay.virtual_offset, w.num_inputs)
            tick += 1
        assert np.array_equal(vram.download_heads(), h_heads)
        assert np.array_equal(vram.download_state(), h_state)
        assert vram.error_flags(clear=True) & N.ERR_WAIT_LIMIT
        # with the default limit the bitmap arrives in time and no bit is raised
        lib.axc_row_engine_wait_limit(prev)
        bm = S.input_bitmask(w.seed, tick, 16, w.num_inputs, w.rate_q32)
        eng.step_day_phase_batch(16, io, bm, None, None, lay.virtual_offset, w.num_inputs, None, w.v_seg, 0, tick)
        oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick, 16, bm, words,
                         lay.virtual_offset, w.num_inputs)
        eng.synchronize()
        assert np.array_equal(vram.download_state(), h_state)
        assert vram.error_flags() == 0
    finally:
        lib.axc_row_engine_wait_limit(prev)
        lib.gpu_free(d_ids)
        vram.free()


def test_hot_reload_between_batches(gpu):
    lib = N.lib()
    w = W.small(dims=(16, 16, 8), slots=80, inputs=64, p=0.1)
    lay, h_state, h_heads, vram, eng = _shard(w)
    words = (w.num_inputs + 31) // 32
    io = S.IoDeviceBuffers(words, 0, 0, 20)
    luts = [w.lut]
    l2 = w.lut.copy()
    for v in (0, 1):
        l2[v]["inertia_curve"] = np.array([128, 100, 80, 60] + [0] * 12, np.uint8)
        l2[v]["gsop_potentiation"] = 14
        l2[v]["homeostasis_penalty"] = 30
        l2[v]["homeostasis_decay"] = 3
    l2[1]["signal_propagation_length"] = 6
    luts.append(l2)
    l3 = l2.copy()
    l3[0]["leak_rate"] = 60
    l3[1]["signal_propagation_length"] = 4
    luts.append(l3)
    try:
        tick = 0
        for i, lut in enumerate(luts):
            if i:
                lut_c = np.ascontiguousarray(lut)
                lib.update_constant_memory_hot_reload(N.ptr(lut_c), eng.stream)
            for _ in range(2):
                bm = S.input_bitmask(w.seed, tick, 20, w.num_inputs, w.rate_q32)
                eng.step_day_phase_batch(20, io, bm, None, None, lay.virtual_offset, w.num_inputs, None, w.v_seg,
                                         0, tick)
                oracle.run_ticks(h_state, h_heads, lut, lay.padded_n, lay.total_axons, w.v_seg, tick, 20, bm, words,
                                 lay.virtual_offset, w.num_inputs)
                tick += 20
                eng.synchronize()
                assert np.array_equal(vram.download_heads(), h_heads), f"LUT {i}: heads differ at tick {tick}"
                assert np.array_equal(vram.download_state(), h_state), f"LUT {i}: state differs at tick {tick}"
    finally:
        S.upload_lut(w.lut)
        vram.free()
