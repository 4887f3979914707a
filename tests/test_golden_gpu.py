"""The engine against the committed golden traces (tests/golden/day_phase_traces.json).

The traces are the oracle's (tests/golden/make_golden.py): per-tick spike
counts, the SHA-256 of the whole spike raster and of the final .state and
.axons bytes, for three seeded brains (a small one, one with adaptive leak,
homeostasis, heartbeat and dopamine, and the 16k-neuron configuration over
300 ticks).  Here the GPU engine runs the same ticks through the batch entry
point (every neuron read out every tick) and through the per-tick entry point,
and must reproduce every hash.
"""
import ctypes as C
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from test_golden_cpu import golden_cases

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "day_phase_traces.json").read_text())


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


@pytest.mark.parametrize("path", ["batch", "per_tick"])
@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_engine_reproduces_golden_trace(gpu, name, path):
    cases, _ = golden_cases()
    w, g = cases[name], GOLDEN[name]
    lay, state, heads = S.generate_brain(w.spec())
    Np, A = lay.padded_n, lay.total_axons
    S.upload_lut(w.lut)
    vram = S.VramState(Np, A)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    words = (w.num_inputs + 31) // 32
    bm = S.input_bitmask(w.seed, 0, w.ticks, w.num_inputs, w.rate_q32)
    ids = np.arange(Np, dtype=np.uint32)
    d_ids = S.device_array(ids)
    out = np.zeros(w.ticks * Np, np.uint8)
    lib = N.lib()
    try:
        if path == "batch":
            batch = 20 if w.ticks % 20 == 0 else w.ticks
            eng = S.ShardEngine(vram)
            io = S.IoDeviceBuffers(words, 0, Np, batch)
            for t0 in range(0, w.ticks, batch):
                part = np.zeros(batch * Np, np.uint8)
                eng.step_day_phase_batch(batch, io, bm[t0 * words:(t0 + batch) * words], None, None,
                                         lay.virtual_offset, w.num_inputs, d_ids, w.v_seg, w.dopamine, t0,
                                         h_output_history=part)
                out[t0 * Np:(t0 + batch) * Np] = part
            eng.synchronize()
        else:
            d_out = lib.gpu_malloc(Np)
            d_bm = S.device_array(bm)
            try:
                for k in range(w.ticks):
                    assert lib.cu_step_day_phase(C.byref(vram.ptrs), Np, A, w.v_seg, k, d_bm + k * words * 4,
                                                 lay.virtual_offset, w.num_inputs, None, 0, d_ids, d_out, Np,
                                                 w.dopamine, None) == 0
                    row = np.zeros(Np, np.uint8)
                    assert lib.gpu_memcpy_device_to_host(N.ptr(row), d_out, Np)
                    out[k * Np:(k + 1) * Np] = row
            finally:
                lib.gpu_free(d_out)
                lib.gpu_free(d_bm)
        raster = np.packbits(out.reshape(w.ticks, Np), axis=1, bitorder="little")
        counts = np.unpackbits(raster, axis=1, bitorder="little").sum(1)
        assert counts.tolist() == g["spike_counts"], f"{name}/{path}: spike counts differ"
        assert _sha(raster) == g["raster_sha256"], f"{name}/{path}: raster differs"
        assert _sha(vram.download_state()) == g["final_state_sha256"], f"{name}/{path}: final state differs"
        assert _sha(vram.download_heads()) == g["final_heads_sha256"], f"{name}/{path}: final heads differ"
        assert vram.error_flags() == 0
    finally:
        lib.gpu_free(d_ids)
        vram.free()
