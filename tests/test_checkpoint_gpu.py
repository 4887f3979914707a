"""Checkpoint and resume through the C-ABI, against running straight through.

The reference writes a checkpoint as the downloaded .state blob and
BurstHeads8 array (genesis-node/src/node/shard_thread.rs:231-265, written to
*.tmp and renamed) and prefers that pair over the baked one at boot
(genesis-node/src/boot.rs:39-97), uploading it with cu_upload_state_blob and
cu_upload_axons_blob.  A brain run k ticks, checkpointed, booted into a fresh
shard and run m more ticks must end byte for byte where the same brain run
k + m ticks straight ends, on the batch path and on the per-tick path, and
where the oracle ends.
"""
import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import formats as F
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run(vram, w, lay, bm, words, t0, t1, batch, use_graph):
    eng = S.ShardEngine(vram)
    io = S.IoDeviceBuffers(words, 0, 0, batch)
    for t in range(t0, t1, batch):
        eng.step_day_phase_batch(batch, io, bm[t * words:(t + batch) * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, w.v_seg, w.dopamine, t, use_graph=use_graph)
    eng.synchronize()


@pytest.mark.parametrize("use_graph", [True, False], ids=["batch_path", "per_tick_path"])
def test_resume_equals_straight_run(gpu, tmp_path, use_graph):
    w = W.small(dims=(16, 16, 16), slots=96, inputs=128, p=0.08)
    for v in (0, 1):   # weights keep moving across the checkpoint
        w.lut[v]["inertia_curve"] = np.array([128, 110, 90, 70] + [0] * 12, np.uint8)
    lay, state0, heads0 = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    words = (w.num_inputs + 31) // 32
    k, m, batch = 40, 60, 20
    bm = S.input_bitmask(w.seed, 0, k + m, w.num_inputs, w.rate_q32)

    straight = S.VramState(lay.padded_n, lay.total_axons)
    straight.upload_state(state0)
    straight.upload_axon_heads(heads0)
    _run(straight, w, lay, bm, words, 0, k + m, batch, use_graph)
    end_state, end_heads = straight.download_state(), straight.download_heads()
    straight.free()

    first = S.VramState(lay.padded_n, lay.total_axons)
    first.upload_state(state0)
    first.upload_axon_heads(heads0)
    _run(first, w, lay, bm, words, 0, k, batch, use_graph)
    F.write_pair(tmp_path, "shard", state0, heads0)                     # the baked pair
    F.write_pair(tmp_path, "checkpoint", first.download_state(), first.download_heads())
    first.free()
    assert not list(tmp_path.glob("*.tmp")), "checkpoint files are renamed into place"

    state, heads, stem = F.read_pair(tmp_path, lay.padded_n, lay.total_axons)
    assert stem == "checkpoint", "boot prefers the checkpoint pair (boot.rs:40-51)"
    resumed = S.VramState(lay.padded_n, lay.total_axons)
    resumed.upload_state(state)
    resumed.upload_axon_heads(heads)
    _run(resumed, w, lay, bm, words, k, k + m, batch, use_graph)
    try:
        assert np.array_equal(resumed.download_heads(), end_heads)
        assert np.array_equal(resumed.download_state(), end_state)
        h_state, h_heads = state0.copy(), heads0.copy()
        oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, 0, k + m, bm, words,
                         lay.virtual_offset, w.num_inputs, dopamine=w.dopamine)
        assert np.array_equal(h_state, end_state) and np.array_equal(h_heads, end_heads)
        assert resumed.error_flags() == 0
    finally:
        resumed.free()


def test_short_axons_checkpoint_boots_with_sentinel_tail(gpu, tmp_path):
    """A .axons file shorter than total_axons (memory.rs:156-163): the rest of the heads stay at the sentinel."""
    w = W.small()
    lay, state0, heads0 = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    h = heads0.reshape(-1, 8).copy()
    h[: lay.padded_n // 2, 0] = 3
    short = h[: lay.padded_n // 2].reshape(-1)
    F.write_pair(tmp_path, "checkpoint", state0, short)
    state, heads, _ = F.read_pair(tmp_path, lay.padded_n, lay.total_axons)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    try:
        vram.upload_state(state)
        assert N.lib().cu_upload_axons_blob(N.C.byref(vram.ptrs), N.ptr(short), short.nbytes) == 0
        got = vram.download_heads().reshape(-1, 8)
        assert np.array_equal(got[: lay.padded_n // 2], h[: lay.padded_n // 2])
        assert np.all(got[lay.padded_n // 2:] == 0x80000000)
        assert np.array_equal(got.reshape(-1), heads)
    finally:
        vram.free()
