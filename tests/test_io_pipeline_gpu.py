"""Double-buffered batch I/O (axc_io_pipeline_*) against the oracle.

Batches are queued back to back from one pinned host array: each submit
returns before its batch ran, the readout of batch b is collected after batch
b + 1 was queued (one batch behind, as the overlap intends), and every
readout and the final state must equal the oracle's
(genesis-node/src/node/shard_thread.rs:208-227 reads the same outputs after a
synchronous batch).
"""
import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_pipelined_batches_match_oracle(gpu):
    lib = N.lib()
    w = W.small(dims=(16, 16, 8), slots=64, inputs=64, p=0.1)
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    batch, nb = 16, 7
    words = (w.num_inputs + 31) // 32
    ids = np.arange(0, lay.padded_n, 3, dtype=np.uint32)
    d_ids = S.device_array(ids)
    bm = S.input_bitmask(w.seed, 0, batch * nb, w.num_inputs, w.rate_q32)
    pinned = S.PinnedBuffer(bm.size, np.uint32)
    pinned.array[:] = bm
    pipe = S.IoPipeline(vram, batch, words, ids.size, d_ids, lay.virtual_offset, w.num_inputs, w.v_seg)
    refs = []
    try:
        for k in range(nb):
            pipe.submit(pinned.as_ptr() + k * batch * words * 4, k * batch, 0, eng.stream)
            ref = np.zeros(batch * ids.size, np.uint8)
            oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, k * batch, batch,
                             bm[k * batch * words:(k + 1) * batch * words], words, lay.virtual_offset, w.num_inputs,
                             mapped_soma_ids=ids, outputs=ref)
            refs.append(ref)
            if k >= 1:
                got = pipe.outputs(back=1)
                assert np.array_equal(got, refs[k - 1]), f"readout of batch {k - 1} differs"
        assert np.array_equal(pipe.outputs(back=0), refs[-1])
        eng.synchronize()
        assert np.array_equal(vram.download_heads(), heads)
        assert np.array_equal(vram.download_state(), state)
        assert sum(int(r.sum()) for r in refs) > 0
    finally:
        pipe.close()
        lib.gpu_free(d_ids)
        vram.free()
