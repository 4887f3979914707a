"""The zone batch (every shard's batch and the intra-GPU ghost sync in one graph) against the reference's order.

The reference node loop (genesis-node/src/node/mod.rs:330-420) steps every
shard's batch, waits for the device, then copies each intra-GPU channel's
boundary heads into the destination shard's ghost axons with
launch_ghost_sync (intra_gpu.rs:84, bindings.cu:341-368).  Two shards with
ghost routes both ways are run batch after batch through axc_step_zone_batch
and, on a second copy, through that sequence of calls; both must leave the
same bytes, equal to the oracle's (the oracle restates the tick and the ghost
copy).  Each shard's ghost axons are the last virtual axons of its range,
which its own input bitmask leaves silent.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GHOSTS = 32


class Side:
    """One shard on the GPU (twice: zone path and reference-order path) and on the host."""

    def __init__(self, w, batch):
        self.w = w
        self.lay, state, heads = S.generate_brain(w.spec())
        self.nv = w.num_inputs - GHOSTS            # real inputs; the last GHOSTS virtual axons are ghosts
        self.words = (self.nv + 31) // 32
        self.vz = S.VramState(self.lay.padded_n, self.lay.total_axons)
        self.vr = S.VramState(self.lay.padded_n, self.lay.total_axons)
        for v in (self.vz, self.vr):
            v.upload_state(state)
            v.upload_axon_heads(heads)
        self.h_state, self.h_heads = state, heads
        self.ids = np.arange(self.lay.padded_n, dtype=np.uint32)
        self.d_ids = S.device_array(self.ids)
        self.io_z = S.IoDeviceBuffers(self.words, 0, self.ids.size, batch)
        self.io_r = S.IoDeviceBuffers(self.words, 0, self.ids.size, batch)
        self.eng = S.ShardEngine(self.vr)
        self.ghost0 = self.lay.virtual_offset + self.nv

    def bitmask(self, t0, batch):
        return S.input_bitmask(self.w.seed, t0, batch, self.nv, self.w.rate_q32)


def test_zone_batch_equals_batches_then_ghost_sync(gpu):
    lib = N.lib()
    batch, nb = 16, 6
    a = Side(W.small(dims=(16, 16, 8), slots=64, inputs=96, p=0.1, seed=41), batch)
    b = Side(W.small(dims=(16, 8, 8), slots=48, inputs=64, p=0.1, seed=42), batch)
    rng = np.random.default_rng(6)
    # a -> b: 32 of a's neuron axons into b's ghosts; b -> a likewise (intra_gpu.rs: src ids, dst ghost ids)
    routes_h = []
    for src, dst in ((a, b), (b, a)):
        si = rng.choice(src.lay.num_neurons, size=GHOSTS, replace=False).astype(np.uint32)
        di = (dst.ghost0 + np.arange(GHOSTS)).astype(np.uint32)
        routes_h.append((src, dst, si, di, S.device_array(si), S.device_array(di)))
    shards = (N.AxcZoneShard * 2)()
    routes = (N.AxcGhostRoute * 2)()
    sides = [a, b]
    for r, (src, dst, si, di, dsi, ddi) in enumerate(routes_h):
        routes[r] = N.AxcGhostRoute(sides.index(src), sides.index(dst), dsi, ddi, GHOSTS)
    outs = {}
    try:
        for k in range(nb):
            t0 = k * batch
            bms = [s.bitmask(t0, batch) for s in sides]
            for i, s in enumerate(sides):
                outs[i] = np.zeros(batch * s.ids.size, np.uint8)
                z = shards[i]
                z.vram = s.vz.ptrs
                z.padded_n, z.total_axons = s.lay.padded_n, s.lay.total_axons
                z.io = s.io_z.as_struct()
                z.h_input_bitmask = bms[i].ctypes.data
                z.h_incoming_spikes = None
                z.h_spike_counts = None
                z.virtual_offset, z.num_virtual_axons = s.lay.virtual_offset, s.nv
                z.mapped_soma_ids_device = s.d_ids
                z.v_seg, z.dopamine = s.w.v_seg, 0
                z.h_output_history = outs[i].ctypes.data
            assert lib.axc_step_zone_batch(shards, 2, routes, 2, batch, t0, None) == 0
            # the reference's order: every shard's batch, the device barrier, the ghost sync of every channel
            ref_out = []
            for i, s in enumerate(sides):
                o = np.zeros(batch * s.ids.size, np.uint8)
                s.eng.step_day_phase_batch(batch, s.io_r, bms[i], None, None, s.lay.virtual_offset, s.nv, s.d_ids,
                                           s.w.v_seg, 0, t0, h_output_history=o)
                ref_out.append(o)
            lib.gpu_device_synchronize()
            for src, dst, si, di, dsi, ddi in routes_h:
                lib.launch_ghost_sync(src.vr.ptrs.axon_heads, dst.vr.ptrs.axon_heads, dsi, ddi, GHOSTS, None)
            lib.gpu_stream_synchronize(None)
            # the oracle
            for i, s in enumerate(sides):
                o = np.zeros(batch * s.ids.size, np.uint8)
                oracle.run_ticks(s.h_state, s.h_heads, s.w.lut, s.lay.padded_n, s.lay.total_axons, s.w.v_seg, t0,
                                 batch, bms[i], s.words, s.lay.virtual_offset, s.nv, mapped_soma_ids=s.ids, outputs=o)
                assert np.array_equal(outs[i], o), f"batch {k}, shard {i}: zone raster differs from the oracle"
                assert np.array_equal(ref_out[i], o), f"batch {k}, shard {i}: raster differs from the oracle"
            for src, dst, si, di, dsi, ddi in routes_h:
                oracle.ghost_sync(src.h_heads, dst.h_heads, si, di)
            for i, s in enumerate(sides):
                for v, name in ((s.vz, "zone"), (s.vr, "batches + ghost sync")):
                    assert np.array_equal(v.download_heads(), s.h_heads), f"batch {k}, shard {i}: {name} heads"
                    assert np.array_equal(v.download_state(), s.h_state), f"batch {k}, shard {i}: {name} state"
        # the ghosts carried the other shard's spikes: some ghost head is live
        gh = b.vz.download_heads().reshape(-1, 8)[b.ghost0:b.ghost0 + GHOSTS]
        assert np.any(gh != 0x80000000)
    finally:
        for *_, dsi, ddi in routes_h:
            lib.gpu_free(dsi)
            lib.gpu_free(ddi)
        for s in sides:
            lib.gpu_free(s.d_ids)
            s.vz.free()
            s.vr.free()


def test_zone_batch_refuses_a_shard_twice(gpu):
    lib = N.lib()
    w = W.small()
    lay, state, heads = S.generate_brain(w.spec())
    v = S.VramState(lay.padded_n, lay.total_axons)
    try:
        shards = (N.AxcZoneShard * 2)()
        for i in range(2):
            shards[i].vram = v.ptrs
            shards[i].padded_n, shards[i].total_axons = lay.padded_n, lay.total_axons
        assert lib.axc_step_zone_batch(shards, 2, None, 0, 10, 0, None) != 0
    finally:
        v.free()
