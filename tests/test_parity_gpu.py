"""Bit-exact parity of the CUDA Day Phase with the CPU oracle, every tick.

Compared each tick: the readout of every neuron (the spike raster), and the
whole .state blob (voltage, flags, threshold offsets, timers, soma_to_axon,
targets, weights, dendrite timers) plus every axon head.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView, compute_state_offsets
from helpers import Twin

pytestmark = pytest.mark.gpu


def run_twin(tw, ticks, compare_every=1, incoming_fn=None, dopamine_fn=None):
    try:
        spikes = 0
        for k in range(ticks):
            inc = incoming_fn(k) if incoming_fn else None
            dop = dopamine_fn(k) if dopamine_fn else None
            g, o, err = tw.step_both(inc, dop)
            assert np.array_equal(g, o), f"raster differs at tick {k}: {np.nonzero(g != o)[0][:10]}"
            spikes += int(o.sum())
            if (k + 1) % compare_every == 0:
                tw.compare(f"tick {k}")
        tw.compare("end")
        return spikes
    finally:
        tw.close()


def lut_adaptive():
    lut = W.default_lut()
    lut[0]["adaptive_mode"] = 1
    lut[0]["adaptive_leak_gain"] = 300
    lut[0]["adaptive_leak_max"] = 400
    lut[0]["homeostasis_decay"] = 2
    lut[0]["homeostasis_penalty"] = 50
    lut[1]["spontaneous_firing_period_ticks"] = 7
    lut[1]["homeostasis_penalty"] = 20
    return lut


def lut_mixed_prop():
    lut = W.default_lut()
    lut[0]["signal_propagation_length"] = 6
    lut[1]["signal_propagation_length"] = 3
    return lut


def lut_inertia():
    lut = W.default_lut()
    for v in (0, 1):
        lut[v]["inertia_curve"] = np.array([128, 120, 100, 90, 80, 70, 60, 50, 40, 30, 20, 10, 8, 6, 4, 2], np.uint8)
        lut[v]["d1_affinity"] = 64
        lut[v]["d2_affinity"] = 96
    return lut


@pytest.mark.parametrize("case", ["default", "adaptive", "mixed_prop", "inertia_dopamine", "vseg2", "long_segments",
                                  "dense_input"])
def test_tick_parity_small(gpu, case):
    w = W.small()
    dop = None
    if case == "adaptive":
        w.lut = lut_adaptive()
    elif case == "mixed_prop":
        w.lut = lut_mixed_prop()
    elif case == "inertia_dopamine":
        w.lut = lut_inertia()
        w.w_max = 5000
        dop = lambda k: (k * 37 % 400) - 200
    elif case == "vseg2":
        w.v_seg = 2
        w.lut[0]["signal_propagation_length"] = 3
        w.lut[1]["signal_propagation_length"] = 3
    elif case == "long_segments":
        w = W.small(dims=(96, 4, 4), slots=48, inputs=32)
        w.radius, w.lambda_voxels = 100, 30
    elif case == "dense_input":
        w = W.small(p=0.5, slots=128)
    tw = Twin(w)
    if case == "long_segments":
        segs = StateView(tw.h_state, tw.N).targets >> 24
        assert segs.max() >= 40
    spikes = run_twin(tw, 60, dopamine_fn=dop)
    assert spikes > 0


def test_incoming_spikes_with_duplicates_and_bad_ids(gpu):
    w = W.small()
    rng = np.random.default_rng(3)
    tw = Twin(w)
    A = tw.A

    def inc(k):
        ids = rng.integers(0, A + 50, size=rng.integers(0, 300)).astype(np.uint32)
        if ids.size > 4:
            ids[:3] = ids[3]                 # duplicates push once per occurrence
        return ids

    run_twin(tw, 40, incoming_fn=inc)


def test_error_flags_and_guarded_accesses(gpu):
    w = W.small()
    lay, state, heads = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    sv.targets[3, 10] = 5 << 24                       # axon field 0 -> id 0xFFFFFFFF
    sv.targets[4, 11] = (2 << 24) | (lay.total_axons + 7)
    sv.soma_to_axon[12] = lay.total_axons + 3
    tw = Twin(w, state=state, heads=heads, lay=lay)
    try:
        errs = 0
        for k in range(20):
            g, o, err = tw.step_both()
            errs |= err
            assert np.array_equal(g, o)
        tw.compare("end")
        gerr = tw.vram.error_flags()
        assert errs & N.ERR_TARGET_RANGE
        assert gerr == errs, (hex(gerr), hex(errs))
    finally:
        tw.close()


def test_batch_graph_matches_oracle(gpu):
    """ShardEngine.step_day_phase_batch (graph replay) against the oracle's batch loop."""
    w = W.small(dims=(16, 16, 16), slots=96, inputs=128)
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    batch, nb = 20, 4
    words = (w.num_inputs + 31) // 32
    ids = np.arange(lay.padded_n, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 64, ids.size, batch)
    h_state, h_heads = state.copy(), heads.copy()
    rng = np.random.default_rng(11)
    try:
        for b in range(nb):
            bm = S.input_bitmask(w.seed, b * batch, batch, w.num_inputs, w.rate_q32)
            out = np.zeros(batch * ids.size, np.uint8)
            dop = int(rng.integers(-100, 100))
            eng.step_day_phase_batch(batch, io, bm, None, None, lay.virtual_offset, w.num_inputs, d_ids,
                                     w.v_seg, dop, b * batch, h_output_history=out, use_graph=True)
            ref = np.zeros_like(out)
            err = oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, b * batch,
                                   batch, bm, words, lay.virtual_offset, w.num_inputs, mapped_soma_ids=ids,
                                   outputs=ref, dopamine=dop)
            assert err == 0
            assert np.array_equal(out, ref), f"batch {b}: raster differs"
            assert np.array_equal(vram.download_heads(), h_heads), f"batch {b}: heads differ"
            assert np.array_equal(vram.download_state(), h_state), f"batch {b}: state differs"
    finally:
        N.lib().gpu_free(d_ids)


def test_batch_graph_with_network_spikes(gpu):
    w = W.small()
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    batch, cap = 10, 32
    words = (w.num_inputs + 31) // 32
    io = S.IoDeviceBuffers(words, cap, 0, batch)
    rng = np.random.default_rng(5)
    h_state, h_heads = state.copy(), heads.copy()
    for b in range(3):
        bm = S.input_bitmask(w.seed, b * batch, batch, w.num_inputs, w.rate_q32)
        sched = rng.integers(0, lay.total_axons + 10, size=batch * cap).astype(np.uint32)
        counts = rng.integers(0, cap + 1, size=batch).astype(np.uint32)
        eng.step_day_phase_batch(batch, io, bm, sched, counts, lay.virtual_offset, w.num_inputs, None, w.v_seg, 0,
                                 b * batch, use_graph=True)
        eng.synchronize()
        for k in range(batch):
            oracle.step(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, b * batch + k,
                        bm[k * words:(k + 1) * words], lay.virtual_offset, w.num_inputs,
                        incoming=sched[k * cap:k * cap + counts[k]])
        assert np.array_equal(vram.download_heads(), h_heads)
        assert np.array_equal(vram.download_state(), h_state)


def test_per_tick_loop_matches_graph(gpu):
    """The same batches through cu_step_day_phase per tick and through the graph give identical bytes."""
    w = W.small(dims=(16, 16, 8), slots=64)
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    words = (w.num_inputs + 31) // 32
    results = []
    for use_graph in (False, True):
        vram = S.VramState(lay.padded_n, lay.total_axons)
        vram.upload_state(state)
        vram.upload_axon_heads(heads)
        eng = S.ShardEngine(vram)
        io = S.IoDeviceBuffers(words, 0, 0, 16)
        for b in range(3):
            bm = S.input_bitmask(w.seed, b * 16, 16, w.num_inputs, w.rate_q32)
            eng.step_day_phase_batch(16, io, bm, None, None, lay.virtual_offset, w.num_inputs, None, 1, 0, b * 16,
                                     use_graph=use_graph)
        eng.synchronize()
        results.append((vram.download_state(), vram.download_heads()))
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])


def test_plain_16k_1000_ticks(gpu):
    """The 16,384-neuron brain, 1,000 ticks: raster every tick (batches of 20), full state every batch."""
    w = W.config0()
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    batch = 20
    words = (w.num_inputs + 31) // 32
    ids = np.arange(lay.padded_n, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, ids.size, batch)
    h_state, h_heads = state.copy(), heads.copy()
    total_spikes = 0
    try:
        for b in range(w.ticks // batch):
            bm = S.input_bitmask(w.seed, b * batch, batch, w.num_inputs, w.rate_q32)
            out = np.zeros(batch * ids.size, np.uint8)
            eng.step_day_phase_batch(batch, io, bm, None, None, lay.virtual_offset, w.num_inputs, d_ids, 1, 0,
                                     b * batch, h_output_history=out)
            ref = np.zeros_like(out)
            oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, 1, b * batch, batch, bm, words,
                             lay.virtual_offset, w.num_inputs, mapped_soma_ids=ids, outputs=ref)
            assert np.array_equal(out, ref), f"raster differs in batch {b}"
            assert np.array_equal(vram.download_heads(), h_heads), f"heads differ after batch {b}"
            assert np.array_equal(vram.download_state(), h_state), f"state differs after batch {b}"
            total_spikes += int(ref.sum())
        assert total_spikes > 0
        assert vram.error_flags() == 0
    finally:
        N.lib().gpu_free(d_ids)


def test_plain_1_5m_first_ticks(gpu):
    """The 1.5M-neuron / 150M-synapse brain at full size: the first ticks, whole state every tick."""
    w = W.config1()
    tw = Twin(w, outputs=None)
    try:
        for k in range(12):
            tw.step_both()
        tw.compare("tick 12")
        c = tw.vram.counters()
        assert c[0] == 12
    finally:
        tw.close()


def test_plain_1_5m_steady_state_batches(gpu):
    """The 1.5M-neuron brain at full size in its steady state: 700 ticks through the batch path (by then the
    weights outside the input axons' slots sit at zero-inertia ranks and nearly every axon is fully lit, so
    the movable-first rows, the 189 KB shared-memory bitmap and the deferred pushes all carry the tick),
    then two 10-tick batches on the GPU and on the oracle from the same state, whole state and heads
    compared after each."""
    w = W.config1()
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    del state, heads
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    warm, batch = 700, 10
    bm = S.input_bitmask(w.seed, 0, warm + 2 * batch, w.num_inputs, w.rate_q32)
    io = S.IoDeviceBuffers(words, 0, 0, 100)
    for t in range(0, warm, 100):
        eng.step_day_phase_batch(100, io, bm[t * words:(t + 100) * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, 1, 0, t)
    eng.synchronize()
    h_state, h_heads = vram.download_state(), vram.download_heads()
    sv = StateView(h_state, lay.padded_n)
    live = sv.targets != 0
    frozen = live & (np.abs(sv.weights.astype(np.int32)) >= 2048)
    assert frozen.sum() > 0.99 * live.sum()
    io10 = S.IoDeviceBuffers(words, 0, 0, batch)
    for b in range(2):
        t0 = warm + b * batch
        rows = bm[t0 * words:(t0 + batch) * words]
        eng.step_day_phase_batch(batch, io10, rows, None, None, lay.virtual_offset, w.num_inputs, None, 1, 0, t0)
        eng.synchronize()
        oracle.run_ticks(h_state, h_heads, w.lut, lay.padded_n, lay.total_axons, 1, t0, batch, rows, words,
                         lay.virtual_offset, w.num_inputs)
        assert np.array_equal(vram.download_heads(), h_heads), f"heads differ after ticks {t0}..{t0 + batch}"
        assert np.array_equal(vram.download_state(), h_state), f"state differs after ticks {t0}..{t0 + batch}"
    assert vram.error_flags() == 0


def test_legacy_launchers_match_stages(gpu):
    """launch_propagate_axons / launch_update_neurons / launch_apply_gsop / launch_record_readout
    against the oracle's stages (ffi.rs:193-233)."""
    w = W.small()
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    # give the axons some recent heads
    rng = np.random.default_rng(2)
    h = heads.reshape(-1, 8).copy()
    sel = rng.random(h.shape[0]) < 0.5
    h[sel, 0] = rng.integers(0, 12, size=sel.sum())
    heads = h.reshape(-1)
    vram.upload_axon_heads(heads)
    p = vram.ptrs
    leg = N.VramStateLegacy(lay.padded_n, lay.total_axons, p.soma_voltage, p.soma_flags, p.threshold_offset, p.timers,
                            p.soma_to_axon, p.dendrite_targets, p.dendrite_weights, p.dendrite_timers, p.axon_heads,
                            None, None, None, None)
    lib = N.lib()
    lib.launch_propagate_axons(leg, 1)
    lib.launch_update_neurons(leg, None, 5)
    lib.launch_apply_gsop(leg)
    lib.gpu_device_synchronize()
    hs, hh = state.copy(), heads.copy()
    hv = hh.reshape(-1, 8)
    nz = hv != 0x80000000
    hv[nz] += 1
    oracle.update_neurons(hs, hh, w.lut, lay.padded_n, lay.total_axons, 5)
    oracle.apply_gsop(hs, hh, w.lut, lay.padded_n, lay.total_axons)
    assert np.array_equal(vram.download_heads(), hh)
    assert np.array_equal(vram.download_state(), hs)


@pytest.mark.parametrize("w,causal,expected", [
    (100, True, 180), (100, False, 60), (-32768, True, -32767), (-32768, False, -32728),
    (-500, False, -460), (-5, False, 0), (32767, True, 32767), (1000, True, 1080),
])
def test_gsop_kat_on_gpu(gpu, w, causal, expected):
    """The reference's GSOP known answers (genesis-core/src/physics.rs:273-330) through the GPU GSOP stage."""
    from test_oracle_kat import PAD, gsop_lut, one_slot_shard
    state, heads, o = one_slot_shard(w, causal)
    S.upload_lut(gsop_lut())
    vram = S.VramState(PAD, 32)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    p = vram.ptrs
    leg = N.VramStateLegacy(PAD, 32, p.soma_voltage, p.soma_flags, p.threshold_offset, p.timers, p.soma_to_axon,
                            p.dendrite_targets, p.dendrite_weights, p.dendrite_timers, p.axon_heads, None, None,
                            None, None)
    N.lib().launch_apply_gsop(leg)
    got = vram.download_state()[o.dendrite_weights:o.dendrite_weights + 2].view(np.int16)[0]
    assert int(got) == expected
