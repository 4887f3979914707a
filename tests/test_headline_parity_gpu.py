"""Bit-exact parity at the benchmark sizes, every tick.

- The 1.5M-neuron / 150.7M-synapse brain through the batch entry point, ticks
  0..500 in 10-tick batches: every neuron's readout every tick, the whole
  .state blob and every axon head after every batch.  Ticks 0..500 hold the
  transient in which every spiker's whole row is still movable and GSOP inside
  the update pass does real work.
- The same brain through the per-tick entry point cu_step_day_phase (the
  symbol an unmodified ShardEngine calls, shard.rs:75-120): ticks 0..60, and
  ticks 700..720 in its steady state.
- The 8M-neuron x 128-slot brain (1.02B synapses): ticks 0..20 and ticks
  700..720, batch path, whole state compared.
- The learned engine forced sparse on the quiet 1.5M brain for 300 ticks
  against the plain batch path (the ordering of its GSOP passes after the
  sparse GLIF pass is what this pins).

The reference semantics are physics.cu:159-373 (update and GSOP) in the
order of physics.cu:441-495.
"""
import hashlib

import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import learned as L
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView
from helpers import Twin

pytestmark = pytest.mark.gpu


def _state_diff(gs, hs, Np):
    a, b = StateView(gs, Np), StateView(hs, Np)
    out = []
    for f in ("voltage", "flags", "threshold_offset", "timers", "soma_to_axon", "targets", "weights"):
        x, y = getattr(a, f), getattr(b, f)
        if not np.array_equal(x, y):
            idx = np.argwhere(x != y)
            out.append(f"{f}: {len(idx)} differ, first {idx[0].tolist()}")
    return "; ".join(out)


def _compare(vram, h_state, h_heads, Np, where):
    gh = vram.download_heads()
    assert np.array_equal(gh, h_heads), f"{where}: heads differ at {np.count_nonzero(gh != h_heads)} words"
    gs = vram.download_state()
    if not np.array_equal(gs, h_state):
        raise AssertionError(f"{where}: state differs: {_state_diff(gs, h_state, Np)}")


def _fast_forward(eng, lay, w, bm, words, t0, t1, io):
    for t in range(t0, t1, 100):
        eng.step_day_phase_batch(100, io, bm[t * words:(t + 100) * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, w.v_seg, 0, t)
    eng.synchronize()


def test_config1_batch_path_every_tick_first_500(gpu):
    """Ticks 0..500 of the 1.5M brain through axc_step_day_phase_batch in 10-tick batches."""
    w = W.config1()
    lay, state, heads = S.generate_brain(w.spec())
    Np, A = lay.padded_n, lay.total_axons
    S.upload_lut(w.lut)
    vram = S.VramState(Np, A)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    batch, total = 10, 500
    words = (w.num_inputs + 31) // 32
    ids = np.arange(Np, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, ids.size, batch)
    bm = S.input_bitmask(w.seed, 0, total, w.num_inputs, w.rate_q32)
    out = np.zeros(batch * ids.size, np.uint8)
    ref = np.zeros_like(out)
    gsop_moved = 0
    try:
        for t0 in range(0, total, batch):
            rows = bm[t0 * words:(t0 + batch) * words]
            eng.step_day_phase_batch(batch, io, rows, None, None, lay.virtual_offset, w.num_inputs, d_ids, w.v_seg,
                                     0, t0, h_output_history=out)
            w_before = StateView(state, Np).weights.copy() if t0 in (0, 250) else None
            err = oracle.run_ticks(state, heads, w.lut, Np, A, w.v_seg, t0, batch, rows, words, lay.virtual_offset,
                                   w.num_inputs, mapped_soma_ids=ids, outputs=ref)
            assert err == 0
            if not np.array_equal(out, ref):
                bad = np.nonzero(out != ref)[0]
                raise AssertionError(f"ticks {t0}..{t0 + batch}: raster differs at {bad.size} (tick, neuron) pairs, "
                                     f"first tick {t0 + bad[0] // Np} neuron {bad[0] % Np}")
            if w_before is not None:
                gsop_moved += int(np.count_nonzero(StateView(state, Np).weights != w_before))
            _compare(vram, state, heads, Np, f"after ticks {t0}..{t0 + batch}")
        assert gsop_moved > 1_000_000, "the transient must move weights (GSOP at work)"
        assert vram.error_flags() == 0
    finally:
        N.lib().gpu_free(d_ids)
        vram.free()


def test_config1_per_tick_entry_point(gpu):
    """cu_step_day_phase on the 1.5M brain: ticks 0..60 (transient) and 700..720 (steady state)."""
    lib = N.lib()
    prev = lib.axc_tick_engine_mode(1)
    w = W.config1()
    ids = np.linspace(0, 1_507_327, 8192).astype(np.uint32)
    tw = Twin(w, outputs=ids)
    try:
        for k in range(60):
            g, o, err = tw.step_both()
            assert np.array_equal(g, o), f"readout differs at tick {k}"
            if (k + 1) % 20 == 0:
                tw.compare(f"tick {k}")
        # on to tick 700 on the batch path; both sides then continue from the GPU's state
        eng = S.ShardEngine(tw.vram)
        io = S.IoDeviceBuffers(tw.words, 0, 0, 100)
        bm = S.input_bitmask(w.seed, 0, 720, w.num_inputs, w.rate_q32)
        eng.step_day_phase_batch(40, io, bm[60 * tw.words:100 * tw.words], None, None, tw.voff, tw.nv, None,
                                 w.v_seg, 0, 60)
        _fast_forward(eng, tw.lay, w, bm, tw.words, 100, 700, io)
        tw.h_state, tw.h_heads = tw.vram.download_state(), tw.vram.download_heads()
        tw.tick = 700
        for k in range(700, 720):
            g, o, err = tw.step_both()
            assert np.array_equal(g, o), f"readout differs at tick {k}"
        tw.compare("tick 720")
        sv = StateView(tw.h_state, tw.N)
        live = sv.targets != 0
        assert np.count_nonzero(live & (np.abs(sv.weights.astype(np.int32)) >= 2048)) > 0.99 * live.sum()
    finally:
        tw.close()
        lib.axc_tick_engine_mode(prev)


def test_config4_8m_batch_path(gpu):
    """The 8M-neuron x 128-slot brain: ticks 0..20 and ticks 700..720 on the batch path against the oracle."""
    w = W.config4()
    lay, state, heads = S.generate_brain(w.spec())
    Np, A = lay.padded_n, lay.total_axons
    S.upload_lut(w.lut)
    vram = S.VramState(Np, A)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    bm = S.input_bitmask(w.seed, 0, 720, w.num_inputs, w.rate_q32)
    ids = np.arange(0, Np, 7, dtype=np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, ids.size, 20)
    io100 = S.IoDeviceBuffers(words, 0, 0, 100)
    out = np.zeros(20 * ids.size, np.uint8)
    ref = np.zeros_like(out)
    try:
        for t0 in (0, 700):
            if t0 == 700:
                eng.step_day_phase_batch(80, io100, bm[20 * words:100 * words], None, None, lay.virtual_offset,
                                         w.num_inputs, None, w.v_seg, 0, 20)
                _fast_forward(eng, lay, w, bm, words, 100, 700, io100)
                state, heads = vram.download_state(), vram.download_heads()
            rows = bm[t0 * words:(t0 + 20) * words]
            eng.step_day_phase_batch(20, io, rows, None, None, lay.virtual_offset, w.num_inputs, d_ids, w.v_seg, 0,
                                     t0, h_output_history=out)
            oracle.run_ticks(state, heads, w.lut, Np, A, w.v_seg, t0, 20, rows, words, lay.virtual_offset,
                             w.num_inputs, mapped_soma_ids=ids, outputs=ref)
            assert np.array_equal(out, ref), f"readout differs in ticks {t0}..{t0 + 20}"
            assert int(ref.sum()) > 0
            _compare(vram, state, heads, Np, f"after ticks {t0}..{t0 + 20}")
        assert vram.error_flags() == 0
    finally:
        N.lib().gpu_free(d_ids)
        vram.free()


def _digest(vram):
    h = hashlib.sha256()
    h.update(vram.download_state().tobytes())
    h.update(vram.download_heads().tobytes())
    return h.hexdigest()


def test_learned_forced_sparse_on_quiet_1_5m_matches_plain(gpu):
    """The learned engine with every tick on the sparse form (the spikers of the sparse GLIF pass go to the
    GSOP passes after it) against the plain batch path: 300 ticks of the quiet 1.5M brain, sha256 of the
    final state and heads, and both against the oracle."""
    ticks = 300
    w = W.homeostatic(W.config1(ticks=ticks))
    lay, state, heads = S.generate_brain(w.spec())
    words = (w.num_inputs + 31) // 32
    S.upload_lut(w.lut)
    bm = S.input_bitmask(w.seed, 0, ticks, w.num_inputs, w.rate_q32)
    d_bm = S.device_array(bm)
    plain = S.VramState(lay.padded_n, lay.total_axons)
    plain.upload_state(state)
    plain.upload_axon_heads(heads)
    learned = S.VramState(lay.padded_n, lay.total_axons)
    learned.upload_state(state)
    learned.upload_axon_heads(heads)
    oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, 0, ticks, bm, words,
                     lay.virtual_offset, w.num_inputs)
    eng = S.ShardEngine(plain)
    io = S.IoDeviceBuffers(words, 0, 0, 100)
    le = L.LearnedEngine(learned, lay.padded_n, lay.total_axons, lay.virtual_offset, w.num_inputs, d_bm, words,
                         ticks, w.v_seg, 0, 0, 0)
    try:
        le.set_policy(L.Policy(policy=1))
        le.run(0, ticks, 100)
        _fast_forward(eng, lay, w, bm, words, 0, ticks, io)
        N.lib().gpu_device_synchronize()
        st = le.stats()
        assert st["sparse_ticks"] + st["overflow_reruns"] == ticks and st["sparse_ticks"] > ticks // 2, st
        for name, v in (("plain", plain), ("learned", learned)):
            gs, gh = v.download_state(), v.download_heads()
            same = np.array_equal(gs, state) and np.array_equal(gh, heads)
            assert same, f"{name} differs from the oracle after {ticks} ticks: {_state_diff(gs, state, lay.padded_n)}"
        assert _digest(learned) == _digest(plain)
    finally:
        le.close()
        N.lib().gpu_free(d_bm)
        plain.free()
        learned.free()
