"""The learned-schedule engine: MLP kernels against the oracle, and every
schedule (dense, sparse, predictor-chosen, overflowing, stale index)
bit-exact against the oracle."""
import time

import numpy as np
import pytest

import oracle
from oracle import predictor_oracle as M
from axicor_gb300 import _native as N
from axicor_gb300 import learned as L
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_oracle(gpu):
    """The tensor-core training kernel against the oracle's restatement of its order.  The tolerance is the
    tensor cores' FP32 accumulation of the hidden layer (unspecified order: last bits of a, and through them,
    rarely, one BF16 step of an activation): loss within 1e-5, every gradient entry within 2e-3 of the largest,
    and the whole gradient within 1e-3 in relative L2 norm."""
    rng = np.random.Generator(np.random.PCG64(11))
    p = M.init_params(7)
    x = rng.uniform(0, 1, (200, M.FEATURES)).astype(np.float32)
    t = rng.uniform(0, 1, 200).astype(np.float32)
    loss, g = L.mlp_loss_grad(p, x, t)
    lo, go = M.loss_grad(p, x, t)
    assert loss == pytest.approx(lo, rel=1e-5)
    assert np.abs(g - go).max() <= 2e-3 * np.abs(go).max()
    assert np.linalg.norm(g - go) <= 1e-3 * np.linalg.norm(go)


def test_mlp_predict_matches_oracle(gpu):
    """Predictions on the tensor cores against the oracle's restatement, within the same tolerance."""
    rng = np.random.Generator(np.random.PCG64(12))
    p = M.init_params(8)
    x = rng.uniform(0, 1, (300, M.FEATURES)).astype(np.float32)
    y = L.mlp_predict(p, x)
    yo, _, _ = M.forward(p, x)
    assert np.mean(y == yo) > 0.9
    assert np.abs(y - yo).max() <= 1e-3 * max(1.0, np.abs(yo).max())


class LBrain:
    """One brain on the learned engine, with its initial state kept for the oracle."""

    def __init__(self, w, ticks, sample_capacity=0, lay=None, state=None, heads=None):
        if state is None:
            lay, state, heads = S.generate_brain(w.spec())
        self.w, self.lay, self.ticks = w, lay, ticks
        self.state0, self.heads0 = state.copy(), heads.copy()
        S.upload_lut(w.lut)
        self.vram = S.VramState(lay.padded_n, lay.total_axons)
        self.vram.upload_state(state)
        self.vram.upload_axon_heads(heads)
        self.words = max((w.num_inputs + 31) // 32, 1)
        self.bm = S.input_bitmask(w.seed, 0, ticks, w.num_inputs, w.rate_q32)
        self.d_bm = S.device_array(self.bm)
        self.eng = L.LearnedEngine(self.vram, lay.padded_n, lay.total_axons, lay.virtual_offset, w.num_inputs,
                                   self.d_bm, self.words, ticks, w.v_seg, w.dopamine, 0, sample_capacity)

    def oracle(self, ticks, state=None, heads=None):
        hs = self.state0.copy() if state is None else state
        hh = self.heads0.copy() if heads is None else heads
        oracle.run_ticks(hs, hh, self.w.lut, self.lay.padded_n, self.lay.total_axons, self.w.v_seg, 0, ticks,
                         self.bm, self.words, self.lay.virtual_offset, self.w.num_inputs, dopamine=self.w.dopamine)
        return hs, hh

    def check(self, hs, hh, what=""):
        N.lib().gpu_device_synchronize()
        gs, gh = self.vram.download_state(), self.vram.download_heads()
        assert np.array_equal(gh, hh), f"{what}: heads differ"
        if not np.array_equal(gs, hs):
            a, o = StateView(gs, self.lay.padded_n), StateView(hs, self.lay.padded_n)
            bad = [f for f in ("voltage", "flags", "threshold_offset", "timers", "weights")
                   if not np.array_equal(getattr(a, f), getattr(o, f))]
            raise AssertionError(f"{what}: state differs in {bad}")

    def close(self):
        self.eng.close()
        N.lib().gpu_free(self.d_bm)
        self.vram.free()


def brain(kind, dims=(16, 16, 8), slots=64, ticks=60):
    w = W.small(dims=dims, slots=slots, inputs=64, p=0.08, ticks=ticks, seed=21)
    return W.homeostatic(w) if kind == "quiet" else w


@pytest.mark.parametrize("kind", ["saturated", "quiet"])
@pytest.mark.parametrize("policy", [0, 1])
def test_fixed_schedules_bit_exact(gpu, kind, policy):
    ticks = 60
    b = LBrain(brain(kind, ticks=ticks), ticks)
    try:
        b.eng.set_policy(L.Policy(policy=policy))
        b.eng.run(0, ticks, 20)
        st = b.eng.stats()
        assert st["ticks"] == ticks and st["stale_ticks"] == 0
        assert st["sparse_ticks"] == (ticks if policy == 1 else 0) and st["overflow_reruns"] == 0
        b.check(*b.oracle(ticks), f"{kind} policy {policy}")
    finally:
        b.close()


def test_predictor_collect_train_run_bit_exact(gpu):
    """Traces from dense ticks, GPU training, then predictor-chosen schedules."""
    ticks = 240
    w = brain("quiet", dims=(32, 32, 16), slots=64, ticks=ticks)
    b = LBrain(w, ticks, sample_capacity=4000)
    try:
        b.eng.set_policy(L.Policy(policy=0))
        b.eng.collect(True, reset=True)
        b.eng.run(0, 120, 20)
        b.eng.collect(False)
        st = b.eng.stats()
        assert st["samples"] == st["tiles"] * 119            # pairs (x of tick t-1, y of tick t), t = 1..119
        x, y = b.eng.samples(0, st["samples"])
        assert np.all(np.isfinite(x)) and np.all((y >= 0) & (y <= 1))
        loss, val = b.eng.train(epochs=40, batch=256, lr=2e-3, seed=3)
        assert loss[-1] < loss[0] and np.isfinite(val)
        b.eng.set_policy(L.Policy(policy=-1, ratio=4.0, margin=0.5, slack=64))
        b.eng.reset_stats()
        b.eng.run(120, 120, 20)
        st = b.eng.stats()
        assert st["ticks"] == 120 and st["judged_ticks"] > 100
        b.check(*b.oracle(ticks), "trained predictor")
    finally:
        b.close()


def test_untrained_predictor_overflows_to_dense(gpu):
    """All-zero predictions with no slack: every planned-sparse tick with an
    active axon outgrows its buffers and re-runs dense; the state stays exact."""
    ticks = 40
    b = LBrain(brain("saturated", ticks=ticks), ticks)
    try:
        b.eng.set_params(np.zeros(L.param_count(), np.float32))
        b.eng.set_policy(L.Policy(policy=-1, ratio=4.0, margin=0.0, slack=0))
        b.eng.run(0, ticks, 20)
        st = b.eng.stats()
        assert st["planned_sparse"] > 0
        assert st["overflow_reruns"] + st["sparse_ticks"] == st["planned_sparse"]
        assert st["overflow_reruns"] > 0
        b.check(*b.oracle(ticks), "overflow")
    finally:
        b.close()


def test_stale_index_runs_dense_until_refresh(gpu):
    ticks = 40
    w = brain("saturated", ticks=ticks)
    b = LBrain(w, ticks)
    try:
        # new targets after the index was built
        sv = StateView(b.state0, b.lay.padded_n)
        live = np.nonzero(sv.targets[0] != 0)[0][:50]
        sv.targets[0, live] = (sv.targets[0, live] & 0xFF000000) | ((sv.targets[0, live] & 0x00FFFFFF) % 97 + 1)
        b.vram.upload_state(b.state0)
        b.eng.set_policy(L.Policy(policy=1))
        b.eng.run(0, 20, 20)
        st = b.eng.stats()
        assert st["stale_ticks"] == 20 and st["sparse_ticks"] == 0
        b.eng.refresh()
        b.eng.run(20, 20, 20)
        st = b.eng.stats()
        assert st["stale_ticks"] == 20 and st["sparse_ticks"] == 20
        b.check(*b.oracle(ticks), "stale then refreshed")
    finally:
        b.close()


def test_learned_schedule_faster_than_plain_on_quiet_brain(gpu):
    """What the trained predictor gains: on a homeostatic brain (a few spikes
    per thousand neurons per tick) it picks the sparse form and beats the plain
    row pass, with the same final state."""
    warm, collect, ticks = 300, 200, 300
    total = warm + collect + ticks
    w = W.homeostatic(W.small(dims=(128, 64, 64), slots=100, inputs=4096, p=0.05, ticks=total, seed=31))
    b = LBrain(w, total, sample_capacity=100_000)
    lay = b.lay
    plain = S.VramState(lay.padded_n, lay.total_axons)
    plain.upload_state(b.state0)
    plain.upload_axon_heads(b.heads0)
    eng = S.ShardEngine(plain)
    io = S.IoDeviceBuffers(b.words, 0, 0, 100)
    try:
        b.eng.set_policy(L.Policy(policy=0))
        b.eng.run(0, warm, 100)
        b.eng.collect(True, reset=True)
        b.eng.run(warm, collect, 100)
        b.eng.collect(False)
        b.eng.train(epochs=30, batch=512, lr=2e-3, seed=5)
        for t in range(0, warm + collect, 100):
            eng.step_day_phase_batch(100, io, b.bm[t * b.words:(t + 100) * b.words], None, None,
                                     lay.virtual_offset, w.num_inputs, None, w.v_seg, w.dopamine, t)
        eng.synchronize()
        b.eng.set_policy(L.Policy(policy=-1))
        b.eng.reset_stats()
        t0 = time.perf_counter()
        b.eng.run(warm + collect, ticks, 100)
        N.lib().gpu_device_synchronize()
        t_learned = time.perf_counter() - t0
        t0 = time.perf_counter()
        for t in range(warm + collect, total, 100):
            eng.step_day_phase_batch(100, io, b.bm[t * b.words:(t + 100) * b.words], None, None,
                                     lay.virtual_offset, w.num_inputs, None, w.v_seg, w.dopamine, t)
        eng.synchronize()
        t_plain = time.perf_counter() - t0
        st = b.eng.stats()
        assert np.array_equal(plain.download_state(), b.vram.download_state())
        assert np.array_equal(plain.download_heads(), b.vram.download_heads())
        assert st["sparse_ticks"] > ticks // 2, st
        assert t_plain / t_learned > 1.2, (t_plain, t_learned, st)
    finally:
        b.close()
        plain.free()


def test_gate_follows_the_brain_from_dense_to_sparse(gpu):
    """Policy -1 on a brain that bursts (ticks 20..100: up to 14 % of the neurons spike per tick) and then goes
    quiet: while it bursts the predictor chooses the dense form for a whole chunk, so the gate puts the next
    chunks on the plain graph; once the brain is quiet the plain graph's own exact counts end the gate (well
    before its 64-chunk limit) and the predictor runs sparse ticks again.  Bit-exact against the oracle."""
    ticks, tpg = 800, 20
    b = LBrain(brain("quiet", dims=(32, 32, 16), slots=64, ticks=ticks), ticks)
    try:
        b.eng.set_params(np.zeros(L.param_count(), np.float32))   # residual on the last tick: the last-tick rule
        b.eng.set_policy(L.Policy(policy=-1))
        hist = []
        for t in range(0, ticks, tpg):
            b.eng.run(t, tpg, tpg)
            st = b.eng.stats()
            hist.append((st["gated_ticks"], st["sparse_ticks"]))
        gated = [i for i in range(len(hist)) if hist[i][0] > (hist[i - 1][0] if i else 0)]
        assert gated, hist
        first, last = gated[0], gated[-1]
        assert last - first + 1 < 64, hist
        later_sparse = hist[-1][1] - hist[last][1]
        assert later_sparse > 0, ("no sparse tick after the gate ended", hist)
        b.check(*b.oracle(ticks), "gated and ungated chunks")
    finally:
        b.close()
