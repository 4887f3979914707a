"""What the trained activity predictor gains over a predictor without training.

The learned engine sizes each tile's compaction buffer for a sparse tick from
the predicted active synapses of the next tick; an under-prediction overflows
the buffer and the tick re-runs dense (exact, but slower).  The baseline is
the last-tick rule, "next tick's activity = this tick's": the network
predicts a residual on feature 8 (the tile's active-synapse fraction of the
tick just run), so all-zero weights are exactly that rule, and both run
through the same kernels on the same ticks of a quiet brain (homeostasis on,
input rate following a 100-tick sinusoid).  The trained network must predict
the held-out pairs with a lower error and mispredict fewer planned sparse
ticks; both schedules end bit-exact with the plain path.
"""
import numpy as np
import pytest

from axicor_gb300 import _native as N
from axicor_gb300 import learned as L
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from test_learned_gpu import LBrain

pytestmark = pytest.mark.gpu

LAST_TICK_FEATURE = 8   # channel 1 (active-synapse fraction), lag 0


def last_tick_params():
    return np.zeros(L.param_count(), np.float32)   # output = feature 8 + 0


def test_trained_predictor_beats_last_tick_rule(gpu):
    warm, collect, run = 300, 200, 300
    total = warm + collect + run
    w = W.homeostatic(W.small(dims=(96, 64, 64), slots=96, inputs=2048, p=0.05, ticks=total, seed=33))
    a = LBrain(w, total, sample_capacity=60_000)
    lay = a.lay
    try:
        a.eng.set_policy(L.Policy(policy=0))
        a.eng.run(0, warm, 100)
        a.eng.collect(True, reset=True)
        a.eng.run(warm, collect, 100)
        a.eng.collect(False)
        n = a.eng.stats()["samples"]
        x, y = a.eng.samples(0, n)
        loss, val_mse = a.eng.train(epochs=30, batch=512, lr=2e-3, seed=5)
        held = slice(int(n * 0.9), n)                # the split axc_learned_train validates on
        last_mse = float(np.mean((x[held, LAST_TICK_FEATURE] - y[held]) ** 2))
        assert val_mse < 0.9 * last_mse, (val_mse, last_mse)
        trained = a.eng.params()
        # a second copy of the brain at the same tick, predicting with the last-tick rule
        N.lib().gpu_device_synchronize()
        b = LBrain(w, total, sample_capacity=0, lay=lay, state=a.vram.download_state(),
                   heads=a.vram.download_heads())
        try:
            b.eng.set_params(last_tick_params())
            stats = {}
            for name, br in (("trained", a), ("last_tick", b)):
                br.eng.set_policy(L.Policy(policy=-1))
                br.eng.reset_stats()
                br.eng.run(warm + collect, run, 100)
                stats[name] = br.eng.stats()
            N.lib().gpu_device_synchronize()
            assert np.array_equal(a.vram.download_state(), b.vram.download_state())
            assert np.array_equal(a.vram.download_heads(), b.vram.download_heads())
            st_t, st_l = stats["trained"], stats["last_tick"]
            assert st_t["planned_sparse"] > run // 2 and st_l["planned_sparse"] > run // 2, stats
            miss_t = st_t["overflow_reruns"] / st_t["planned_sparse"]
            miss_l = st_l["overflow_reruns"] / st_l["planned_sparse"]
            assert miss_t < miss_l, (miss_t, miss_l, stats)
            err_t = st_t["abs_err_synapses"] / max(st_t["actual_synapses"], 1)
            err_l = st_l["abs_err_synapses"] / max(st_l["actual_synapses"], 1)
            print(f"held-out MSE trained {val_mse:.3e} last-tick {last_mse:.3e}; mispredicted sparse ticks "
                  f"trained {miss_t:.3f} last-tick {miss_l:.3f}; |error| / actual trained {err_t:.3f} "
                  f"last-tick {err_l:.3f}")
            # both schedules equal the plain path
            hs, hh = a.oracle(total)
            assert np.array_equal(a.vram.download_state(), hs)
            assert np.array_equal(a.vram.download_heads(), hh)
            assert trained.size == L.param_count()
        finally:
            b.close()
    finally:
        a.close()
