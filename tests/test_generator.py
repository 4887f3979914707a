"""The seeded brain generator: determinism and the properties the workloads promise."""
import hashlib

import numpy as np
import pytest

from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView


def sha(a):
    return hashlib.sha256(a.view(np.uint8).tobytes()).hexdigest()


def test_same_seed_same_bytes_any_thread_count(engine_lib):
    w = W.small()
    outs = {(sha(s), sha(h)) for t in (1, 2, 5, 8) for _, s, h in [S.generate_brain(w.spec(), threads=t)]}
    assert len(outs) == 1


def test_different_seed_different_brain(engine_lib):
    a = W.small(seed=1)
    b = W.small(seed=2)
    assert sha(S.generate_brain(a.spec())[1]) != sha(S.generate_brain(b.spec())[1])


@pytest.fixture(scope="module")
def brain16k(engine_lib):
    w = W.config0()
    lay, state, heads = S.generate_brain(w.spec())
    return w, lay, StateView(state, lay.padded_n), heads


def test_layout_16k(brain16k):
    w, lay, sv, heads = brain16k
    assert (lay.num_neurons, lay.padded_n, lay.total_axons, lay.virtual_offset) == (16384, 16384, 16640, 16384)
    assert lay.state_bytes == 910 * 16384
    assert (heads == N.AXON_SENTINEL).all()


def test_every_neuron_binds_all_slots_to_distinct_axons(brain16k):
    w, lay, sv, _ = brain16k
    t = sv.targets[:, : lay.num_neurons]
    assert (t[: w.slots] != 0).all() and (t[w.slots:] == 0).all()
    ax = (t.astype(np.int64) & 0xFFFFFF) - 1
    srt = np.sort(ax, axis=0)
    assert (np.diff(srt, axis=0) != 0).all(), "a neuron binds the same axon twice"
    assert (ax != np.arange(lay.num_neurons)[None, :]).all(), "self-synapse"
    assert (ax < lay.total_axons).all()
    seg = t >> 24
    assert seg.min() >= 1 and seg.max() <= 63


def test_weights_follow_dale_and_range(brain16k):
    w, lay, sv, _ = brain16k
    t = sv.targets[:, : lay.num_neurons]
    wt = sv.weights[:, : lay.num_neurons]
    ax = (t.astype(np.int64) & 0xFFFFFF) - 1
    inhib_pre = np.zeros(lay.total_axons, bool)
    inhib_pre[: lay.num_neurons] = (sv.flags[: lay.num_neurons] >> 4) == 1
    neg = inhib_pre[ax]
    assert (wt[neg] <= -50).all() and (wt[neg] >= -800).all()
    assert (wt[~neg] >= 50).all() and (wt[~neg] <= 800).all()
    frac_i = np.mean((sv.flags[: lay.num_neurons] >> 4) == 1)
    assert 0.18 < frac_i < 0.22
    assert set(np.unique(sv.flags[: lay.num_neurons])) <= {0x00, 0x10}


def test_inputs_and_padding(brain16k):
    w, lay, sv, _ = brain16k
    t = sv.targets[:, : lay.num_neurons]
    ax = (t.astype(np.int64) & 0xFFFFFF) - 1
    inp = ax[ax >= lay.padded_n] - lay.padded_n
    assert inp.size > 0 and inp.max() < w.num_inputs
    assert len(np.unique(inp)) > 0.9 * w.num_inputs
    assert (sv.soma_to_axon[: lay.num_neurons] == np.arange(lay.num_neurons)).all()


def test_padding_neurons_are_empty(engine_lib):
    w = W.small(dims=(10, 10, 10))
    lay, state, _ = S.generate_brain(w.spec())
    sv = StateView(state, lay.padded_n)
    assert lay.padded_n == 1024 and lay.num_neurons == 1000
    assert (sv.soma_to_axon[1000:] == N.NO_AXON).all()
    assert (sv.targets[:, 1000:] == 0).all() and (sv.flags[1000:] == 0).all()


def test_distance_law(brain16k):
    """P(bind) ~ exp(-d/4): counts per segment (two voxels each) fall off with distance."""
    w, lay, sv, _ = brain16k
    seg = (sv.targets[: w.slots, : lay.num_neurons] >> 24).ravel()
    counts = np.bincount(seg, minlength=20)
    assert counts[3] > counts[8] > counts[12] > counts[16]
    assert np.argmax(counts) in (2, 3, 4)


def test_input_bitmask_rate(engine_lib):
    bm = S.input_bitmask(5, 0, 2000, 256, np.array([W.p_q32(0.05)], np.uint32))
    rate = np.unpackbits(bm.view(np.uint8)).mean()
    assert 0.045 < rate < 0.055
    assert np.array_equal(bm[:8 * 100], S.input_bitmask(5, 0, 100, 256, np.array([W.p_q32(0.05)], np.uint32)))
    assert np.array_equal(bm[8 * 50:8 * 60], S.input_bitmask(5, 50, 10, 256, np.array([W.p_q32(0.05)], np.uint32)))
