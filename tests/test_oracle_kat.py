"""Pins the CPU oracle to the reference's own known-answer tests.

Sources (restated, not copied):
- active-tail predicate: genesis-core/src/signal.rs:67-103, genesis-core/src/test_signal.rs:7-98
- train model coverage: genesis-core/src/test_train_model.rs:8-129
- GSOP weight update: genesis-core/src/physics.rs:273-330
- homeostasis: genesis-core/src/physics.rs:236-266
- inertia rank: genesis-core/src/physics.rs:318-327 (CUDA clamps at 15, physics.cu:329-331)

The Rust helpers differ from the CUDA kernel in a few places (rank clamp 14 vs
15, a slot-decay factor the kernel fixes at 128, burst multiplier); each KAT is
restated under the conditions where both agree, and goes through the oracle's
kernel restatement (one-slot shards), not through a scalar helper.
"""
import numpy as np
import pytest

import oracle
from axicor_gb300 import _native as N
from axicor_gb300.formats import compute_state_offsets, pack_dendrite_target, state_blob_size

SENT = 0x80000000


def tail(head, seg, prop):
    return oracle.segment_hit([head] + [SENT] * 7, seg, prop)


# ---- signal.rs:67-103 ------------------------------------------------------
def test_active_tail_normal_overlap(oracle_lib):
    assert tail(10, 8, 3) and tail(10, 10, 3) and tail(10, 9, 3)


def test_active_tail_outside(oracle_lib):
    assert not tail(10, 7, 3)
    assert not tail(10, 0, 3)


def test_sentinel_edge_case(oracle_lib):
    assert not tail(SENT, 5, 3)
    assert not tail(SENT, 0, 255)
    assert not tail(SENT, 1000, 100)


def test_active_tail_zero_propagation(oracle_lib):
    assert not tail(10, 10, 0)
    assert not tail(10, 9, 0)


# ---- test_signal.rs:7-98 ---------------------------------------------------
def test_sentinel_is_never_active(oracle_lib):
    assert not tail(SENT, 0, 10)
    assert not tail(SENT, 100, 1)


def test_segment_in_tail_and_outside(oracle_lib):
    assert tail(10, 8, 3) and tail(10, 9, 3) and tail(10, 10, 3)
    assert not tail(10, 7, 3) and not tail(10, 0, 3)


def test_axon_fires_after_length_ticks(oracle_lib):
    length, prop = 5, 3
    head = (SENT - length) & 0xFFFFFFFF          # initial_axon_head(5), signal.rs:54-56
    assert head != SENT and head != 0
    heads = np.array([head] + [SENT] * 7, dtype=np.uint32)
    for _ in range(length - prop):               # propagation, physics.cu:137-154
        heads[heads != SENT] += 1
    assert oracle.segment_hit(heads, (SENT - length) & 0xFFFFFFFF, prop)


def test_tail_width_equals_propagation_length(oracle_lib):
    assert sum(tail(100, s, 7) for s in range(200)) == 7


def test_zero_propagation_never_active(oracle_lib):
    assert not any(tail(100, s, 0) for s in range(95, 106))


def test_sentinel_always_dead(oracle_lib):
    # is_segment_active has an explicit sentinel test; the kernel relies on
    # signal_propagation_length being a u8 (<= 255), so the KAT is restated
    # over the kernel's domain.
    for p in (0, 1, 10, 255):
        assert not tail(SENT, 0, p)


# ---- test_train_model.rs:8-129 ----------------------------------------------
def _covered(start, v_seg, prop, ticks, seg_hi):
    heads = np.array([start] + [SENT] * 7, dtype=np.uint32)
    cov = set()
    for _ in range(ticks):
        heads[heads != SENT] += v_seg
        cov |= {s for s in range(seg_hi) if oracle.segment_hit(heads, s, prop)}
    return cov


def test_no_gap_v_seg_1(oracle_lib):
    cov = _covered(100, 1, 5, 50, 200)
    assert all(s in cov for s in range(101, 100 + 50 - 5 + 2))


def test_no_gap_v_seg_large(oracle_lib):
    cov = _covered(100, 5, 5, 20, 300)
    assert all(s in cov for s in range(105, 100 + 100 - 5 + 2))


def test_gap_when_prop_lt_v_seg(oracle_lib):
    cov = _covered(100, 5, 3, 20, 300)
    assert 106 not in cov and 107 not in cov


def test_roundtrip_fire_to_overlap(oracle_lib):
    length, prop = 10, 3
    heads = np.array([(SENT - length) & 0xFFFFFFFF] + [SENT] * 7, dtype=np.uint32)
    for _ in range(length - 1):
        heads[heads != SENT] += 1
    assert oracle.segment_hit(heads, SENT - 1, prop)


# ---- one-slot shards for the update / GSOP KATs -----------------------------
PAD = 64


def one_slot_shard(weight, causal, flags=0x03, voltage=0, thr_off=0, seg=5):
    """Neuron 0 of a 64-neuron shard with one slot bound to axon 0 at `seg`."""
    state = np.zeros(state_blob_size(PAD), dtype=np.uint8)
    o = compute_state_offsets(PAD)
    state[o.soma_flags] = flags
    state[o.soma_voltage:o.soma_voltage + 4].view(np.int32)[0] = voltage
    state[o.threshold_offset:o.threshold_offset + 4].view(np.int32)[0] = thr_off
    state[o.soma_to_axon:o.dendrite_targets].view(np.uint32)[:] = N.NO_AXON
    state[o.dendrite_targets:o.dendrite_targets + 4].view(np.uint32)[0] = pack_dendrite_target(0, seg)
    state[o.dendrite_weights:o.dendrite_weights + 2].view(np.int16)[0] = weight
    heads = np.full(32 * 8, SENT, dtype=np.uint32)
    if causal:
        heads[0] = seg           # min_dist 0: cooling shift 0
    return state, heads, o


def gsop_lut(pot=80, dep=40, inertia=None):
    lut = np.zeros(16, dtype=N.VARIANT_DTYPE)
    lut[0]["gsop_potentiation"] = pot
    lut[0]["gsop_depression"] = dep
    lut[0]["signal_propagation_length"] = 4
    lut[0]["inertia_curve"] = np.full(16, 128, np.uint8) if inertia is None else np.asarray(inertia, np.uint8)
    return lut


def run_gsop(weight, causal, lut=None):
    state, heads, o = one_slot_shard(weight, causal)
    oracle.apply_gsop(state, heads, gsop_lut() if lut is None else lut, PAD, 32)
    return int(state[o.dendrite_weights:o.dendrite_weights + 2].view(np.int16)[0])


# physics.rs:273-330 (burst count 1 via flags 0x03, dopamine 0, cooling shift 0)
@pytest.mark.parametrize("w,causal,expected", [
    (100, True, 180), (100, False, 60), (-32768, True, -32767), (-32768, False, -32728),
    (-500, False, -460), (-5, False, 0), (32767, True, 32767), (1000, True, 1080),
])
def test_gsop_weight_kat(oracle_lib, w, causal, expected):
    assert run_gsop(w, causal) == expected


def test_gsop_sign_never_flips(oracle_lib):
    for w in (-800, -50, -5, -1):
        assert run_gsop(w, False) <= 0
    for w in (0, 1, 5, 50):
        assert run_gsop(w, False) >= 0


# physics.rs:318-327: rank = |w| >> 11 (clamped at 15 by the kernel, 14 by the Rust helper)
@pytest.mark.parametrize("absw,rank", [(0, 0), (2047, 0), (2048, 1), (4095, 1), (4096, 2), (32767, 15)])
def test_inertia_rank_kat(oracle_lib, absw, rank):
    causal = absw < 32767            # 32767 can only move down
    curve = np.zeros(16, np.uint8)
    curve[rank] = 128
    if absw > 0 or causal:
        assert run_gsop(absw, causal, gsop_lut(inertia=curve)) != absw
    curve2 = np.full(16, 128, np.uint8)
    curve2[rank] = 0
    assert run_gsop(absw, causal, gsop_lut(inertia=curve2)) == absw


# physics.rs:236-266 through the update stage (physics.cu:209-213, 249)
@pytest.mark.parametrize("offset,decay,spiking,penalty,expected", [
    (5, 10, False, 100, 0), (100, 3, False, 15, 97), (100, 3, True, 15, 112), (0, 0, False, 15, 0),
    (0, 0, True, 15, 15),
])
def test_homeostasis_kat(oracle_lib, offset, decay, spiking, penalty, expected):
    lut = np.zeros(16, dtype=N.VARIANT_DTYPE)
    lut[0]["threshold"] = 0 if spiking else 1 << 30
    lut[0]["homeostasis_decay"] = decay
    lut[0]["homeostasis_penalty"] = penalty
    lut[0]["signal_propagation_length"] = 4
    state, heads, o = one_slot_shard(0, False, flags=0x00, voltage=1000 if spiking else 0, thr_off=offset)
    oracle.update_neurons(state, heads, lut, PAD, 32, 0)
    got = int(state[o.threshold_offset:o.threshold_offset + 4].view(np.int32)[0])
    assert got == expected
    assert bool(state[o.soma_flags] & 1) == spiking


def test_push_burst_head(oracle_lib):
    """physics.cu:32-41"""
    assert list(oracle.push(list(range(1, 9)))) == [0, 1, 2, 3, 4, 5, 6, 7]


def test_spike_sets_burst_count_two(oracle_lib):
    """physics.cu:255 sets bit 1, then :271-273 increments: a spike leaves burst count 2
    (flags = type | 0b101), so GSOP's burst multiplier is 2 on the live path."""
    lut = np.zeros(16, dtype=N.VARIANT_DTYPE)
    lut[0]["signal_propagation_length"] = 4
    state, heads, o = one_slot_shard(0, False, flags=0x10, voltage=10)
    lut[1]["threshold"] = 0
    oracle.update_neurons(state, heads, lut, PAD, 32, 0)
    assert state[o.soma_flags] == 0x15
