"""The reference's binary formats (genesis-compute/src/memory.rs, genesis-core/src/layout.rs,
genesis-node/src/boot.rs, shard_thread.rs checkpoints)."""
import numpy as np
import pytest

from axicor_gb300 import formats as F


def test_state_blob_is_910_bytes_per_neuron():
    assert F.BYTES_PER_NEURON == 910
    for n in (64, 1024, 1507328):
        assert F.state_blob_size(n) == 910 * n


def test_state_offsets_follow_shardvramptrs_order():
    o = F.compute_state_offsets(64)
    assert (o.soma_voltage, o.soma_flags, o.threshold_offset, o.timers, o.soma_to_axon) == (0, 256, 320, 576, 640)
    assert o.dendrite_targets == 896
    assert o.dendrite_weights == 896 + 64 * 128 * 4
    assert o.dendrite_timers == o.dendrite_weights + 64 * 128 * 2
    assert o.total_bytes == o.dendrite_timers + 64 * 128


def test_align_to_warp_and_total_axons():
    assert F.align_to_warp(1) == 64 and F.align_to_warp(64) == 64 and F.align_to_warp(65) == 128
    # boot.rs:64-71
    assert F.total_axons_for(1507328, 4096) == 1511424
    assert F.total_axons_for(64, 1, 0) == 96
    assert F.total_axons_for(64, 1, 0, file_axons=200) == 224


def test_dendrite_target_packing_kat():
    """genesis-core/src/layout.rs:388-404"""
    t0 = F.pack_dendrite_target(0, 0)
    assert t0 != 0
    assert F.unpack_axon_id(t0) == 0 and F.unpack_segment_offset(t0) == 0
    t_max = F.pack_dendrite_target(0x00FFFFFE, 255)
    assert F.unpack_axon_id(t_max) == 0x00FFFFFE and F.unpack_segment_offset(t_max) == 255
    t_mix = F.pack_dendrite_target(0x123456, 0xAB)
    assert F.unpack_axon_id(t_mix) == 0x123456 and F.unpack_segment_offset(t_mix) == 0xAB
    with pytest.raises(ValueError):
        F.pack_dendrite_target(0x00FFFFFF, 0)
    with pytest.raises(ValueError):
        F.pack_dendrite_target(1, 256)


def test_columnar_idx_kat():
    """genesis-core/src/layout.rs:377-385"""
    assert F.columnar_idx(1024, 0, 0) == 0
    assert F.columnar_idx(1024, 0, 1) == 1024
    assert F.columnar_idx(1024, 1, 0) == 1
    with pytest.raises(IndexError):
        F.columnar_idx(1024, 1024, 0)


def test_checkpoint_pair_roundtrip_and_boot_preference(tmp_path):
    n, a = 64, 96
    rng = np.random.default_rng(0)
    base = rng.integers(0, 256, F.state_blob_size(n), dtype=np.uint8)
    heads = F.empty_heads(a)
    F.write_pair(tmp_path, "shard", base, heads)
    s, h, stem = F.read_pair(tmp_path, n, a)
    assert stem == "shard" and np.array_equal(s, base) and np.array_equal(h, heads)
    ck = base.copy()
    ck[:10] = 7
    heads2 = heads.copy()
    heads2[:8] = 3
    F.write_pair(tmp_path, "checkpoint", ck, heads2)
    s, h, stem = F.read_pair(tmp_path, n, a)
    assert stem == "checkpoint" and np.array_equal(s, ck) and np.array_equal(h, heads2)
    assert not list(tmp_path.glob("*.tmp"))


def test_short_axons_blob_keeps_sentinels(tmp_path):
    n, a = 64, 96
    F.write_pair(tmp_path, "shard", np.zeros(F.state_blob_size(n), np.uint8), np.zeros(40 * 8, np.uint32))
    _, h, _ = F.read_pair(tmp_path, n, a)
    assert (h[:320] == 0).all() and (h[320:] == 0x80000000).all()


def test_boot_rejects_bad_files(tmp_path):
    n, a = 64, 96
    (tmp_path / "shard.state").write_bytes(b"\0" * (F.state_blob_size(n) - 1))
    (tmp_path / "shard.axons").write_bytes(b"\0" * 64)
    with pytest.raises(ValueError, match="size mismatch"):
        F.read_pair(tmp_path, n, a)
    (tmp_path / "shard.state").write_bytes(b"\0" * F.state_blob_size(n))
    (tmp_path / "shard.axons").write_bytes(b"\0" * 65)
    with pytest.raises(ValueError, match="multiple of 32"):
        F.read_pair(tmp_path, n, a)
    (tmp_path / "shard.axons").write_bytes(b"\0" * (a + 1) * 32)
    with pytest.raises(ValueError, match="too large"):
        F.read_pair(tmp_path, n, a)
