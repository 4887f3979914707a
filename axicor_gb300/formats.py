"""The reference's binary formats: ``.state`` and ``.axons`` blobs, target packing.

- ``.state``: no header, the SoA arrays in ShardVramPtrs order, 910 bytes per
  padded neuron (genesis-compute/src/memory.rs:32-86,
  genesis-baker/src/bake/layout.rs:127-159).
- ``.axons``: raw ``BurstHeads8[total_axons]`` (bake/layout.rs:162-169).
- Targets: ``(segment << 24) | (axon_id + 1)`` (genesis-core/src/layout.rs:254-277).

Checkpoints are the same pair of files (genesis-node/src/node/shard_thread.rs:231-265,
genesis-node/src/boot.rs:39-97): written to ``*.tmp`` and renamed.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from ._native import MAX_DENDRITES, TARGET_AXON_MASK, TARGET_SEG_SHIFT

BYTES_PER_NEURON = 4 + 1 + 4 + 1 + 4 + MAX_DENDRITES * (4 + 2 + 1)  # 910


def align_to_warp(n: int) -> int:
    """genesis-core/src/layout.rs:77-79 (multiple of 64)."""
    return (n + 63) & ~63


def total_axons_for(padded_n: int, virtual_axons: int, ghosts: int = 0, file_axons: int = 0) -> int:
    """genesis-node/src/boot.rs:64-71"""
    return (max(padded_n + virtual_axons + ghosts, file_axons) + 31) & ~31


@dataclass(frozen=True)
class StateOffsets:
    """genesis-compute/src/memory.rs:59-86"""
    soma_voltage: int
    soma_flags: int
    threshold_offset: int
    timers: int
    soma_to_axon: int
    dendrite_targets: int
    dendrite_weights: int
    dendrite_timers: int
    total_bytes: int


def compute_state_offsets(padded_n: int) -> StateOffsets:
    n = padded_n
    off = 0
    fields = []
    for size in (4 * n, n, 4 * n, n, 4 * n, 4 * n * MAX_DENDRITES, 2 * n * MAX_DENDRITES, n * MAX_DENDRITES):
        fields.append(off)
        off += size
    return StateOffsets(*fields, total_bytes=off)


def state_blob_size(padded_n: int) -> int:
    return compute_state_offsets(padded_n).total_bytes


class StateView:
    """numpy views of the fields of a host ``.state`` blob (no copies)."""

    def __init__(self, blob: np.ndarray, padded_n: int):
        if blob.dtype != np.uint8 or blob.size != state_blob_size(padded_n):
            raise ValueError(f".state blob size mismatch: got {blob.size}, expected {state_blob_size(padded_n)}")
        o = compute_state_offsets(padded_n)
        n = padded_n
        self.blob = blob
        self.padded_n = n
        self.voltage = blob[o.soma_voltage:o.soma_flags].view(np.int32)
        self.flags = blob[o.soma_flags:o.threshold_offset]
        self.threshold_offset = blob[o.threshold_offset:o.timers].view(np.int32)
        self.timers = blob[o.timers:o.soma_to_axon]
        self.soma_to_axon = blob[o.soma_to_axon:o.dendrite_targets].view(np.uint32)
        self.targets = blob[o.dendrite_targets:o.dendrite_weights].view(np.uint32).reshape(MAX_DENDRITES, n)
        self.weights = blob[o.dendrite_weights:o.dendrite_timers].view(np.int16).reshape(MAX_DENDRITES, n)
        self.dendrite_timers = blob[o.dendrite_timers:o.total_bytes].reshape(MAX_DENDRITES, n)


def pack_dendrite_target(axon_id: int, segment_offset: int) -> int:
    """genesis-core/src/layout.rs:254-265"""
    if axon_id >= TARGET_AXON_MASK:
        raise ValueError("axon id exceeds 24 bits")
    if segment_offset >= 256:
        raise ValueError("segment offset exceeds 8 bits")
    return (segment_offset << TARGET_SEG_SHIFT) | ((axon_id + 1) & TARGET_AXON_MASK)


def unpack_axon_id(target: int) -> int:
    """genesis-core/src/layout.rs:268-271 (saturating at 0)."""
    return max((target & TARGET_AXON_MASK) - 1, 0)


def unpack_segment_offset(target: int) -> int:
    """genesis-core/src/layout.rs:274-277"""
    return target >> TARGET_SEG_SHIFT


def columnar_idx(padded_n: int, neuron_idx: int, slot: int) -> int:
    """genesis-core/src/layout.rs:238-242"""
    if not (neuron_idx < padded_n and slot < MAX_DENDRITES):
        raise IndexError(f"columnar_idx: neuron {neuron_idx} / slot {slot} out of range")
    return slot * padded_n + neuron_idx


def empty_heads(total_axons: int) -> np.ndarray:
    """All heads at the sentinel (bindings.cu:560-568), as u32[total_axons*8]."""
    return np.full(total_axons * 8, 0x80000000, dtype=np.uint32)


def write_pair(directory: Path, stem: str, state_blob: np.ndarray, heads: np.ndarray) -> None:
    """Atomically writes ``stem.state`` and ``stem.axons`` (shard_thread.rs:231-265)."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    for ext, arr in (("state", state_blob), ("axons", heads)):
        tmp = directory / f"{stem}.{ext}.tmp"
        with open(tmp, "wb") as f:
            f.write(np.ascontiguousarray(arr).view(np.uint8).tobytes())
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, directory / f"{stem}.{ext}")


def read_pair(directory: Path, padded_n: int, total_axons: int,
              prefer: tuple[str, ...] = ("checkpoint", "shard")) -> tuple[np.ndarray, np.ndarray, str]:
    """Boot read (genesis-node/src/boot.rs:39-97): the checkpoint pair when both
    files exist, else the baked pair.  Validates the blob size and the 32-byte
    alignment of ``.axons``; a short ``.axons`` keeps sentinel heads after it."""
    directory = Path(directory)
    for stem in prefer:
        sp, ap = directory / f"{stem}.state", directory / f"{stem}.axons"
        if sp.exists() and ap.exists():
            state = np.fromfile(sp, dtype=np.uint8)
            raw = np.fromfile(ap, dtype=np.uint8)
            if raw.size % 32:
                raise ValueError(f"{ap}: size {raw.size} is not a multiple of 32 bytes")
            if state.size != state_blob_size(padded_n):
                raise ValueError(f"{sp}: .state blob size mismatch, expected {state_blob_size(padded_n)}, "
                                 f"got {state.size}")
            if raw.size > total_axons * 32:
                raise ValueError(f"{ap}: axon_heads blob too large ({raw.size} > {total_axons * 32})")
            heads = empty_heads(total_axons)
            heads[: raw.size // 4] = raw.view(np.uint32)
            return state, heads, stem
    raise FileNotFoundError(f"no .state/.axons pair in {directory}")
