"""CPU oracle of the reference Day Phase — TEST INFRASTRUCTURE ONLY.

``day_phase_oracle.c`` restates genesis-compute/src/cuda/physics.cu and the
side kernels of bindings.cu in plain C (each function cites its reference
lines).  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, as the checker; the engine never calls it.

Pinning: the restatement is checked against every known-answer test the
reference holds for this path (active-tail predicate, target packing, GSOP
weight update, homeostasis), in tests/test_oracle_kat.py.  The reference has
no test that runs a whole tick, so full ticks are pinned against the
reference's own CUDA kernels, compiled from its sources (build_ref.py) and run
on the GPU tick by tick from the oracle's state (refgpu.py,
tests/test_reference_gpu.py).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB, build

_lib = None

P = C.c_void_p
U32, I32, I16, U64 = C.c_uint32, C.c_int32, C.c_int16, C.c_uint64


class _Ptrs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("soma_voltage", "soma_flags", "threshold_offset", "timers",
                                          "soma_to_axon", "dendrite_targets", "dendrite_weights",
                                          "dendrite_timers", "axon_heads")]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB))
        sig = {
            "orc_push_burst_head": (None, [P]),
            "orc_segment_hit": (C.c_int, [P, U32, U32]),
            "orc_min_dist": (U32, [P, U32, U32]),
            "orc_run_ticks": (U32, [P, P, P, U32, U32, U32, U32, U32, P, U32, U32, U32, P, P, U32, I16, P, P,
                                    C.c_int]),
            "orc_step_day_phase": (U32, [C.POINTER(_Ptrs), P, U32, U32, U32, U32, P, U32, U32, P, U32, P, P, U32,
                                         I16, P, C.c_int]),
            "orc_slice_state": (None, [P, U32, P, C.POINTER(_Ptrs)]),
            "orc_apply_gsop": (U32, [C.POINTER(_Ptrs), P, U32, U32, I16, P, C.c_int]),
            "orc_update_neurons": (U32, [C.POINTER(_Ptrs), P, U32, U32, U32, P, P, C.c_int]),
            "orc_sort_and_prune": (None, [C.POINTER(_Ptrs), U32, I16, C.c_int]),
            "orc_extract_outgoing_spikes": (U32, [P, P, P, U32, U32, U32, P, U32]),
            "orc_ghost_sync": (None, [P, P, P, P, U32]),
            "orc_extract_telemetry": (U32, [P, U32, P]),
            "orc_record_readout": (U32, [P, U32, P, P, U32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def _p(a):
    return None if a is None else int(a.ctypes.data)


def slice_state(state: np.ndarray, padded_n: int, heads: np.ndarray) -> _Ptrs:
    s = _Ptrs()
    lib().orc_slice_state(_p(state), padded_n, _p(heads), C.byref(s))
    return s


def run_ticks(state: np.ndarray, heads: np.ndarray, lut: np.ndarray, padded_n: int, total_axons: int,
              v_seg: int, tick_base: int, ticks: int, bitmask: np.ndarray | None, words_per_tick: int,
              virtual_offset: int, num_virtual: int, mapped_soma_ids: np.ndarray | None = None,
              outputs: np.ndarray | None = None, dopamine: int = 0, raster: np.ndarray | None = None,
              stats: np.ndarray | None = None, threads: int = 0) -> int:
    """Runs `ticks` ticks of the batch loop in place on (state, heads).
    Returns the AXC_ERR_* bits raised."""
    assert state.dtype == np.uint8 and heads.dtype == np.uint32
    num_outputs = 0 if mapped_soma_ids is None else int(mapped_soma_ids.size)
    lut = np.ascontiguousarray(lut)
    return int(lib().orc_run_ticks(_p(state), _p(heads), _p(lut), padded_n, total_axons, v_seg, tick_base, ticks,
                                   _p(bitmask), words_per_tick, virtual_offset, num_virtual, _p(mapped_soma_ids),
                                   _p(outputs), num_outputs, dopamine, _p(raster), _p(stats), threads))


def step(state: np.ndarray, heads: np.ndarray, lut: np.ndarray, padded_n: int, total_axons: int, v_seg: int,
         tick: int, bitmask: np.ndarray | None, virtual_offset: int, num_virtual: int,
         incoming: np.ndarray | None = None, mapped_soma_ids: np.ndarray | None = None,
         outputs: np.ndarray | None = None, dopamine: int = 0, stats: np.ndarray | None = None,
         threads: int = 0) -> int:
    """One cu_step_day_phase (physics.cu:441-495) on host arrays, in place."""
    s = slice_state(state, padded_n, heads)
    lut = np.ascontiguousarray(lut)
    n_in = 0 if incoming is None else int(incoming.size)
    n_out = 0 if mapped_soma_ids is None else int(mapped_soma_ids.size)
    return int(lib().orc_step_day_phase(C.byref(s), _p(lut), padded_n, total_axons, v_seg, tick, _p(bitmask),
                                        virtual_offset, num_virtual, _p(incoming), n_in, _p(mapped_soma_ids),
                                        _p(outputs), n_out, dopamine, _p(stats), threads))


def segment_hit(heads8, seg: int, prop: int) -> bool:
    h = np.ascontiguousarray(heads8, dtype=np.uint32)
    return bool(lib().orc_segment_hit(_p(h), seg, prop))


def min_dist(heads8, seg: int, prop: int) -> int:
    h = np.ascontiguousarray(heads8, dtype=np.uint32)
    return int(lib().orc_min_dist(_p(h), seg, prop))


def push(heads8) -> np.ndarray:
    h = np.array(heads8, dtype=np.uint32)
    lib().orc_push_burst_head(_p(h))
    return h


def apply_gsop(state, heads, lut, padded_n, total_axons, dopamine=0, threads=1) -> int:
    s = slice_state(state, padded_n, heads)
    return int(lib().orc_apply_gsop(C.byref(s), _p(np.ascontiguousarray(lut)), padded_n, total_axons, dopamine,
                                    None, threads))


def update_neurons(state, heads, lut, padded_n, total_axons, tick, threads=1) -> int:
    s = slice_state(state, padded_n, heads)
    return int(lib().orc_update_neurons(C.byref(s), _p(np.ascontiguousarray(lut)), padded_n, total_axons, tick,
                                        None, None, threads))


def sort_and_prune(state, heads, padded_n, threshold, threads=0) -> None:
    s = slice_state(state, padded_n, heads)
    lib().orc_sort_and_prune(C.byref(s), padded_n, threshold, threads)


def extract_outgoing_spikes(heads, src_idx, dst_ghost, sync_batch_ticks, v_seg, capacity) -> np.ndarray:
    out = np.zeros(capacity * 2, dtype=np.uint32)
    n = lib().orc_extract_outgoing_spikes(_p(heads), _p(src_idx), _p(dst_ghost), src_idx.size, sync_batch_ticks,
                                          v_seg, _p(out), capacity)
    return out[: 2 * min(n, capacity)].reshape(-1, 2)


def ghost_sync(src_heads, dst_heads, src_idx, dst_idx) -> None:
    lib().orc_ghost_sync(_p(src_heads), _p(dst_heads), _p(src_idx), _p(dst_idx), src_idx.size)


def spiking_ids(flags: np.ndarray) -> np.ndarray:
    out = np.empty(flags.size, dtype=np.uint32)
    n = lib().orc_extract_telemetry(_p(flags), flags.size, _p(out))
    return out[:n].copy()
