"""ctypes binding of ``include/axicor_day.h`` (the engine's C-ABI).

The library is the in-tree ``axicor_gb300/lib/libaxicor_day.so``; there is no
other implementation of the Day Phase in this package, so importing a
symbol from a missing library raises instead of falling back.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libaxicor_day.so"

MAX_DENDRITES = 128
AXON_SENTINEL = 0x80000000
NO_AXON = 0xFFFFFFFF
TARGET_AXON_MASK = 0x00FFFFFF
TARGET_SEG_SHIFT = 24

ERR_TARGET_RANGE = 0x1
ERR_SOMA_AXON = 0x2
ERR_VIRTUAL_RANGE = 0x4
ERR_READOUT_RANGE = 0x8
ERR_WAIT_LIMIT = 0x10   # a bounded on-device wait gave up (the kernel took its path without the staged data)

# VariantParameters, genesis-core/src/layout.rs:12-48 (64 bytes)
VARIANT_DTYPE = np.dtype(
    {
        "names": ["threshold", "rest_potential", "leak_rate", "homeostasis_penalty",
                  "spontaneous_firing_period_ticks", "initial_synapse_weight", "gsop_potentiation",
                  "gsop_depression", "homeostasis_decay", "refractory_period",
                  "synapse_refractory_period", "signal_propagation_length", "is_inhibitory",
                  "inertia_curve", "adaptive_leak_max", "adaptive_leak_gain", "adaptive_mode",
                  "d1_affinity", "d2_affinity"],
        "formats": ["<i4", "<i4", "<i4", "<i4", "<u4", "<u2", "<u2", "<u2", "<u2", "u1", "u1", "u1",
                    "u1", ("u1", (16,)), "<i4", "<u2", "u1", "u1", "u1"],
        "offsets": [0, 4, 8, 12, 16, 20, 22, 24, 26, 28, 29, 30, 31, 32, 48, 52, 54, 58, 59],
        "itemsize": 64,
    }
)
assert VARIANT_DTYPE.itemsize == 64


class ShardVramPtrs(C.Structure):
    """genesis-compute/src/ffi.rs:25-42"""
    _fields_ = [
        ("soma_voltage", C.c_void_p),
        ("soma_flags", C.c_void_p),
        ("threshold_offset", C.c_void_p),
        ("timers", C.c_void_p),
        ("soma_to_axon", C.c_void_p),
        ("dendrite_targets", C.c_void_p),
        ("dendrite_weights", C.c_void_p),
        ("dendrite_timers", C.c_void_p),
        ("axon_heads", C.c_void_p),
    ]


class VramStateLegacy(C.Structure):
    """genesis-core/src/layout.rs:281-307 (by-value state of the legacy launchers)"""
    _fields_ = [
        ("padded_n", C.c_uint32), ("total_axons", C.c_uint32),
        ("voltage", C.c_void_p), ("flags", C.c_void_p), ("threshold_offset", C.c_void_p),
        ("refractory_timer", C.c_void_p), ("soma_to_axon", C.c_void_p),
        ("dendrite_targets", C.c_void_p), ("dendrite_weights", C.c_void_p),
        ("dendrite_timers", C.c_void_p), ("axon_heads", C.c_void_p),
        ("input_bitmask", C.c_void_p), ("output_history", C.c_void_p),
        ("telemetry_count", C.c_void_p), ("telemetry_spikes", C.c_void_p),
    ]


class AxcIoBuffers(C.Structure):
    _fields_ = [
        ("d_input_bitmask", C.c_void_p),
        ("d_incoming_spikes", C.c_void_p),
        ("d_output_history", C.c_void_p),
        ("max_spikes_per_tick", C.c_uint32),
        ("input_words_per_tick", C.c_uint32),
        ("num_outputs", C.c_uint32),
    ]


class AxcZoneShard(C.Structure):
    _fields_ = [
        ("vram", ShardVramPtrs),
        ("padded_n", C.c_uint32), ("total_axons", C.c_uint32),
        ("io", AxcIoBuffers),
        ("h_input_bitmask", C.c_void_p), ("h_incoming_spikes", C.c_void_p), ("h_spike_counts", C.c_void_p),
        ("virtual_offset", C.c_uint32), ("num_virtual_axons", C.c_uint32),
        ("mapped_soma_ids_device", C.c_void_p), ("v_seg", C.c_uint32), ("dopamine", C.c_int16),
        ("h_output_history", C.c_void_p),
    ]


class AxcGhostRoute(C.Structure):
    _fields_ = [
        ("src_shard", C.c_uint32), ("dst_shard", C.c_uint32),
        ("d_src_indices", C.c_void_p), ("d_dst_indices", C.c_void_p), ("count", C.c_uint32),
    ]


class AxcPopBrainDesc(C.Structure):
    _fields_ = [
        ("vram", ShardVramPtrs),
        ("padded_n", C.c_uint32), ("total_axons", C.c_uint32),
        ("virtual_offset", C.c_uint32), ("num_virtual", C.c_uint32),
        ("d_input_bitmask", C.c_void_p), ("words_per_tick", C.c_uint32), ("v_seg", C.c_uint32),
        ("d_lut", C.c_void_p), ("dopamine", C.c_int32), ("tick_base", C.c_uint32),
        ("bitmask_ticks", C.c_uint32),
    ]


class AxcPopSchedule(C.Structure):
    _fields_ = [("lanes_per_neuron", C.c_uint32), ("update_blocks_per_sm", C.c_uint32),
                ("aux_blocks_per_sm", C.c_uint32)]


class AxcLearnedDesc(C.Structure):
    _fields_ = [
        ("vram", ShardVramPtrs),
        ("padded_n", C.c_uint32), ("total_axons", C.c_uint32),
        ("virtual_offset", C.c_uint32), ("num_virtual", C.c_uint32),
        ("d_input_bitmask", C.c_void_p), ("words_per_tick", C.c_uint32), ("bitmask_ticks", C.c_uint32),
        ("v_seg", C.c_uint32), ("dopamine", C.c_int32), ("tick_base", C.c_uint32),
        ("sample_capacity", C.c_uint32),
    ]


class AxcBrainSpec(C.Structure):
    _fields_ = [
        ("dim_x", C.c_uint32), ("dim_y", C.c_uint32), ("dim_z", C.c_uint32),
        ("slots", C.c_uint32), ("num_inputs", C.c_uint32), ("inhibitory_permille", C.c_uint32),
        ("radius", C.c_uint32), ("lambda_voxels", C.c_uint32),
        ("w_min", C.c_int32), ("w_max", C.c_int32), ("seed", C.c_uint64),
    ]


class AxcBrainLayout(C.Structure):
    _fields_ = [
        ("num_neurons", C.c_uint32), ("padded_n", C.c_uint32), ("total_axons", C.c_uint32),
        ("virtual_offset", C.c_uint32), ("state_bytes", C.c_uint64), ("axons_bytes", C.c_uint64),
    ]


P = C.c_void_p
U32, I32, U16, I16, U8 = C.c_uint32, C.c_int32, C.c_uint16, C.c_int16, C.c_uint8
PV = C.POINTER(ShardVramPtrs)

# name -> (restype, argtypes); mirrors include/axicor_day.h
SIGNATURES: dict[str, tuple] = {
    "cu_allocate_shard": (I32, [U32, U32, PV]),
    "cu_reset_burst_counters": (None, [PV, U32, P]),
    "cu_upload_state_blob": (I32, [PV, P, C.c_size_t]),
    "cu_upload_axons_blob": (I32, [PV, P, C.c_size_t]),
    "cu_free_shard": (None, [PV]),
    "cu_step_day_phase": (I32, [PV, U32, U32, U32, U32, P, U32, U32, P, U32, P, P, U32, I16, P]),
    "cu_upload_constant_memory": (I32, [P]),
    "gpu_malloc": (P, [C.c_size_t]),
    "gpu_free": (None, [P]),
    "gpu_host_alloc": (P, [C.c_size_t]),
    "gpu_host_free": (None, [P]),
    "gpu_memcpy_host_to_device_async": (None, [P, P, C.c_size_t, P]),
    "gpu_memcpy_device_to_host_async": (None, [P, P, C.c_size_t, P]),
    "gpu_memcpy_host_to_device": (C.c_bool, [P, P, C.c_size_t]),
    "gpu_memcpy_device_to_host": (C.c_bool, [P, P, C.c_size_t]),
    "gpu_stream_create": (I32, [C.POINTER(P)]),
    "gpu_stream_destroy": (I32, [P]),
    "gpu_stream_synchronize": (None, [P]),
    "gpu_set_device": (None, [I32]),
    "gpu_device_synchronize": (None, []),
    "gpu_synchronize": (None, []),
    "gpu_load_constants": (None, [P]),
    "update_constant_memory_hot_reload": (None, [P, P]),
    "launch_sort_and_prune": (None, [PV, U32, I16]),
    "launch_extract_outgoing_spikes": (None, [P, P, P, U32, U32, U32, P, P, P]),
    "launch_ghost_sync": (None, [P, P, P, P, U32, P]),
    "launch_inject_inputs": (None, [VramStateLegacy, P, U32, U32]),
    "launch_apply_spike_batch": (None, [VramStateLegacy, P, U32]),
    "launch_propagate_axons": (None, [VramStateLegacy, U32]),
    "launch_update_neurons": (None, [VramStateLegacy, P, U32]),
    "launch_apply_gsop": (None, [VramStateLegacy]),
    "launch_record_readout": (None, [VramStateLegacy, P, P, U32, U32]),
    "gpu_reset_telemetry_count": (None, [PV, P]),
    "launch_extract_telemetry": (None, [PV, U32, P, P, P]),
    "cu_allocate_io_buffers": (I32, [U32, U32, U32, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "cu_dma_h2d_io": (I32, [P, P, U32, P, P, U32, P]),
    "cu_dma_d2h_io": (I32, [P, P, U32, P]),
    "axc_version": (C.c_char_p, []),
    "axc_shard_error_flags": (I32, [PV, U32, C.POINTER(U32)]),
    "axc_last_spikes": (I32, [PV, C.POINTER(U32), P, U32, P]),
    "axc_step_day_phase_batch": (I32, [PV, U32, U32, U32, C.POINTER(AxcIoBuffers), P, P, P, U32, U32, P, U32,
                                       I16, U32, P, P]),
    "axc_shard_counters": (I32, [PV, U32, C.POINTER(C.c_uint64)]),
    "axc_profile_ticks": (I32, [PV, U32, U32, U32, U32, U32, P, U32, U32, U32, I16, I32, P, C.POINTER(C.c_float),
                                C.POINTER(C.c_uint64)]),
    "axc_batch_engine_mode": (I32, [I32]),
    "axc_tick_engine_mode": (I32, [I32]),
    "axc_shard_invalidate": (I32, [PV]),
    "axc_row_engine_fix_capacity": (U32, [U32]),
    "axc_row_engine_wait_limit": (U32, [U32]),
    "axc_extract_outgoing_spikes_noalloc": (I32, [P, P, P, U32, U32, U32, P, P, P]),
    "axc_population_create": (I32, [P, U32, C.POINTER(P)]),
    "axc_step_zone_batch": (I32, [C.POINTER(AxcZoneShard), U32, C.POINTER(AxcGhostRoute), U32, U32, U32, P]),
    "axc_io_pipeline_create": (I32, [PV, U32, U32, U32, U32, U32, P, U32, U32, U32, C.POINTER(P)]),
    "axc_io_pipeline_submit": (I32, [P, P, I16, U32, P]),
    "axc_io_pipeline_outputs": (I32, [P, U32, C.POINTER(P)]),
    "axc_io_pipeline_wait_input": (I32, [P]),
    "axc_io_pipeline_destroy": (None, [P]),
    "axc_population_run": (I32, [P, U32, U32, U32, P]),
    "axc_population_tune": (I32, [P, U32, U32, P, P, C.POINTER(C.c_float), U32]),
    "axc_population_set_schedule": (I32, [P, P]),
    "axc_population_counters": (I32, [P, C.POINTER(C.c_uint64)]),
    "axc_population_destroy": (None, [P]),
    "axc_population_fix_capacity": (U32, [U32]),
    "axc_learned_create": (I32, [C.POINTER(AxcLearnedDesc), C.POINTER(P)]),
    "axc_learned_refresh": (I32, [P, P]),
    "axc_learned_set_policy": (I32, [P, I32, C.c_float, C.c_float, U32]),
    "axc_learned_collect": (I32, [P, U32, U32, U32]),
    "axc_learned_run": (I32, [P, U32, U32, U32, P]),
    "axc_learned_train": (I32, [P, U32, U32, C.c_float, C.c_uint64, C.POINTER(C.c_float),
                                C.POINTER(C.c_float), P]),
    "axc_learned_params": (I32, [P, P, P]),
    "axc_learned_samples": (I32, [P, U32, U32, P, P]),
    "axc_learned_stats": (I32, [P, C.POINTER(C.c_uint64)]),
    "axc_learned_reset_stats": (I32, [P]),
    "axc_learned_destroy": (None, [P]),
    "axc_mlp_param_count": (U32, []),
    "axc_mlp_loss_grad": (I32, [P, P, P, U32, P, P, P]),
    "axc_mlp_predict": (I32, [P, P, U32, P, P]),
    "axc_brain_layout": (I32, [C.POINTER(AxcBrainSpec), C.POINTER(AxcBrainLayout)]),
    "axc_brain_generate": (I32, [C.POINTER(AxcBrainSpec), P, P, I32]),
    "axc_input_bitmask": (I32, [C.c_uint64, U32, U32, U32, P, U32, P]),
}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Loads the engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"engine library {LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(str(LIB_PATH), mode=os.RTLD_LOCAL)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def ptr(a) -> int | None:
    """Host address of a numpy array (None for None)."""
    if a is None:
        return None
    return int(a.ctypes.data)


def check(err: int, what: str) -> None:
    if err != 0:
        raise RuntimeError(f"{what} failed with CUDA error {err}")
