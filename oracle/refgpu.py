"""Runs the reference's own Day Phase kernels on the GPU (test and baseline infrastructure).

oracle/build_ref.py compiles genesis-compute/src/cuda/physics.cu into
oracle/_ref/physics_ref.cubin.  This module loads it with the CUDA driver API
and launches its kernels in the order and shapes of cu_step_day_phase
(physics.cu:441-495): 256-thread blocks, reset, inject, spike batch,
propagate, update, GSOP, readout.  Kernel names are the Itanium-mangled
names of the reference's kernel signatures.  The tests use it to check the
oracle against the reference itself; the benchmark times it as the
reference's own GPU Day Phase beside the engine's per-tick entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "physics_ref.cubin"

KERNELS = {
    "reset": "_Z30cu_reset_burst_counters_kernel13ShardVramPtrsj",
    "inject": "_Z23cu_inject_inputs_kernelP11BurstHeads8PKjjj",
    "spike_batch": "_Z27cu_apply_spike_batch_kernelP11BurstHeads8PKjjj",
    "propagate": "_Z25cu_propagate_axons_kernelP11BurstHeads8jj",
    "update": "_Z24cu_update_neurons_kernel13ShardVramPtrsjj",
    "gsop": "_Z20cu_apply_gsop_kernel13ShardVramPtrsjs",
    "readout": "_Z24cu_record_readout_kernelPKhPKjPhj",
}


def available() -> bool:
    return CUBIN.exists()


class ReferenceKernels:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        cu = self.cu
        cu.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 7 + [C.c_void_p, C.c_void_p, C.c_void_p]
        cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        cu.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self._chk(cu.cuInit(0), "cuInit")
        dev = C.c_int()
        self._chk(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
        ctx = C.c_void_p()
        self._chk(cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self._chk(cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.mod = C.c_void_p()
        self._chk(cu.cuModuleLoad(C.byref(self.mod), str(CUBIN).encode()), "cuModuleLoad")
        self.fn = {}
        for k, name in KERNELS.items():
            f = C.c_void_p()
            self._chk(cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), f"cuModuleGetFunction {k}")
            self.fn[k] = f
        self.lut_ptr = C.c_uint64()
        size = C.c_size_t()
        self._chk(cu.cuModuleGetGlobal_v2(C.byref(self.lut_ptr), C.byref(size), self.mod, b"VARIANT_LUT"),
                  "cuModuleGetGlobal")
        assert size.value == 1024

    @staticmethod
    def _chk(r, what):
        if r != 0:
            raise RuntimeError(f"{what} failed: CUresult {r}")

    def upload_lut(self, lut: np.ndarray):
        lut = np.ascontiguousarray(lut)
        self._chk(self.cu.cuMemcpyHtoD_v2(self.lut_ptr, C.c_void_p(lut.ctypes.data), C.c_size_t(1024)), "lut")

    def _launch(self, name, n, args):
        if n == 0:
            return
        holders = []
        ptrs = (C.c_void_p * len(args))()
        for i, a in enumerate(args):
            holders.append(a)
            ptrs[i] = C.cast(C.byref(a), C.c_void_p)
        grid = (n + 255) // 256
        self._chk(self.cu.cuLaunchKernel(self.fn[name], grid, 1, 1, 256, 1, 1, 0, None, C.cast(ptrs, C.c_void_p),
                                         None), name)

    def step(self, vram, padded_n, total_axons, v_seg, tick, d_bitmask, voff, nv, d_incoming, n_in, d_ids, d_out,
             n_out, dopamine, sync=True):
        """physics.cu:441-495 with the reference's own kernels, on the legacy default stream."""
        u32 = C.c_uint32
        vp = vram.ptrs  # ShardVramPtrs (ctypes struct of 9 pointers), passed by value
        self._launch("reset", padded_n, [vp, u32(padded_n)])
        if nv > 0 and d_bitmask:
            self._launch("inject", nv, [C.c_void_p(vp.axon_heads), C.c_void_p(d_bitmask), u32(voff), u32(nv)])
        if n_in > 0 and d_incoming:
            self._launch("spike_batch", n_in, [C.c_void_p(vp.axon_heads), C.c_void_p(d_incoming), u32(n_in),
                                               u32(total_axons)])
        self._launch("propagate", total_axons, [C.c_void_p(vp.axon_heads), u32(total_axons), u32(v_seg)])
        self._launch("update", padded_n, [vp, u32(padded_n), u32(tick)])
        self._launch("gsop", padded_n, [vp, u32(padded_n), C.c_int16(dopamine)])
        if n_out > 0 and d_ids and d_out:
            self._launch("readout", n_out, [C.c_void_p(vp.soma_flags), C.c_void_p(d_ids), C.c_void_p(d_out),
                                            u32(n_out)])
        if sync:
            self._chk(self.cu.cuCtxSynchronize(), "sync")
