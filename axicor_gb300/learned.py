"""The learned-schedule engine (axc_learned_* C-ABI) and the MLP entry points.

`LearnedEngine` steps one brain like `ShardEngine.step_day_phase_batch`, but a
per-tile activity predictor chooses, tick by tick, between the dense row pass
and a sparse axon-driven gather; the state stays bit-exact with the plain
path whatever it chooses.  Typical use: `collect` traces on a dense run,
`train`, then `run` with policy -1.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import shard as S

FEATURES, HIDDEN = 64, 128
TILE = 1024

STAT_NAMES = ("ticks", "sparse_ticks", "overflow_reruns", "schedule_mismatches", "abs_err_synapses",
              "actual_synapses", "judged_ticks", "planned_sparse", "stale_ticks", "gated_ticks", "r10", "r11",
              "samples", "history", "tiles", "index_capacity")


def param_count() -> int:
    return int(N.lib().axc_mlp_param_count())


@dataclass
class Policy:
    policy: int = -1          # -1 predictor, 0 always dense, 1 always sparse (exact buffers)
    ratio: float = 3.0
    margin: float = 0.25
    slack: int = 64


class LearnedEngine:
    def __init__(self, vram: S.VramState, padded_n: int, total_axons: int, virtual_offset: int, num_virtual: int,
                 d_bitmask: int | None, words_per_tick: int, bitmask_ticks: int, v_seg: int = 1, dopamine: int = 0,
                 tick_base: int = 0, sample_capacity: int = 0):
        d = N.AxcLearnedDesc()
        d.vram = vram.ptrs
        d.padded_n, d.total_axons = padded_n, total_axons
        d.virtual_offset, d.num_virtual = virtual_offset, num_virtual
        d.d_input_bitmask = d_bitmask
        d.words_per_tick, d.bitmask_ticks = words_per_tick, bitmask_ticks
        d.v_seg, d.dopamine, d.tick_base = v_seg, dopamine, tick_base
        d.sample_capacity = sample_capacity
        h = C.c_void_p()
        N.check(N.lib().axc_learned_create(C.byref(d), C.byref(h)), "axc_learned_create")
        self.handle = h.value
        self.tiles = (total_axons + TILE - 1) // TILE

    def set_policy(self, p: Policy) -> None:
        N.check(N.lib().axc_learned_set_policy(self.handle, p.policy, p.ratio, p.margin, p.slack),
                "axc_learned_set_policy")

    def collect(self, enable: bool, sample_every: int = 1, reset: bool = False) -> None:
        N.check(N.lib().axc_learned_collect(self.handle, int(enable), sample_every, int(reset)), "axc_learned_collect")

    def run(self, tick0: int, ticks: int, ticks_per_graph: int, stream=None) -> None:
        N.check(N.lib().axc_learned_run(self.handle, tick0, ticks, ticks_per_graph, stream), "axc_learned_run")

    def refresh(self, stream=None) -> None:
        N.check(N.lib().axc_learned_refresh(self.handle, stream), "axc_learned_refresh")

    def train(self, epochs: int, batch: int = 1024, lr: float = 1e-3, seed: int = 1) -> tuple[list[float], float]:
        loss = (C.c_float * max(epochs, 1))()
        val = C.c_float()
        N.check(N.lib().axc_learned_train(self.handle, epochs, batch, lr, seed, loss, C.byref(val), None),
                "axc_learned_train")
        return [float(x) for x in loss[:epochs]], float(val.value)

    def params(self) -> np.ndarray:
        out = np.zeros(param_count(), np.float32)
        N.check(N.lib().axc_learned_params(self.handle, N.ptr(out), None), "axc_learned_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == param_count()
        N.check(N.lib().axc_learned_params(self.handle, None, N.ptr(p)), "axc_learned_params")

    def samples(self, first: int, count: int) -> tuple[np.ndarray, np.ndarray]:
        x = np.zeros((count, FEATURES), np.float32)
        y = np.zeros(count, np.float32)
        N.check(N.lib().axc_learned_samples(self.handle, first, count, N.ptr(x), N.ptr(y)), "axc_learned_samples")
        return x, y

    def stats(self) -> dict[str, int]:
        out = np.zeros(16, np.uint64)
        N.check(N.lib().axc_learned_stats(self.handle, out.ctypes.data_as(C.POINTER(C.c_uint64))),
                "axc_learned_stats")
        return {k: int(v) for k, v in zip(STAT_NAMES, out)}

    def reset_stats(self) -> None:
        N.check(N.lib().axc_learned_reset_stats(self.handle), "axc_learned_reset_stats")

    def close(self) -> None:
        if self.handle:
            N.lib().axc_learned_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_loss_grad(params: np.ndarray, x: np.ndarray, y: np.ndarray) -> tuple[float, np.ndarray]:
    """Loss and gradient of the MLP on the GPU (axc_mlp_loss_grad)."""
    lib = N.lib()
    dp, dx, dy = S.device_array(params.astype(np.float32)), S.device_array(x.astype(np.float32)), \
        S.device_array(y.astype(np.float32))
    dg = S.device_array(np.zeros(params.size, np.float32))
    dl = S.device_array(np.zeros(1, np.float32))
    try:
        N.check(lib.axc_mlp_loss_grad(dp, dx, dy, int(y.size), dg, dl, None), "axc_mlp_loss_grad")
        g = np.zeros(params.size, np.float32)
        l = np.zeros(1, np.float32)
        lib.gpu_memcpy_device_to_host(N.ptr(g), dg, g.nbytes)
        lib.gpu_memcpy_device_to_host(N.ptr(l), dl, 4)
        return float(l[0]), g
    finally:
        for p in (dp, dx, dy, dg, dl):
            lib.gpu_free(p)


def mlp_predict(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    lib = N.lib()
    dp, dx = S.device_array(params.astype(np.float32)), S.device_array(x.astype(np.float32))
    do = S.device_array(np.zeros(x.shape[0], np.float32))
    try:
        N.check(lib.axc_mlp_predict(dp, dx, int(x.shape[0]), do, None), "axc_mlp_predict")
        out = np.zeros(x.shape[0], np.float32)
        lib.gpu_memcpy_device_to_host(N.ptr(out), do, out.nbytes)
        return out
    finally:
        for p in (dp, dx, do):
            lib.gpu_free(p)
