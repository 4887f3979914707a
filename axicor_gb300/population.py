"""A batched population of independent brains on one GPU (axc_population_* C-ABI).

Each brain is a normal shard (cu_allocate_shard + uploads) with its own LUT and
input bitmask in device memory; the population steps all of them with one
launch per stage per tick.  `run_alone` steps one brain through the ordinary
batch entry point, the reference for bit-exactness.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import shard as S


class Brain:
    def __init__(self, w, ticks: int, tick_base: int = 0):
        self.w = w
        self.lay, self.state0, self.heads0 = S.generate_brain(w.spec())
        self.vram = S.VramState(self.lay.padded_n, self.lay.total_axons)
        self.words = max((w.num_inputs + 31) // 32, 1)
        self.ticks = ticks
        self.bitmask = S.input_bitmask(w.seed, tick_base, ticks, w.num_inputs, w.rate_q32)
        self.d_bitmask = S.device_array(self.bitmask)
        self.d_lut = S.device_array(np.ascontiguousarray(w.lut))
        self.tick_base = tick_base
        self.reset()

    def reset(self) -> None:
        self.vram.upload_state(self.state0)
        self.vram.upload_axon_heads(self.heads0)

    def desc(self) -> N.AxcPopBrainDesc:
        d = N.AxcPopBrainDesc()
        d.vram = self.vram.ptrs
        d.padded_n = self.lay.padded_n
        d.total_axons = self.lay.total_axons
        d.virtual_offset = self.lay.virtual_offset
        d.num_virtual = self.w.num_inputs
        d.d_input_bitmask = self.d_bitmask
        d.words_per_tick = self.words
        d.v_seg = self.w.v_seg
        d.d_lut = self.d_lut
        d.dopamine = self.w.dopamine
        d.tick_base = self.tick_base
        d.bitmask_ticks = self.ticks
        return d

    @property
    def synapses(self) -> int:
        from .formats import StateView
        return int(np.count_nonzero(StateView(self.state0, self.lay.padded_n).targets))

    def run_alone(self, tick0: int, ticks: int, batch: int, engine: S.ShardEngine | None = None) -> None:
        """The same ticks through axc_step_day_phase_batch (the process LUT is set to this brain's)."""
        if tick0 + ticks > self.ticks:
            raise ValueError(f"ticks {tick0}..{tick0 + ticks} exceed the brain's {self.ticks}-tick input bitmask")
        S.upload_lut(self.w.lut)
        eng = engine or S.ShardEngine(self.vram)
        io = S.IoDeviceBuffers(self.words, 0, 0, batch)
        lib = N.lib()
        for t in range(tick0, tick0 + ticks, batch):
            src = self.d_bitmask + t * self.words * 4
            err = lib.axc_step_day_phase_batch(C.byref(self.vram.ptrs), self.lay.padded_n, self.lay.total_axons, batch,
                                               C.byref(io.as_struct()), src, None, None, self.lay.virtual_offset,
                                               self.w.num_inputs, None, self.w.v_seg, self.w.dopamine,
                                               self.tick_base + t, None, eng.stream)
            if err:
                raise RuntimeError(f"axc_step_day_phase_batch failed: {err}")
        eng.synchronize()

    def free(self) -> None:
        lib = N.lib()
        for p in (self.d_bitmask, self.d_lut):
            if p:
                lib.gpu_free(p)
        self.d_bitmask = self.d_lut = None
        self.vram.free()


class Population:
    def __init__(self, brains: list[Brain]):
        self.brains = brains
        descs = (N.AxcPopBrainDesc * len(brains))(*[b.desc() for b in brains])
        h = C.c_void_p()
        N.check(N.lib().axc_population_create(descs, len(brains), C.byref(h)), "axc_population_create")
        self.handle = h.value

    def tune(self, tick0: int, trial_ticks: int, stream=None) -> tuple[N.AxcPopSchedule, list[float]]:
        sc = N.AxcPopSchedule()
        ms = (C.c_float * 32)()
        N.check(N.lib().axc_population_tune(self.handle, tick0, trial_ticks, stream, C.byref(sc), ms, 32),
                "axc_population_tune")
        return sc, [float(x) for x in ms[:12]]

    def set_schedule(self, lanes: int, update_blocks: int, aux_blocks: int) -> None:
        sc = N.AxcPopSchedule(lanes, update_blocks, aux_blocks)
        N.check(N.lib().axc_population_set_schedule(self.handle, C.byref(sc)), "axc_population_set_schedule")

    def run(self, tick0: int, ticks: int, ticks_per_graph: int, stream=None) -> None:
        N.check(N.lib().axc_population_run(self.handle, tick0, ticks, ticks_per_graph, stream), "axc_population_run")

    def counters(self) -> np.ndarray:
        out = np.zeros(8, np.uint64)
        N.check(N.lib().axc_population_counters(self.handle, out.ctypes.data_as(C.POINTER(C.c_uint64))),
                "axc_population_counters")
        return out

    def close(self) -> None:
        if self.handle:
            N.lib().axc_population_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
