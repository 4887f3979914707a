"""Host-side mirror of the reference's compute crate over the C-ABI.

``VramState`` follows genesis-compute/src/memory.rs:98-184, ``PinnedBuffer``
memory.rs:193-236, ``IoDeviceBuffers`` and ``ShardEngine``
genesis-compute/src/compute/shard.rs:4-132: same method names, argument
meanings and fail-fast errors (the Rust side asserts on every non-zero
cudaError; here a RuntimeError is raised).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .formats import BYTES_PER_NEURON, StateView, state_blob_size


def generate_brain(spec: N.AxcBrainSpec, threads: int = 0) -> tuple[N.AxcBrainLayout, np.ndarray, np.ndarray]:
    """Generates a seeded brain: (layout, .state blob u8, .axons heads u32[A*8])."""
    lib = N.lib()
    lay = N.AxcBrainLayout()
    N.check(lib.axc_brain_layout(C.byref(spec), C.byref(lay)), "axc_brain_layout")
    state = np.empty(lay.state_bytes, dtype=np.uint8)
    heads = np.empty(lay.total_axons * 8, dtype=np.uint32)
    N.check(lib.axc_brain_generate(C.byref(spec), N.ptr(state), N.ptr(heads), threads), "axc_brain_generate")
    return lay, state, heads


def input_bitmask(seed: int, tick0: int, ticks: int, num_inputs: int, rate_q32: np.ndarray) -> np.ndarray:
    """[ticks][ceil(num_inputs/32)] u32 words of seeded Bernoulli input spikes."""
    words = (num_inputs + 31) // 32
    out = np.zeros(ticks * max(words, 1), dtype=np.uint32)
    rates = np.ascontiguousarray(rate_q32, dtype=np.uint32)
    N.check(N.lib().axc_input_bitmask(seed, tick0, ticks, num_inputs, N.ptr(rates), rates.size, N.ptr(out)),
            "axc_input_bitmask")
    return out


def upload_lut(lut: np.ndarray) -> None:
    """cu_upload_constant_memory (physics.cu:504-506) of a 16-entry LUT."""
    lut = np.ascontiguousarray(lut)
    if lut.dtype != N.VARIANT_DTYPE or lut.size != 16:
        raise ValueError("LUT must be 16 VariantParameters")
    N.check(N.lib().cu_upload_constant_memory(N.ptr(lut)), "cu_upload_constant_memory")


class PinnedBuffer:
    """Page-locked host buffer (memory.rs:193-236) exposed as a numpy array."""

    def __init__(self, length: int, dtype=np.uint8):
        self.dtype = np.dtype(dtype)
        self.len = int(length)
        self._ptr = None
        self.array = np.zeros(0, dtype=self.dtype)
        if self.len:
            nbytes = self.len * self.dtype.itemsize
            p = N.lib().gpu_host_alloc(nbytes)
            if not p:
                raise RuntimeError(f"PinnedBuffer: gpu_host_alloc failed for {nbytes} bytes")
            self._ptr = p
            self.array = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(p)).view(self.dtype)

    def as_ptr(self) -> int | None:
        return self._ptr

    def __del__(self):
        if self._ptr:
            N.lib().gpu_host_free(self._ptr)
            self._ptr = None


class VramState:
    """Owner of one shard's device memory (memory.rs:98-184)."""

    def __init__(self, padded_n: int, total_axons: int, total_ghosts: int = 0):
        self.ptrs = N.ShardVramPtrs()
        err = N.lib().cu_allocate_shard(padded_n, total_axons, C.byref(self.ptrs))
        if err != 0:
            raise RuntimeError(f"FATAL: cu_allocate_shard failed (cudaError={err})")
        self.padded_n = padded_n
        self.total_axons = total_axons
        self.total_ghosts = total_ghosts

    @classmethod
    def allocate(cls, padded_n: int, total_axons: int, total_ghosts: int = 0) -> "VramState":
        return cls(padded_n, total_axons, total_ghosts)

    def virtual_offset(self) -> int:
        """Virtual axons start after the local and ghost axons (memory.rs:127-130)."""
        return self.padded_n + self.total_ghosts

    def upload_state(self, flat_blob: np.ndarray) -> None:
        expected = state_blob_size(self.padded_n)
        if flat_blob.nbytes != expected:
            raise RuntimeError(f"FATAL: .state blob size mismatch: got {flat_blob.nbytes} expected {expected}")
        blob = np.ascontiguousarray(flat_blob)
        N.check(N.lib().cu_upload_state_blob(C.byref(self.ptrs), N.ptr(blob), blob.nbytes), "cu_upload_state_blob")

    def upload_axon_heads(self, axon_heads_blob: np.ndarray) -> None:
        expected = self.total_axons * 32
        blob = np.ascontiguousarray(axon_heads_blob)
        if blob.nbytes > expected:
            raise RuntimeError(f"FATAL: axon_heads blob too large: got {blob.nbytes} expected max {expected}")
        if blob.nbytes == 0:
            return
        N.check(N.lib().cu_upload_axons_blob(C.byref(self.ptrs), N.ptr(blob), blob.nbytes), "cu_upload_axons_blob")

    def download_state(self) -> np.ndarray:
        out = np.empty(state_blob_size(self.padded_n), dtype=np.uint8)
        if not N.lib().gpu_memcpy_device_to_host(N.ptr(out), self.ptrs.soma_voltage, out.nbytes):
            raise RuntimeError("state download failed")
        return out

    def download_heads(self) -> np.ndarray:
        out = np.empty(self.total_axons * 8, dtype=np.uint32)
        if not N.lib().gpu_memcpy_device_to_host(N.ptr(out), self.ptrs.axon_heads, out.nbytes):
            raise RuntimeError("heads download failed")
        return out

    def state_view(self) -> StateView:
        return StateView(self.download_state(), self.padded_n)

    def error_flags(self, clear: bool = True) -> int:
        v = C.c_uint32(0)
        N.check(N.lib().axc_shard_error_flags(C.byref(self.ptrs), 1 if clear else 0, C.byref(v)),
                "axc_shard_error_flags")
        return v.value

    def counters(self, reset: bool = False) -> np.ndarray:
        out = np.zeros(8, dtype=np.uint64)
        N.check(N.lib().axc_shard_counters(C.byref(self.ptrs), 1 if reset else 0,
                                           out.ctypes.data_as(C.POINTER(C.c_uint64))), "axc_shard_counters")
        return out

    def last_spikes(self, stream: int | None = None) -> np.ndarray:
        cnt = C.c_uint32(0)
        ids = np.empty(self.padded_n, dtype=np.uint32)
        N.check(N.lib().axc_last_spikes(C.byref(self.ptrs), C.byref(cnt), N.ptr(ids), ids.size, stream),
                "axc_last_spikes")
        return ids[: cnt.value].copy()

    def free(self) -> None:
        if self.ptrs.soma_voltage or self.ptrs.axon_heads:
            N.lib().cu_free_shard(C.byref(self.ptrs))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class IoDeviceBuffers:
    """Per-batch device I/O buffers (shard.rs:4-11, bindings.cu:717-746)."""

    def __init__(self, input_words_per_tick: int, max_spikes_per_tick: int, num_outputs: int, batch: int):
        bm, sp, out = C.c_void_p(), C.c_void_p(), C.c_void_p()
        err = N.lib().cu_allocate_io_buffers(input_words_per_tick * batch, max_spikes_per_tick * batch,
                                            num_outputs * batch, C.byref(bm), C.byref(sp), C.byref(out))
        if err != 0:
            raise RuntimeError("cu_allocate_io_buffers failed")
        self.d_input_bitmask = bm.value
        self.d_incoming_spikes = sp.value
        self.d_output_history = out.value
        self.max_spikes_per_tick = max_spikes_per_tick
        self.input_words_per_tick = input_words_per_tick
        self.num_outputs = num_outputs
        self.batch = batch

    def as_struct(self) -> N.AxcIoBuffers:
        return N.AxcIoBuffers(self.d_input_bitmask, self.d_incoming_spikes, self.d_output_history,
                              self.max_spikes_per_tick, self.input_words_per_tick, self.num_outputs)

    def __del__(self):
        for p in (self.d_input_bitmask, self.d_incoming_spikes, self.d_output_history):
            if p:
                N.lib().gpu_free(p)


class ShardEngine:
    """Drives one shard on its own non-blocking stream (shard.rs:18-132)."""

    def __init__(self, vram: VramState):
        self.vram = vram
        s = C.c_void_p()
        err = N.lib().gpu_stream_create(C.byref(s))
        if err != 0:
            raise RuntimeError("FATAL: cudaStreamCreate failed")
        self.stream = s.value

    def step_day_phase_batch(self, sync_batch_ticks: int, io_buffers: IoDeviceBuffers,
                             h_input_bitmask: np.ndarray | None, h_incoming_spikes: np.ndarray | None,
                             h_spike_counts: np.ndarray | None, virtual_offset: int, num_virtual_axons: int,
                             mapped_soma_ids_device: int | None, v_seg: int, dopamine: int, tick_base: int,
                             h_output_history: np.ndarray | None = None, use_graph: bool = True) -> None:
        """One batch: bulk H2D, burst reset, `sync_batch_ticks` ticks.

        use_graph=True runs the native batch loop (axc_step_day_phase_batch,
        CUDA-graph replay); use_graph=False issues one cu_step_day_phase per
        tick from here, exactly as shard.rs:75-120 does."""
        lib = N.lib()
        vp = C.byref(self.vram.ptrs)
        if use_graph:
            io = io_buffers.as_struct()
            err = lib.axc_step_day_phase_batch(
                vp, self.vram.padded_n, self.vram.total_axons, sync_batch_ticks, C.byref(io),
                N.ptr(h_input_bitmask), N.ptr(h_incoming_spikes), N.ptr(h_spike_counts), virtual_offset,
                num_virtual_axons, mapped_soma_ids_device, v_seg, dopamine, tick_base, N.ptr(h_output_history),
                self.stream)
            if err != 0:
                raise RuntimeError(f"FATAL: Day Phase batch failed (cudaError={err})")
            return
        words, cap = io_buffers.input_words_per_tick, io_buffers.max_spikes_per_tick
        N.check(lib.cu_dma_h2d_io(io_buffers.d_input_bitmask, N.ptr(h_input_bitmask),
                                  words * sync_batch_ticks if h_input_bitmask is not None else 0,
                                  io_buffers.d_incoming_spikes, N.ptr(h_incoming_spikes),
                                  cap * sync_batch_ticks if h_incoming_spikes is not None else 0, self.stream),
                "cu_dma_h2d_io")
        lib.cu_reset_burst_counters(vp, self.vram.padded_n, self.stream)
        for tick in range(sync_batch_ticks):
            bm = io_buffers.d_input_bitmask + tick * words * 4 if io_buffers.d_input_bitmask else None
            sp = io_buffers.d_incoming_spikes + tick * cap * 4 if io_buffers.d_incoming_spikes else None
            out = io_buffers.d_output_history + tick * io_buffers.num_outputs if io_buffers.d_output_history else None
            cnt = int(h_spike_counts[tick]) if h_spike_counts is not None else 0
            err = lib.cu_step_day_phase(vp, self.vram.padded_n, self.vram.total_axons, v_seg, tick_base + tick, bm,
                                        virtual_offset, num_virtual_axons, sp, cnt, mapped_soma_ids_device, out,
                                        io_buffers.num_outputs, dopamine, self.stream)
            if err != 0:
                raise RuntimeError(f"FATAL: Day Phase Pipeline failed at tick {tick} (cudaError={err})")
        if h_output_history is not None and io_buffers.d_output_history:
            N.check(lib.cu_dma_d2h_io(N.ptr(h_output_history), io_buffers.d_output_history,
                                      io_buffers.num_outputs * sync_batch_ticks, self.stream), "cu_dma_d2h_io")
            self.synchronize()

    def synchronize(self) -> None:
        N.lib().gpu_stream_synchronize(self.stream)

    def __del__(self):
        try:
            if self.stream:
                N.lib().gpu_stream_destroy(self.stream)
        except Exception:
            pass


class IoPipeline:
    """Double-buffered batch I/O of one shard (axc_io_pipeline_*): the device side of the reference's input
    swapchain (io_server.rs:20-85) and per-batch output download (shard_thread.rs:208-227).  submit() queues a
    batch and returns at once; outputs(back) waits for the readout of the batch submitted `back` submits ago."""

    def __init__(self, vram: VramState, sync_batch_ticks: int, input_words_per_tick: int, num_outputs: int,
                 mapped_soma_ids_device: int | None, virtual_offset: int, num_virtual_axons: int, v_seg: int = 1):
        h = C.c_void_p()
        N.check(N.lib().axc_io_pipeline_create(C.byref(vram.ptrs), vram.padded_n, vram.total_axons,
                                               sync_batch_ticks, input_words_per_tick, num_outputs,
                                               mapped_soma_ids_device, virtual_offset, num_virtual_axons, v_seg,
                                               C.byref(h)), "axc_io_pipeline_create")
        self.handle = h.value
        self.batch, self.num_outputs = sync_batch_ticks, num_outputs if mapped_soma_ids_device else 0

    def submit(self, h_input_bitmask_ptr: int | None, tick_base: int, dopamine: int = 0,
               stream: int | None = None) -> None:
        N.check(N.lib().axc_io_pipeline_submit(self.handle, h_input_bitmask_ptr, dopamine, tick_base, stream),
                "axc_io_pipeline_submit")

    def outputs(self, back: int = 0) -> np.ndarray:
        p = C.c_void_p()
        N.check(N.lib().axc_io_pipeline_outputs(self.handle, back, C.byref(p)), "axc_io_pipeline_outputs")
        n = self.batch * self.num_outputs
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n,)).copy() if n else np.zeros(0,
                                                                                                          np.uint8)

    def wait_input(self) -> None:
        N.check(N.lib().axc_io_pipeline_wait_input(self.handle), "axc_io_pipeline_wait_input")

    def close(self) -> None:
        if self.handle:
            N.lib().axc_io_pipeline_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_array(host: np.ndarray) -> int:
    """Copies a host array to a new device buffer (gpu_malloc); returns the device pointer."""
    host = np.ascontiguousarray(host)
    p = N.lib().gpu_malloc(max(host.nbytes, 1))
    if not p:
        raise RuntimeError("gpu_malloc failed")
    if host.nbytes and not N.lib().gpu_memcpy_host_to_device(p, N.ptr(host), host.nbytes):
        raise RuntimeError("device upload failed")
    return p


__all__ = ["VramState", "ShardEngine", "IoDeviceBuffers", "IoPipeline", "PinnedBuffer", "generate_brain", "input_bitmask",
           "upload_lut", "device_array", "BYTES_PER_NEURON"]
