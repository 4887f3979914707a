"""Shared helpers: run the same seeded brain on the engine and on the oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np

import oracle
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300.formats import StateView


class Twin:
    """One brain loaded twice: on the GPU through the C-ABI and on the host for the oracle."""

    def __init__(self, w, state=None, heads=None, lay=None, outputs="all"):
        if state is None:
            lay, state, heads = S.generate_brain(w.spec())
        self.w, self.lay = w, lay
        self.N, self.A = lay.padded_n, lay.total_axons
        self.voff, self.nv = lay.virtual_offset, w.num_inputs
        self.words = max((w.num_inputs + 31) // 32, 1)
        self.h_state, self.h_heads = state.copy(), heads.copy()
        S.upload_lut(w.lut)
        self.vram = S.VramState(self.N, self.A)
        self.vram.upload_state(state)
        self.vram.upload_axon_heads(heads)
        self.ids = np.arange(self.N, dtype=np.uint32) if isinstance(outputs, str) and outputs == "all" else outputs
        self.d_ids = S.device_array(self.ids) if self.ids is not None else None
        self.d_out = N.lib().gpu_malloc(max(self.N, 1))
        self.d_bm = N.lib().gpu_malloc(self.words * 4)
        self.d_in = None
        self.tick = 0

    def bitmask(self, ticks, tick0=None):
        t0 = self.tick if tick0 is None else tick0
        return S.input_bitmask(self.w.seed, t0, ticks, self.w.num_inputs, self.w.rate_q32)

    def gpu_step(self, bm_words, incoming=None, dopamine=None):
        lib = N.lib()
        if bm_words is not None:
            assert lib.gpu_memcpy_host_to_device(self.d_bm, N.ptr(bm_words), bm_words.nbytes)
        n_in = 0
        if incoming is not None and incoming.size:
            if self.d_in:
                lib.gpu_free(self.d_in)
            self.d_in = S.device_array(incoming)
            n_in = incoming.size
        nout = 0 if self.ids is None else self.ids.size
        err = lib.cu_step_day_phase(C.byref(self.vram.ptrs), self.N, self.A, self.w.v_seg, self.tick,
                                    self.d_bm if bm_words is not None else None, self.voff, self.nv,
                                    self.d_in if n_in else None, n_in, self.d_ids, self.d_out, nout,
                                    self.w.dopamine if dopamine is None else dopamine, None)
        assert err == 0
        out = np.empty(nout, dtype=np.uint8)
        if nout:
            assert lib.gpu_memcpy_device_to_host(N.ptr(out), self.d_out, nout)
        return out

    def oracle_step(self, bm_words, incoming=None, dopamine=None):
        nout = 0 if self.ids is None else self.ids.size
        out = np.empty(nout, dtype=np.uint8)
        err = oracle.step(self.h_state, self.h_heads, self.w.lut, self.N, self.A, self.w.v_seg, self.tick,
                          bm_words, self.voff, self.nv if bm_words is not None else 0, incoming=incoming,
                          mapped_soma_ids=self.ids, outputs=out if nout else None,
                          dopamine=self.w.dopamine if dopamine is None else dopamine)
        return out, err

    def step_both(self, incoming=None, dopamine=None):
        bm = self.bitmask(1)
        g = self.gpu_step(bm, incoming, dopamine)
        o, err = self.oracle_step(bm, incoming, dopamine)
        self.tick += 1
        return g, o, err

    def compare(self, where=""):
        gs = self.vram.download_state()
        gh = self.vram.download_heads()
        if not np.array_equal(gh, self.h_heads):
            bad = np.nonzero(gh != self.h_heads)[0]
            raise AssertionError(f"{where}: heads differ at {bad.size} words, first axon {bad[0] // 8}: "
                                 f"gpu {gh[bad[0] // 8 * 8:bad[0] // 8 * 8 + 8]} "
                                 f"oracle {self.h_heads[bad[0] // 8 * 8:bad[0] // 8 * 8 + 8]}")
        if not np.array_equal(gs, self.h_state):
            a, b = StateView(gs, self.N), StateView(self.h_state, self.N)
            msgs = []
            for f in ("voltage", "flags", "threshold_offset", "timers", "soma_to_axon", "targets", "weights",
                      "dendrite_timers"):
                x, y = getattr(a, f), getattr(b, f)
                if not np.array_equal(x, y):
                    idx = np.argwhere(x != y)
                    msgs.append(f"{f}: {len(idx)} differ, first {idx[0].tolist()} gpu {x[tuple(idx[0])]} "
                                f"oracle {y[tuple(idx[0])]}")
            raise AssertionError(f"{where}: state differs: " + "; ".join(msgs))

    def close(self):
        lib = N.lib()
        for p in (self.d_ids, self.d_out, self.d_bm, self.d_in):
            if p:
                lib.gpu_free(p)
        self.vram.free()
