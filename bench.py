#!/usr/bin/env python3
"""Day Phase benchmark: synaptic events/s and ticks/s of one seeded brain.

Default workload: 1,507,328 integer GLIF neurons on a 128x128x92 grid, 100
dendrite slots each (150.7M synapses), 4,096 Bernoulli inputs at p=0.05,
GSOP on.  One step = one batch of `--ticks-per-step` ticks through the
engine's batch entry point (CUDA-graph replay of the tick loop).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Synaptic events/s = ticks/s x non-empty dendrite slots (the reference's own
definition, examples/cartpole_exp/benchmark.py:112).  `value` is measured
with the batch's inputs already in device memory; `e2e` through the same
public call with pinned host inputs and a device-to-host read of the output
readout every step.  `--impl reference` times the CPU restatement of the
reference kernels (the reference has no CPU Day Phase of its own) on the
host cores.  With N > 1 (torchrun), every rank runs an independent replica.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CONFIGS = {"plain-1.5M": "config1", "plain-16k": "config0", "plain-8M": "config4"}
# learned-schedule workloads (brain, homeostatic): the 1.5M brain as configured (saturated
# dynamics), the same brain with homeostasis on and the 0.01..0.2 sinusoidal input (quiet), and
# the 8M brain as configured
LEARNED = {"learned-1.5M": ("config1", False), "learned-homeostatic-1.5M": ("config1", True),
           "learned-8M": ("config4", False)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 3 warm-up batches + 97 timed = the 10,000 ticks of the 1.5M configuration
    ap.add_argument("--steps", type=int, default=97)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plain-1.5M",
                    choices=sorted(CONFIGS) + ["population-512"] + sorted(LEARNED))
    ap.add_argument("--learned-ticks", type=int, default=10000)
    ap.add_argument("--learned-epochs", type=int, default=30)
    ap.add_argument("--learned-ratio", type=float, default=3.0)
    ap.add_argument("--pop-brains", type=int, default=512)
    ap.add_argument("--pop-ticks", type=int, default=2000)
    ap.add_argument("--pop-warmup", type=int, default=600)
    ap.add_argument("--ticks-per-step", type=int, default=100)
    ap.add_argument("--outputs", type=int, default=4096)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-per-tick", action="store_true",
                    help="skip the per-tick entry point leg (cu_step_day_phase vs the reference's own kernels)")
    ap.add_argument("--engine", default="rows", choices=["rows", "columnar"],
                    help="batch kernels: neuron-major row engine (default) or the per-tick columnar kernels")
    return ap.parse_args()


class Dist:
    def __init__(self, n_gpus: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = os.environ.get("AXC_BENCH_BACKEND", "gloo")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """Samples SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("AXC_CLOCKS_CSV", f"/tmp/axc_clocks_{os.getpid()}.csv"))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines()[1:]:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# DRAM traffic per launch of the dominant kernel (ncu dram__bytes_read.sum + dram__bytes_write.sum) from one
# capture of the same kernel on the same workload in its steady state (tick ~1,200).  The prologue's was
# taken with one axon and neuron per thread; at this size it now runs two per thread, which move the same
# bytes.
TRAFFIC = {("plain-1.5M", "k_rows_update_lsum"): 66.5e6, ("plain-1.5M", "k_rows_prologue_plain"): 66.1e6}


def cpu_model() -> str | None:
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        return None
    for line in out.splitlines():
        if line.startswith("Model name:"):
            return line.split(":", 1)[1].strip()
    return None


def workload(name: str):
    from axicor_gb300 import workloads as W
    return getattr(W, CONFIGS[name])()


def synapse_count(state: np.ndarray, padded_n: int) -> int:
    from axicor_gb300.formats import StateView
    return int(np.count_nonzero(StateView(state, padded_n).targets))


def algorithmic_bytes(ticks, evaluated, spikes, gsop_slots, N, A, I, num_outputs):
    """Bytes a tick must move (per the Day Phase's data flow):
    6 B per evaluated slot (u32 target + i16 weight), 64 B per axon (heads read
    and written), 20 B per neuron (voltage and threshold r/w 16 B, flags and
    timer r/w 4 B), 4 B per spike (soma_to_axon), 8 B per GSOP slot (target
    re-read, weight read and written), 4 B per input word and 6 B per output."""
    return (6 * evaluated + ticks * (64 * A + 20 * N + 4 * ((I + 31) // 32) + 6 * num_outputs)
            + 4 * spikes + 8 * gsop_slots)


def update_kernel_bytes(ticks, evaluated, spikes, N):
    """Algorithmic bytes of the columnar update kernel: 6 B per evaluated slot, 20 B per neuron, 4 B per spike."""
    return 6 * evaluated + ticks * 20 * N + 4 * spikes


def rows_update_kernel_bytes(evaluated_slots, evaluated_neurons, spikes, ticks=1, lit_ticks=0, tested=0):
    """Bytes the row engine's update stage must move.  On a full-pass tick (k_rows_update): 6 B per evaluated
    slot (u32 target + i16 weight read), 24 B per evaluated neuron (flags, slot count, list entry, voltage and
    threshold read; voltage, flags, threshold, timer written), 4 B per spike (soma_to_axon).  On a lit-sum tick
    (k_rows_update_lsum) the row's frozen slots on fully-lit axons arrive as one 8-byte record (sum, tested
    length) instead of 6 B a slot: 32 B per evaluated neuron, 6 B per tested slot, 4 B per spike.  GSOP's
    write-back of the movable weights (a few hundred kB per tick in the steady state) is not counted.  With both
    forms in the window the per-neuron and per-slot terms are split by the fraction of lit-sum ticks."""
    f = lit_ticks / ticks if ticks else 0.0
    full = 6 * evaluated_slots + 24 * evaluated_neurons
    lit = 32 * evaluated_neurons + 6 * tested / f if f else 0.0
    return (1 - f) * full + f * lit + 4 * spikes


def run_gb300(args, dist: Dist) -> dict | None:
    import __graft_entry__ as G
    G.build()
    from axicor_gb300 import _native as N
    from axicor_gb300 import shard as S

    lib = N.lib()
    lib.gpu_set_device(dist.local_rank)
    engine = 1 if args.engine == "rows" else 0
    lib.axc_batch_engine_mode(engine)
    w = workload(args.workload)
    B, K, Wm = args.ticks_per_step, args.steps, args.warmup
    lay, state, heads = S.generate_brain(w.spec())
    synapses = synapse_count(state, lay.padded_n)
    S.upload_lut(w.lut)
    vram = S.VramState(lay.padded_n, lay.total_axons)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    del heads
    eng = S.ShardEngine(vram)
    words = (w.num_inputs + 31) // 32
    n_out = min(args.outputs, lay.num_neurons)
    ids = np.linspace(0, lay.num_neurons - 1, n_out).astype(np.uint32)
    d_ids = S.device_array(ids)
    io = S.IoDeviceBuffers(words, 0, n_out, B)

    total_ticks = (Wm + 2 * K + 2) * B
    bm_all = S.input_bitmask(w.seed, 0, total_ticks, w.num_inputs, w.rate_q32)
    d_bm_all = S.device_array(bm_all)
    tick = 0

    def step_device(t0):
        src = d_bm_all + t0 * words * 4
        err = lib.axc_step_day_phase_batch(C.byref(vram.ptrs), lay.padded_n, lay.total_axons, B,
                                           C.byref(io.as_struct()), src, None, None, lay.virtual_offset,
                                           w.num_inputs, d_ids, w.v_seg, w.dopamine, t0, None, eng.stream)
        if err:
            raise RuntimeError(f"axc_step_day_phase_batch failed: {err}")

    for _ in range(Wm):
        step_device(tick)
        tick += B
    eng.synchronize()

    import torch
    torch.cuda.set_device(dist.local_rank)
    stream = torch.cuda.ExternalStream(eng.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    vram.counters(reset=True)
    clocks = Clocks(dist.local_rank)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    torch.cuda.nvtx.range_push("timed")   # ncu --nvtx --nvtx-include "timed/" selects these launches
    ev0.record(stream)
    for _ in range(K):
        step_device(tick)
        tick += B
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    ctr = vram.counters()
    t_max = dist.max(ms / 1e3)
    ticks_timed = K * B
    value_tps = dist.world * ticks_timed / t_max

    # e2e: pinned host inputs and a host read of every batch's readout, through the double-buffered batch I/O
    # (axc_io_pipeline_*): each step queues one batch from host memory and reads the previous batch's readout on
    # the host, so the next upload and the last readout overlap the running batch
    h_bm = S.PinnedBuffer(K * B * words, np.uint32)
    h_bm.array[:] = bm_all[tick * words:(tick + K * B) * words]
    pipe = S.IoPipeline(vram, B, words, n_out, d_ids, lay.virtual_offset, w.num_inputs, w.v_seg)
    pipe.submit(h_bm.as_ptr(), tick, w.dopamine, eng.stream)          # warm: both buffer slots' graphs
    pipe.submit(h_bm.as_ptr() + B * words * 4, tick + B, w.dopamine, eng.stream)
    pipe.outputs(1)
    pipe.outputs(0)
    tick += 2 * B
    h_bm.array[:] = bm_all[tick * words:(tick + K * B) * words]
    readout_spikes = 0
    dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    wall0 = time.perf_counter()
    e0.record(stream)
    for k in range(K):
        pipe.submit(h_bm.as_ptr() + k * B * words * 4, tick, w.dopamine, eng.stream)
        if k:
            readout_spikes += int(pipe.outputs(1).sum())
        tick += B
    readout_spikes += int(pipe.outputs(0).sum())
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    pipe.close()
    e2e_s = dist.max(max(e0.elapsed_time(e1) / 1e3, wall))
    e2e_tps = dist.world * K * B / e2e_s

    # per-kernel CUDA-event timing on the launching stream (same regime, right after)
    prof_ticks = min(50, B)
    out_ms = (C.c_float * 5)()
    out_cnt = (C.c_uint64 * 7)()
    d_prof_bm = S.device_array(bm_all[:prof_ticks * words])
    err = lib.axc_profile_ticks(C.byref(vram.ptrs), lay.padded_n, lay.total_axons, w.v_seg, tick, prof_ticks,
                                d_prof_bm, words, lay.virtual_offset, w.num_inputs, w.dopamine, engine, eng.stream,
                                out_ms, out_cnt)
    if err:
        raise RuntimeError(f"axc_profile_ticks failed: {err}")
    stage_ms = list(out_ms)
    if engine == 1:
        names = ["network_ids", "prologue", "update", "update_lsum", "gsop_fixup_push"]
        kernels = {"prologue": "k_rows_prologue_plain", "update": "k_rows_update", "update_lsum": "k_rows_update_lsum",
                   "gsop_fixup_push": "k_rows_fixup+k_rows_push"}
    else:
        names = ["network_ids", "axons", "update", "push", "gsop"]
        kernels = {"axons": "k_axons", "update": "k_update", "push": "k_push", "gsop": "k_gsop"}
    top = int(np.argmax(stage_ms))
    ev, hits, spk, gs, nev, lit_ticks, tested = (int(x) for x in out_cnt)
    A_ = lay.total_axons
    if engine == 1 and names[top] in ("update", "update_lsum"):
        # the bytes of the ticks that pass ran (the other returns at once)
        f = lit_ticks / prof_ticks
        both = rows_update_kernel_bytes(ev, nev, spk, prof_ticks, lit_ticks, tested)
        full_only = (1 - f) * (6 * ev + 24 * nev + 4 * spk)
        kb = full_only if names[top] == "update" else both - full_only
    elif names[top] == "update":
        kb = update_kernel_bytes(prof_ticks, ev, spk, lay.padded_n)
    elif names[top] == "gsop":
        kb = 8 * gs
    elif names[top] == "prologue":
        # per axon: heads read and written (64), split masks written (8), owner count (4), pending pushes (4);
        # per neuron: timer read (1), and for the refractory ones timer written and flags read and written (3);
        # per evaluated neuron its list entry (4); per spiker its pending-push count cleared (4)
        Np_ = lay.padded_n
        kb = prof_ticks * (80 * A_ + Np_) + 3 * (prof_ticks * Np_ - nev) + 4 * nev + 4 * spk
    elif names[top] == "axons":
        kb = prof_ticks * (64 * A_ + 4 * A_ + (4 + 4) * lay.padded_n)
    else:
        kb = 68 * spk
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = kb / (stage_ms[top] / 1e3) / 1e9
    tick_bytes = algorithmic_bytes(ticks_timed, int(ctr[1]), int(ctr[3]), int(ctr[4]), lay.padded_n,
                                   lay.total_axons, w.num_inputs, n_out)

    result = {
        "ticks_per_s": value_tps,
        "events_per_s": value_tps * synapses,
        "e2e_events_per_s": e2e_tps * synapses,
        "e2e_ticks_per_s": e2e_tps,
        "ms_per_step": t_max * 1e3 / K,
        "synapses": synapses,
        "neurons": lay.num_neurons,
        "clocks": clk,
        "h2d": B * words * 4,
        "d2h": B * n_out,
        # per batch of B ticks: rows: prologue, 8-lane pass, lit-sum pass, fix-up per tick (one of the two
        # passes returns at once); push on the last tick; batch control, burst reset, list reset, layout
        # start, owner counts, row layout (the three layout kernels return at once on batches that keep
        # the copy), write-back
        "launches": K * ((4 * B + 8) if engine == 1 else (4 * B + 2)),
        "roofline": {"bound": "hbm", "kernel": kernels.get(names[top], names[top]),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": TRAFFIC.get((args.workload, kernels.get(names[top], names[top]))),
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                     "algorithmic_bytes_per_launch": kb / prof_ticks,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
        "stage_ms_per_tick": {n: m / prof_ticks for n, m in zip(names, stage_ms)},
        "tick_algorithmic_gbs": tick_bytes / (ms / 1e3) / 1e9,
        "per_tick": {"evaluated_slots": int(ctr[1]) / ticks_timed, "hits": int(ctr[2]) / ticks_timed,
                     "spikes": int(ctr[3]) / ticks_timed, "gsop_slots": int(ctr[4]) / ticks_timed,
                     "evaluated_neurons": int(ctr[5]) / ticks_timed},
        "engine": args.engine,
        "delivered_events_per_s": value_tps * int(ctr[2]) / ticks_timed,
        "lay": lay, "w": w, "vram": vram, "eng": eng, "state0": state,
    }
    lib.gpu_free(d_ids)
    lib.gpu_free(d_bm_all)
    lib.gpu_free(d_prof_bm)
    return result


def digest(vram) -> str:
    import hashlib
    h = hashlib.sha256()
    h.update(vram.download_state().tobytes())
    h.update(vram.download_heads().tobytes())
    return h.hexdigest()


def per_tick_leg(r, t0=500, ticks=100, lead=10) -> dict:
    """cu_step_day_phase, the symbol an unmodified ShardEngine calls once per tick (shard.rs:75-120), on ticks
    [t0, t0 + ticks) of the brain, against the reference's own GPU Day Phase (physics.cu compiled for sm_103a
    from the reference sources, launched in cu_step_day_phase's order) on the same ticks from the same state.
    The brain is brought from its initial state to tick t0 - lead by the batch path; `lead` untimed per-tick
    calls then precede the timed ticks on both sides (the engine's first call rebuilds its row copy).  CUDA
    events on each launching stream.  The engine's result is checked against the batch path's over the same
    ticks (sha256 of state and heads)."""
    import torch
    from axicor_gb300 import _native as N
    from axicor_gb300 import shard as S
    from oracle import refgpu   # the reference's own kernels, timed as a baseline only

    lib = N.lib()
    w, lay, vram, eng = r["w"], r["lay"], r["vram"], r["eng"]
    Np, A = lay.padded_n, lay.total_axons
    words = (w.num_inputs + 31) // 32
    start = t0 - lead
    bm = S.input_bitmask(w.seed, 0, t0 + ticks, w.num_inputs, w.rate_q32)
    d_bm = S.device_array(bm)
    io = S.IoDeviceBuffers(words, 0, 0, 100)
    try:
        vram.upload_state(r["state0"])
        vram.upload_axon_heads(np.full(A * 8, 0x80000000, np.uint32))
        t = 0
        while t < start:
            b = min(100, start - t)
            eng.step_day_phase_batch(b, io, bm[t * words:(t + b) * words], None, None, lay.virtual_offset,
                                     w.num_inputs, None, w.v_seg, w.dopamine, t)
            t += b
        eng.synchronize()
        snap_s, snap_h = vram.download_state(), vram.download_heads()
        stream = torch.cuda.ExternalStream(eng.stream)

        def engine_ticks(a, b):
            for k in range(a, b):
                err = lib.cu_step_day_phase(C.byref(vram.ptrs), Np, A, w.v_seg, k, d_bm + k * words * 4,
                                            lay.virtual_offset, w.num_inputs, None, 0, None, None, 0, w.dopamine,
                                            eng.stream)
                if err:
                    raise RuntimeError(f"cu_step_day_phase failed: {err}")

        engine_ticks(start, t0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("per_tick")   # ncu --nvtx --nvtx-include "per_tick/"
        e0.record(stream)
        engine_ticks(t0, t0 + ticks)
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        ours_s = e0.elapsed_time(e1) / 1e3
        d_ours = digest(vram)
        # the batch path over the same ticks from the same state
        vram.upload_state(snap_s)
        vram.upload_axon_heads(snap_h)
        eng.step_day_phase_batch(lead, io, bm[start * words:t0 * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, w.v_seg, w.dopamine, start)
        eng.step_day_phase_batch(ticks, io, bm[t0 * words:(t0 + ticks) * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, w.v_seg, w.dopamine, t0)
        eng.synchronize()
        same = digest(vram) == d_ours
        out = {"ticks": [t0, t0 + ticks], "entry_point": "cu_step_day_phase",
               "engine_ticks_per_s": ticks / ours_s, "engine_events_per_s": ticks * r["synapses"] / ours_s,
               "bitexact_vs_batch_path": same}
        if not refgpu.available():
            out["reference_kernels"] = "unavailable: reference cubin not built (oracle/build_ref.py needs the sources)"
            return out
        vram.upload_state(snap_s)
        vram.upload_axon_heads(snap_h)
        rk = refgpu.ReferenceKernels()
        rk.upload_lut(w.lut)
        for k in range(start, t0):
            rk.step(vram, Np, A, w.v_seg, k, d_bm + k * words * 4, lay.virtual_offset, w.num_inputs, None, 0, None,
                    None, 0, w.dopamine, sync=False)
        torch.cuda.synchronize()
        default = torch.cuda.default_stream()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(default)
        for k in range(t0, t0 + ticks):
            rk.step(vram, Np, A, w.v_seg, k, d_bm + k * words * 4, lay.virtual_offset, w.num_inputs, None, 0, None,
                    None, 0, w.dopamine, sync=False)
        r1.record(default)
        torch.cuda.synchronize()
        ref_s = r0.elapsed_time(r1) / 1e3
        out.update({"reference_kernels_ticks_per_s": ticks / ref_s,
                    "reference_kernels_events_per_s": ticks * r["synapses"] / ref_s,
                    "speedup_vs_reference_kernels": ref_s / ours_s,
                    "reference_kernels": "physics.cu compiled for sm_103a from the reference sources, launched in "
                                         "cu_step_day_phase's order (physics.cu:441-495), legacy stream"})
        return out
    finally:
        lib.gpu_free(d_bm)


def cpu_sample(w, state, heads, lay, tick0, budget_s, threads) -> dict:
    """Times the CPU restatement of the reference kernels on `threads` host threads."""
    import oracle
    from axicor_gb300 import shard as S
    words = (w.num_inputs + 31) // 32
    t_once = None
    ticks = 0
    t0 = time.perf_counter()
    while True:
        bm = S.input_bitmask(w.seed, tick0 + ticks, 1, w.num_inputs, w.rate_q32)
        s = time.perf_counter()
        oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick0 + ticks, 1, bm, words,
                         lay.virtual_offset, w.num_inputs, threads=threads)
        ticks += 1
        t_once = time.perf_counter() - s
        if time.perf_counter() - t0 + t_once > budget_s or ticks >= 200:
            break
    el = time.perf_counter() - t0
    return {"ticks": ticks, "seconds": el, "ticks_per_s": ticks / el}


def run_reference(args, dist: Dist) -> None:
    """CPU arm: the oracle (a C restatement of physics.cu) on all host cores."""
    if dist.rank != 0:
        return
    import oracle
    from axicor_gb300 import shard as S
    import __graft_entry__ as G
    G.build()
    w = workload(args.workload)
    lay, state, heads = S.generate_brain(w.spec())
    synapses = synapse_count(state, lay.padded_n)
    threads = os.cpu_count() or 1
    words = (w.num_inputs + 31) // 32
    pre = 16                      # untimed ticks that bring the brain to its steady activity
    bm = S.input_bitmask(w.seed, 0, pre, w.num_inputs, w.rate_q32)
    oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, 0, pre, bm, words,
                     lay.virtual_offset, w.num_inputs, threads=threads)
    tick = pre
    per_step = 1
    for _ in range(args.warmup):
        bm = S.input_bitmask(w.seed, tick, per_step, w.num_inputs, w.rate_q32)
        oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick, per_step, bm, words,
                         lay.virtual_offset, w.num_inputs, threads=threads)
        tick += per_step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bm = S.input_bitmask(w.seed, tick, per_step, w.num_inputs, w.rate_q32)
        oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, tick, per_step, bm, words,
                         lay.virtual_offset, w.num_inputs, threads=threads)
        tick += per_step
    el = time.perf_counter() - t0
    tps = args.steps * per_step / el
    v = tps * synapses
    line = {
        "metric": "synaptic_events_per_s", "value": v, "unit": "events/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator)", "ticks_per_s": tps,
        "config": {"workload": args.workload, "neurons": lay.num_neurons, "synapses": synapses,
                   "ticks_per_step": per_step, "pre_ticks_untimed": pre,
                   "parallelism": "single" if dist.world == 1 else "replicas"},
        "cpu_baseline": {"value": v, "unit": "events/s", "cores": threads, "cpu_model": cpu_model(), "kind": "port",
                         "sample": f"{args.steps} ticks of the {args.workload} brain after {pre + args.warmup} "
                                   f"untimed ticks, C restatement of physics.cu with OpenMP"},
        "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_population(args) -> None:
    """512 independent brains (neurons log-uniform in [1k,100k], slots in {32,64,96,128}, per-brain
    threshold / leak shift / GSOP / input rate), ticks [warm-up, warm-up + 2,000) of each timed: the population
    engine against the same brains stepped one after another through the batch entry point; every final
    state compared.  The schedule is tuned on live ticks after the warm-up (the weights' GSOP settles in the
    first few hundred ticks, and the fastest schedule differs before and after); both arms run the warm-up
    untimed from the same initial states."""
    import hashlib
    import torch
    import __graft_entry__ as G
    G.build()
    from axicor_gb300 import _native as N
    from axicor_gb300 import population as Pop
    from axicor_gb300 import workloads as W
    lib = N.lib()
    lib.gpu_set_device(0)
    count, ticks, tpg, warm = args.pop_brains, args.pop_ticks, args.ticks_per_step, args.pop_warmup
    assert warm % tpg == 0 and ticks % tpg == 0
    t0 = time.perf_counter()
    ws = W.population(count=count, ticks=warm + ticks)
    brains = [Pop.Brain(w, warm + ticks) for w in ws]
    synapses = sum(b.synapses for b in brains)
    neurons = sum(b.lay.num_neurons for b in brains)
    setup_s = time.perf_counter() - t0

    def digest(b):
        h = hashlib.sha256()
        h.update(b.vram.download_state().tobytes())
        h.update(b.vram.download_heads().tobytes())
        return h.hexdigest()

    pop = Pop.Population(brains)
    if warm:
        pop.run(0, warm, tpg)                  # untimed
    sc, cand_ms = pop.tune(warm, 2, None)      # 12 candidates x 2 live ticks
    for b in brains:
        b.reset()
    pop.run(0, warm if warm else tpg, tpg)     # the warm-up again with the chosen schedule (captures its graph)
    if not warm:
        for b in brains:
            b.reset()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(0)
    clocks.start()
    torch.cuda.nvtx.range_push("timed")
    e0.record()
    pop.run(warm, ticks, tpg)
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    pop_s = e0.elapsed_time(e1) / 1e3
    ctr = pop.counters()
    pop_digest = [digest(b) for b in brains]
    pop.close()
    # sequential: each brain alone through the batch entry point (graphs captured untimed first)
    for b in brains:
        b.reset()
        b.run_alone(0, warm if warm else tpg, batch=tpg)   # untimed (captures the graphs)
        if not warm:
            b.reset()
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    for b in brains:
        b.run_alone(warm, ticks, batch=tpg)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - s0
    same = sum(1 for b, d in zip(brains, pop_digest) if digest(b) == d)
    events = synapses * ticks
    line = {
        "metric": "synaptic_events_per_s", "value": events / pop_s, "unit": "events/s", "n_gpus": 1, "steps": 1,
        "warmup": 0, "ms_per_step": pop_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded generator, inputs resident in HBM)",
        "config": {"workload": f"population-{count}", "brains": count, "neurons": neurons, "synapses": synapses,
                   "ticks": ticks, "timed_ticks": [warm, warm + ticks], "warmup_ticks": warm,
                   "ticks_per_graph": tpg,
                   "schedule": {"lanes_per_neuron": sc.lanes_per_neuron,
                                "update_blocks_per_sm": sc.update_blocks_per_sm,
                                "aux_blocks_per_sm": sc.aux_blocks_per_sm}},
        "tuner_candidate_ms": cand_ms,
        "sequential": {"value": events / seq_s, "unit": "events/s", "seconds": seq_s,
                       "how": "each brain alone through axc_step_day_phase_batch, batches of "
                              f"{tpg} ticks, one after another"},
        "speedup_vs_sequential": seq_s / pop_s,
        "bitexact_brains": f"{same}/{count}",
        "per_tick": {"evaluated_slots": int(ctr[1]) / ticks, "spikes": int(ctr[3]) / ticks},
        "errors": int(ctr[6]),
        "clocks": clk, "setup_s": setup_s,
    }
    print(json.dumps(line), flush=True)
    for b in brains:
        b.free()


def run_learned(args) -> None:
    """The learned schedule against the plain path on the same brain and ticks.

    Ticks [0, trace): dense with trace recording (200k tile-ticks), then GPU
    training; [trace, total-200): the predictor's schedule (timed);
    [total-200, total): the predictor running but the schedule forced dense
    (the learned engine's cost over the plain path when it never goes
    sparse, in the steady state: with the gate, mostly chunks on the plain
    graph and a probe now and then).  The plain copy of the brain runs the same
    ticks through axc_step_day_phase_batch; final states are compared."""
    import hashlib
    import torch
    import __graft_entry__ as G
    G.build()
    from axicor_gb300 import _native as N
    from axicor_gb300 import learned as L
    from axicor_gb300 import shard as S
    from axicor_gb300 import workloads as W
    lib = N.lib()
    lib.gpu_set_device(0)
    brain, quiet = LEARNED[args.workload]
    w = getattr(W, brain)()
    if quiet:
        w = W.homeostatic(w)
    tpg = args.ticks_per_step
    total = args.learned_ticks
    lay, state, heads = S.generate_brain(w.spec())
    synapses = synapse_count(state, lay.padded_n)
    S.upload_lut(w.lut)
    words = max((w.num_inputs + 31) // 32, 1)
    bm = S.input_bitmask(w.seed, 0, total, w.num_inputs, w.rate_q32)
    d_bm = S.device_array(bm)
    tiles = (lay.total_axons + 1023) // 1024
    samples_cap = 200_000
    trace = -(-(samples_cap // tiles + 2) // tpg) * tpg
    window = 2 * tpg
    assert total > trace + window and (total - trace - window) % tpg == 0
    vl = S.VramState(lay.padded_n, lay.total_axons)
    vp = S.VramState(lay.padded_n, lay.total_axons)
    for v in (vl, vp):
        v.upload_state(state)
        v.upload_axon_heads(heads)
    eng = L.LearnedEngine(vl, lay.padded_n, lay.total_axons, lay.virtual_offset, w.num_inputs, d_bm, words, total,
                          w.v_seg, w.dopamine, 0, samples_cap)
    plain = S.ShardEngine(vp)
    io = S.IoDeviceBuffers(words, 0, 0, tpg)
    ps = torch.cuda.ExternalStream(plain.stream)

    def plain_run(t0, ticks):
        for t in range(t0, t0 + ticks, tpg):
            err = lib.axc_step_day_phase_batch(C.byref(vp.ptrs), lay.padded_n, lay.total_axons, tpg,
                                               C.byref(io.as_struct()), d_bm + t * words * 4, None, None,
                                               lay.virtual_offset, w.num_inputs, None, w.v_seg, w.dopamine, t,
                                               None, plain.stream)
            assert err == 0, err

    def timed(fn, stream):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    # 1. traces (dense ticks) and training
    eng.set_policy(L.Policy(policy=0))
    eng.collect(True, reset=True)
    eng.run(0, trace, tpg)
    eng.collect(False)
    plain_run(0, trace)
    torch.cuda.synchronize()
    n_samples = eng.stats()["samples"]
    t0 = time.perf_counter()
    loss, val = eng.train(epochs=args.learned_epochs, batch=1024, lr=2e-3, seed=7)
    train_s = time.perf_counter() - t0
    default = torch.cuda.default_stream()
    # 2. the learned schedule
    eng.set_policy(L.Policy(policy=-1, ratio=args.learned_ratio))
    eng.reset_stats()
    t1 = trace
    ticks = total - trace - window
    clocks = Clocks(0)
    clocks.start()
    torch.cuda.nvtx.range_push("timed")
    t_learned = timed(lambda: eng.run(t1, ticks, tpg), default)
    torch.cuda.nvtx.range_pop()
    t_plain = timed(lambda: plain_run(t1, ticks), ps)
    clk = clocks.stop()
    st = eng.stats()
    # 3. the predictor running, schedule forced dense: the learned form's cost when it never goes sparse
    t2 = t1 + ticks
    eng.set_policy(L.Policy(policy=-1, ratio=float("inf")))
    t_over = timed(lambda: eng.run(t2, window, tpg), default)
    t_plain_w = timed(lambda: plain_run(t2, window), ps)

    def digest(v):
        h = hashlib.sha256()
        h.update(v.download_state().tobytes())
        h.update(v.download_heads().tobytes())
        return h.hexdigest()

    same = digest(vl) == digest(vp)
    tps_l, tps_p = ticks / t_learned, ticks / t_plain
    ctr = vl.counters()
    line = {
        "metric": "synaptic_events_per_s", "value": tps_l * synapses, "unit": "events/s", "n_gpus": 1,
        "steps": ticks // tpg, "warmup": t1 // tpg, "ms_per_step": t_learned * 1e3 / (ticks // tpg),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator, inputs resident in HBM)", "ticks_per_s": tps_l,
        "config": {"workload": args.workload, "neurons": lay.padded_n, "synapses": synapses, "ticks": total,
                   "timed_ticks": ticks, "trace_ticks": trace, "tiles": tiles, "samples": n_samples,
                   "epochs": args.learned_epochs, "ratio": args.learned_ratio, "ticks_per_step": tpg},
        "plain": {"value": tps_p * synapses, "unit": "events/s", "ticks_per_s": tps_p,
                  "how": "the same brain and ticks through axc_step_day_phase_batch (row engine)"},
        "speedup_vs_plain": t_plain / t_learned,
        "bitexact_vs_plain": same,
        "predictor": {
            "sparse_ticks": st["sparse_ticks"], "planned_sparse": st["planned_sparse"],
            "gated_ticks": st["gated_ticks"],
            "overflow_reruns": st["overflow_reruns"],
            "misprediction_rate": st["overflow_reruns"] / max(st["planned_sparse"], 1),
            "schedule_mismatch_rate": st["schedule_mismatches"] / max(st["judged_ticks"], 1),
            "mean_abs_err_frac": st["abs_err_synapses"] / max(st["actual_synapses"], 1),
            "overhead_us_per_tick": (t_over - t_plain_w) / window * 1e6,
            "overhead_frac": (t_over - t_plain_w) / t_plain_w,
            "train_s": train_s, "train_loss_first": loss[0] if loss else None,
            "train_loss_last": loss[-1] if loss else None, "val_mse": val,
        },
        "per_tick": {"evaluated_slots": float(ctr[1]) / total, "hits": float(ctr[2]) / total,
                     "spikes": float(ctr[3]) / total},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    eng.close()


def main():
    args = parse()
    if args.workload.startswith("population"):
        run_population(args)
        return
    if args.workload in LEARNED:
        run_learned(args)
        return
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, dist)
            return
        r = run_gb300(args, dist)
        if dist.rank != 0:
            return
        cpu = None
        if not args.no_cpu_baseline and dist.world == 1:
            import oracle  # noqa: F401  (the checker doubles as the timed CPU baseline)
            vram, lay, w = r["vram"], r["lay"], r["w"]
            st, hd = vram.download_state(), vram.download_heads()
            threads = os.cpu_count() or 1
            cs = cpu_sample(w, st, hd, lay, 10 ** 6, args.cpu_sample_s, threads)
            cpu = {"value": cs["ticks_per_s"] * r["synapses"], "unit": "events/s", "cores": threads,
                   "cpu_model": cpu_model(), "kind": "port",
                   "sample": f"{cs['ticks']} ticks ({cs['seconds']:.1f} s) of the {args.workload} brain from the "
                             f"GPU's state after the timed region; C restatement of physics.cu, OpenMP",
                   "ticks_per_s": cs["ticks_per_s"]}
        per_tick = None
        if not args.no_per_tick and dist.world == 1 and args.workload == "plain-1.5M" and args.engine == "rows":
            per_tick = per_tick_leg(r)
        line = {
            "metric": "synaptic_events_per_s", "value": r["events_per_s"], "unit": "events/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded generator, inputs resident in HBM)",
            "ticks_per_s": r["ticks_per_s"],
            "delivered_events_per_s": r["delivered_events_per_s"],
            "config": {"workload": args.workload, "neurons": r["neurons"], "synapses": r["synapses"],
                       "ticks_per_step": args.ticks_per_step, "parallelism": "replicas" if dist.world > 1 else "single",
                       "l2": "inputs larger than L2 (1.37 GB .state per brain)", "gsop": True,
                       "engine": r["engine"],
                       "timed_ticks": [args.warmup * args.ticks_per_step,
                                       (args.warmup + args.steps) * args.ticks_per_step],
                       "e2e_ticks": [(args.warmup + args.steps + 2) * args.ticks_per_step,
                                     (args.warmup + 2 * args.steps + 2) * args.ticks_per_step],
                       "e2e_io": "axc_io_pipeline_*: pinned host bitmask up and readout down every step, "
                                 "double-buffered against the running batch"},
            "e2e": {"value": r["e2e_events_per_s"], "unit": "events/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"], "ticks_per_s": r["e2e_ticks_per_s"]},
            "gpu_launches": r["launches"],
            "roofline": r["roofline"],
            "tick_algorithmic_gbs": r["tick_algorithmic_gbs"],
            "stage_ms_per_tick": r["stage_ms_per_tick"],
            "per_tick": r["per_tick"],
            "clocks": r["clocks"],
            "cpu_baseline": cpu,
            "per_tick_entry_point": per_tick,
        }
        print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
