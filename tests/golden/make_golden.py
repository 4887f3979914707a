"""Generates the golden Day Phase traces in tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

For each case: the seeded brain is generated, its .state/.axons hashes are
recorded, then the oracle runs the batch loop (genesis-compute/src/compute/shard.rs:40-124)
with the case's seeded inputs; per-tick spike counts, the SHA-256 of the
whole spike raster and of the final .state/.axons bytes are stored.  The
tests re-derive these on the CPU, and the GPU tests compare the engine's
output with them.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from axicor_gb300 import shard as S  # noqa: E402
from axicor_gb300 import workloads as W  # noqa: E402

HERE = Path(__file__).resolve().parent


def cases():
    small = W.small(dims=(16, 16, 8), slots=64, inputs=64, p=0.1, ticks=120)
    adaptive = W.small(dims=(12, 12, 12), slots=48, inputs=40, p=0.06, ticks=120, seed=99)
    adaptive.lut[0]["adaptive_mode"] = 1
    adaptive.lut[0]["adaptive_leak_gain"] = 200
    adaptive.lut[0]["adaptive_leak_max"] = 300
    adaptive.lut[0]["homeostasis_decay"] = 3
    adaptive.lut[0]["homeostasis_penalty"] = 40
    adaptive.lut[1]["spontaneous_firing_period_ticks"] = 5
    adaptive.dopamine = 60
    for v in (0, 1):
        adaptive.lut[v]["d1_affinity"] = 50
        adaptive.lut[v]["d2_affinity"] = 70
    plain16k = W.config0(ticks=300)
    return {"small": small, "adaptive": adaptive, "plain-16k-300": plain16k}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def trace(w) -> dict:
    lay, state, heads = S.generate_brain(w.spec())
    rec = {"workload": w.name, "dims": list(w.dims), "slots": w.slots, "inputs": w.num_inputs, "seed": w.seed,
           "ticks": w.ticks, "dopamine": w.dopamine, "v_seg": w.v_seg, "padded_n": lay.padded_n,
           "total_axons": lay.total_axons, "state_sha256": sha(state), "heads_sha256": sha(heads),
           "lut_sha256": sha(w.lut)}
    words = (w.num_inputs + 31) // 32
    bm = S.input_bitmask(w.seed, 0, w.ticks, w.num_inputs, w.rate_q32)
    rec["bitmask_sha256"] = sha(bm)
    raster = np.zeros(w.ticks * ((lay.padded_n + 7) // 8), np.uint8)
    err = oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, 0, w.ticks, bm, words,
                           lay.virtual_offset, w.num_inputs, dopamine=w.dopamine, raster=raster)
    r = np.unpackbits(raster.reshape(w.ticks, -1), axis=1, bitorder="little")
    rec["spike_counts"] = [int(x) for x in r.sum(1)]
    rec["raster_sha256"] = sha(raster)
    rec["final_state_sha256"] = sha(state)
    rec["final_heads_sha256"] = sha(heads)
    rec["errors"] = err
    return rec


def main():
    out = {name: trace(w) for name, w in cases().items()}
    (HERE / "day_phase_traces.json").write_text(json.dumps(out, indent=1) + "\n")
    print({k: sum(v["spike_counts"]) for k, v in out.items()})


if __name__ == "__main__":
    main()
