"""The generator and the oracle reproduce the committed golden traces (tests/golden/).

The traces were produced by tests/golden/make_golden.py; the GPU tests compare
the engine's output with the same files.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from axicor_gb300 import shard as S

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "day_phase_traces.json").read_text())


def golden_cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).resolve().parent / "golden" /
                                                  "make_golden.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.cases(), m.sha


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_generator_and_oracle_match_golden(engine_lib, oracle_lib, name):
    cases, sha = golden_cases()
    w, g = cases[name], GOLDEN[name]
    lay, state, heads = S.generate_brain(w.spec())
    assert (lay.padded_n, lay.total_axons) == (g["padded_n"], g["total_axons"])
    assert sha(state) == g["state_sha256"], "generator output changed"
    assert sha(heads) == g["heads_sha256"]
    assert sha(w.lut) == g["lut_sha256"]
    bm = S.input_bitmask(w.seed, 0, w.ticks, w.num_inputs, w.rate_q32)
    assert sha(bm) == g["bitmask_sha256"]
    words = (w.num_inputs + 31) // 32
    raster = np.zeros(w.ticks * ((lay.padded_n + 7) // 8), np.uint8)
    err = oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, w.v_seg, 0, w.ticks, bm, words,
                           lay.virtual_offset, w.num_inputs, dopamine=w.dopamine, raster=raster)
    counts = np.unpackbits(raster.reshape(w.ticks, -1), axis=1, bitorder="little").sum(1)
    assert counts.tolist() == g["spike_counts"]
    assert sha(raster) == g["raster_sha256"]
    assert sha(state) == g["final_state_sha256"]
    assert sha(heads) == g["final_heads_sha256"]
    assert err == g["errors"] == 0


def test_oracle_thread_count_independent(engine_lib, oracle_lib):
    cases, sha = golden_cases()
    w = cases["small"]
    outs = []
    for threads in (1, 3, 8):
        lay, state, heads = S.generate_brain(w.spec())
        bm = S.input_bitmask(w.seed, 0, 40, w.num_inputs, w.rate_q32)
        oracle.run_ticks(state, heads, w.lut, lay.padded_n, lay.total_axons, 1, 0, 40, bm, (w.num_inputs + 31) // 32,
                         lay.virtual_offset, w.num_inputs, threads=threads)
        outs.append((sha(state), sha(heads)))
    assert outs[0] == outs[1] == outs[2]
