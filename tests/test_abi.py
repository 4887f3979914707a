"""The C-ABI library loads without a GPU and matches include/axicor_day.h.

- every function the header declares is exported and has a ctypes signature;
- struct layouts: a C probe compiled against the header prints sizeof/offsetof,
  compared with the ctypes / numpy mirrors and with the #[repr(C)] layouts of
  genesis-compute/src/ffi.rs:25-42 and genesis-core/src/layout.rs:12-74.
"""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np

from axicor_gb300 import _native as N

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "axicor_day.h"


def header_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:int32_t|void|bool|char|uint32_t)\s*\**\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_functions_exported_and_typed(engine_lib):
    names = header_functions()
    assert len(names) >= 46
    for n in names:
        assert hasattr(engine_lib, n), f"{n} is not exported"
        assert n in N.SIGNATURES, f"{n} has no ctypes signature"
    assert set(N.SIGNATURES) <= set(names), set(N.SIGNATURES) - set(names)


def test_library_loads_without_gpu(engine_lib):
    assert b"sm_103a" in engine_lib.axc_version()


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "axicor_day.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F));
int main(void) {
  printf("VariantParameters %zu %zu\n", sizeof(VariantParameters), _Alignof(VariantParameters));
  printf("BurstHeads8 %zu %zu\n", sizeof(BurstHeads8), _Alignof(BurstHeads8));
  printf("ShardVramPtrs %zu %zu\n", sizeof(ShardVramPtrs), _Alignof(ShardVramPtrs));
  printf("VramState %zu %zu\n", sizeof(VramState), _Alignof(VramState));
  printf("SpikeEvent %zu %zu\n", sizeof(SpikeEvent), _Alignof(SpikeEvent));
  printf("AxcBrainSpec %zu %zu\n", sizeof(AxcBrainSpec), _Alignof(AxcBrainSpec));
  printf("AxcBrainLayout %zu %zu\n", sizeof(AxcBrainLayout), _Alignof(AxcBrainLayout));
  printf("AxcIoBuffers %zu %zu\n", sizeof(AxcIoBuffers), _Alignof(AxcIoBuffers));
  P(VariantParameters, threshold) P(VariantParameters, rest_potential) P(VariantParameters, leak_rate)
  P(VariantParameters, homeostasis_penalty) P(VariantParameters, spontaneous_firing_period_ticks)
  P(VariantParameters, initial_synapse_weight) P(VariantParameters, gsop_potentiation)
  P(VariantParameters, gsop_depression) P(VariantParameters, homeostasis_decay)
  P(VariantParameters, refractory_period) P(VariantParameters, synapse_refractory_period)
  P(VariantParameters, signal_propagation_length) P(VariantParameters, is_inhibitory)
  P(VariantParameters, inertia_curve) P(VariantParameters, adaptive_leak_max)
  P(VariantParameters, adaptive_leak_gain) P(VariantParameters, adaptive_mode)
  P(VariantParameters, d1_affinity) P(VariantParameters, d2_affinity)
  P(ShardVramPtrs, axon_heads) P(AxcBrainSpec, seed) P(AxcIoBuffers, num_outputs)
  P(VramState, voltage) P(VramState, axon_heads) P(VramState, telemetry_spikes)
  printf("AxcZoneShard %zu %zu\n", sizeof(AxcZoneShard), _Alignof(AxcZoneShard));
  printf("AxcGhostRoute %zu %zu\n", sizeof(AxcGhostRoute), _Alignof(AxcGhostRoute));
  P(AxcZoneShard, io) P(AxcZoneShard, h_input_bitmask) P(AxcZoneShard, mapped_soma_ids_device)
  P(AxcZoneShard, dopamine) P(AxcZoneShard, h_output_history) P(AxcGhostRoute, d_src_indices)
  P(AxcGhostRoute, count)
  return 0;
}
"""


def probe(tmp_path):
    src = tmp_path / "probe.c"
    exe = tmp_path / "probe"
    src.write_text(PROBE)
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    vals = {}
    for line in out.splitlines():
        k, *v = line.split()
        vals[k] = tuple(int(x) for x in v)
    return vals


def test_struct_layouts(tmp_path):
    v = probe(tmp_path)
    # genesis-core/src/layout.rs:47-48,73-74
    assert v["VariantParameters"] == (64, 64)
    assert v["BurstHeads8"] == (32, 32)
    # ffi.rs:25-42: nine pointers
    assert v["ShardVramPtrs"] == (72, 8)
    assert v["SpikeEvent"] == (8, 1)
    # VariantParameters field offsets, layout.rs:12-45
    expected = {"threshold": 0, "rest_potential": 4, "leak_rate": 8, "homeostasis_penalty": 12,
                "spontaneous_firing_period_ticks": 16, "initial_synapse_weight": 20, "gsop_potentiation": 22,
                "gsop_depression": 24, "homeostasis_decay": 26, "refractory_period": 28,
                "synapse_refractory_period": 29, "signal_propagation_length": 30, "is_inhibitory": 31,
                "inertia_curve": 32, "adaptive_leak_max": 48, "adaptive_leak_gain": 52, "adaptive_mode": 54,
                "d1_affinity": 58, "d2_affinity": 59}
    for f, off in expected.items():
        assert v[f"VariantParameters.{f}"] == (off,), f
        assert N.VARIANT_DTYPE.fields[f][1] == off, f
    # ctypes mirrors
    assert C.sizeof(N.ShardVramPtrs) == v["ShardVramPtrs"][0]
    assert C.sizeof(N.VramStateLegacy) == v["VramState"][0]
    assert N.VramStateLegacy.axon_heads.offset == v["VramState.axon_heads"][0]
    assert C.sizeof(N.AxcBrainSpec) == v["AxcBrainSpec"][0]
    assert N.AxcBrainSpec.seed.offset == v["AxcBrainSpec.seed"][0]
    assert C.sizeof(N.AxcBrainLayout) == v["AxcBrainLayout"][0]
    assert C.sizeof(N.AxcIoBuffers) == v["AxcIoBuffers"][0]
    assert N.AxcIoBuffers.num_outputs.offset == v["AxcIoBuffers.num_outputs"][0]
    assert C.sizeof(N.AxcZoneShard) == v["AxcZoneShard"][0]
    assert C.sizeof(N.AxcGhostRoute) == v["AxcGhostRoute"][0]
    for f in ("io", "h_input_bitmask", "mapped_soma_ids_device", "dopamine", "h_output_history"):
        assert getattr(N.AxcZoneShard, f).offset == v[f"AxcZoneShard.{f}"][0], f
    for f in ("d_src_indices", "count"):
        assert getattr(N.AxcGhostRoute, f).offset == v[f"AxcGhostRoute.{f}"][0], f


def test_variant_dtype_roundtrip():
    lut = np.zeros(16, dtype=N.VARIANT_DTYPE)
    lut[3]["adaptive_leak_max"] = -5
    lut[3]["d2_affinity"] = 7
    raw = lut.view(np.uint8).reshape(16, 64)
    assert raw[3, 48:52].view(np.int32)[0] == -5
    assert raw[3, 59] == 7
