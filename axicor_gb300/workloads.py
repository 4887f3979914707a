"""Seeded synthetic workloads: brain specs, variant LUTs and input rates.

Mapping of the benchmark configurations onto the reference arithmetic
(genesis-compute/src/cuda/physics.cu):

- threshold 2000, rest 0 (reset = rest), refractory 3 ticks;
- "leak = membrane >> 4": the reference leak is linear (|V - rest| - leak_rate,
  physics.cu:226-235), so leak_rate = threshold >> shift (125 for shift 4);
- signal_propagation_length 4 ("burst length 4"), v_seg = 1;
- GSOP +8 / -4: gsop_potentiation 8, gsop_depression 4, inertia_curve[0] = 128;
  the reference clamps |w| to [0, 32767] with the sign frozen (physics.cu:361-371),
  so the +-2047 clamp becomes inertia_curve[1..15] = 0 (|w| stops moving once
  it reaches 2048);
- variant 0 excitatory, variant 1 inhibitory; inputs are excitatory;
- dopamine 0, no homeostasis, no heartbeat.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._native import VARIANT_DTYPE, AxcBrainSpec

DEFAULT_RADIUS = 48
DEFAULT_LAMBDA = 4


def variant(threshold: int = 2000, leak_shift: int = 4, pot: int = 8, dep: int = 4, refractory: int = 3,
            prop: int = 4, inhibitory: bool = False) -> np.ndarray:
    v = np.zeros((), dtype=VARIANT_DTYPE)
    v["threshold"] = threshold
    v["rest_potential"] = 0
    v["leak_rate"] = threshold >> leak_shift
    v["gsop_potentiation"] = pot
    v["gsop_depression"] = dep
    v["refractory_period"] = refractory
    v["signal_propagation_length"] = prop
    v["is_inhibitory"] = 1 if inhibitory else 0
    curve = np.zeros(16, dtype=np.uint8)
    curve[0] = 128
    v["inertia_curve"] = curve
    return v


def default_lut(**kw) -> np.ndarray:
    lut = np.zeros(16, dtype=VARIANT_DTYPE)
    lut[0] = variant(inhibitory=False, **kw)
    lut[1] = variant(inhibitory=True, **kw)
    return lut


def p_q32(p: float) -> int:
    return min(int(round(p * 4294967296.0)), 0xFFFFFFFF)


@dataclass
class Workload:
    name: str
    dims: tuple[int, int, int]
    slots: int
    num_inputs: int
    ticks: int
    seed: int
    lut: np.ndarray
    rate_q32: np.ndarray            # per-tick input probability table (Q0.32)
    v_seg: int = 1
    dopamine: int = 0
    inhibitory_permille: int = 200
    radius: int = DEFAULT_RADIUS
    lambda_voxels: int = DEFAULT_LAMBDA
    w_min: int = 50
    w_max: int = 800
    extra: dict = field(default_factory=dict)

    @property
    def num_neurons(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    def spec(self) -> AxcBrainSpec:
        return AxcBrainSpec(self.dims[0], self.dims[1], self.dims[2], self.slots, self.num_inputs,
                            self.inhibitory_permille, self.radius, self.lambda_voxels, self.w_min, self.w_max,
                            self.seed)


def config0(seed: int = 0xA11C0, ticks: int = 1000) -> Workload:
    """16,384 neurons on 32x32x16, 128 slots, 256 inputs at p=0.05, 1,000 ticks."""
    return Workload("plain-16k", (32, 32, 16), 128, 256, ticks, seed, default_lut(),
                    np.array([p_q32(0.05)], dtype=np.uint32))


def config1(seed: int = 0xA11C1, ticks: int = 10000) -> Workload:
    """1,507,328 neurons on 128x128x92, 100 slots (150.7M synapses), 4,096 inputs at p=0.05."""
    return Workload("plain-1.5M", (128, 128, 92), 100, 4096, ticks, seed, default_lut(),
                    np.array([p_q32(0.05)], dtype=np.uint32))


def config4(seed: int = 0xA11C4, ticks: int = 5000) -> Workload:
    """8,000,000 neurons on 200^3, 128 slots (1.02B synapses), 8,192 inputs with a
    rate modulated sinusoidally between 0.01 and 0.2 over 100 ticks."""
    rates = np.array([p_q32(0.01 + 0.19 * 0.5 * (1.0 - math.cos(2.0 * math.pi * t / 100.0)))
                      for t in range(100)], dtype=np.uint32)
    return Workload("plain-8M", (200, 200, 200), 128, 8192, ticks, seed, default_lut(), rates)


def sinusoid_rates(lo: float = 0.01, hi: float = 0.2, period: int = 100) -> np.ndarray:
    """Per-tick input probability lo..hi..lo over `period` ticks (Q0.32)."""
    return np.array([p_q32(lo + (hi - lo) * 0.5 * (1.0 - math.cos(2.0 * math.pi * t / period)))
                     for t in range(period)], dtype=np.uint32)


def homeostatic(w: Workload, penalty: int = 16000, decay: int = 80) -> Workload:
    """The same brain with homeostasis on (each spike raises the neuron's
    threshold offset by `penalty`, which then decays by `decay` per tick) and
    the sinusoidal 0.01..0.2 input rate.  After a transient of about 300 ticks
    a few neurons per thousand fire per tick and about 3% of the evaluated
    slots are hit, following the 100-tick input cycle: the quiet regime the
    learned schedule's sparse form is for."""
    lut = w.lut.copy()
    for v in (0, 1):
        lut[v]["homeostasis_penalty"] = penalty
        lut[v]["homeostasis_decay"] = decay
    return Workload(w.name.replace("plain", "homeostatic"), w.dims, w.slots, w.num_inputs, w.ticks, w.seed, lut,
                    sinusoid_rates(), w.v_seg, w.dopamine, w.inhibitory_permille, w.radius, w.lambda_voxels,
                    w.w_min, w.w_max, dict(w.extra))


def small(dims=(16, 16, 8), slots=64, inputs=64, p=0.08, ticks=50, seed=7, **lut_kw) -> Workload:
    """Small brains for parity tests."""
    return Workload(f"small-{dims[0]}x{dims[1]}x{dims[2]}", tuple(dims), slots, inputs, ticks, seed,
                    default_lut(**lut_kw), np.array([p_q32(p)], dtype=np.uint32))


def cube_dims(n: int) -> tuple[int, int, int]:
    x = max(1, int(round(n ** (1.0 / 3.0))))
    z = max(1, -(-n // (x * x)))
    return (x, x, z)


def population(seed: int = 0xA11C2, count: int = 512, ticks: int = 2000) -> list[Workload]:
    """512 brains: neurons log-uniform in [1k, 100k], slots in {32,64,96,128},
    threshold in [1500,2500], leak shift in {3,4,5}, GSOP +[4,16]/-[2,8],
    input rate in [0.01,0.1]; inputs = neurons/64 (the 16k-neuron ratio)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(1000.0), math.log(100000.0)))))
        dims = cube_dims(n)
        slots = int(rng.choice([32, 64, 96, 128]))
        thr = int(rng.integers(1500, 2501))
        shift = int(rng.choice([3, 4, 5]))
        pot = int(rng.integers(4, 17))
        dep = int(rng.integers(2, 9))
        rate = float(rng.uniform(0.01, 0.1))
        nn = dims[0] * dims[1] * dims[2]
        lut = default_lut(threshold=thr, leak_shift=shift, pot=pot, dep=dep)
        out.append(Workload(f"pop-{i}", dims, slots, max(32, nn // 64), ticks, seed * 1000 + i, lut,
                            np.array([p_q32(rate)], dtype=np.uint32)))
    return out
