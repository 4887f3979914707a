"""axicor_gb300 — a GB300 (sm_103a) Day Phase engine for the Axicor spiking-brain simulator.

The engine is the C-ABI library ``lib/libaxicor_day.so`` (CUDA kernels and
host runtime, built from ``csrc/`` by ``build.py``); this package is its
host-side mirror of genesis-compute's Rust interface (``shard``), the
reference's binary formats (``formats``) and the benchmark workloads
(``workloads``).
"""
from . import _native, formats, workloads  # noqa: F401

__version__ = "0.1.0"
