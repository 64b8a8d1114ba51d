"""pfdd_gb300 -- GB300-native PFDD TDGL hot path (elasticity + Ginzburg-Landau step).

The compute path is hand-written CUDA for sm_103a behind a C ABI
(``include/pfdd_gpu.h``, library ``pfdd_gb300/_lib/libpfdd_gb300.so``); this
package holds the ctypes mirror of that ABI (:mod:`pfdd_gb300.native`), the
seeded workload generators (:mod:`pfdd_gb300.workloads`), the reference file
formats (:mod:`pfdd_gb300.refio`) and the in-tree build (:mod:`pfdd_gb300.build`).
"""
from . import refio, workloads  # noqa: F401

__all__ = ["refio", "workloads", "native", "build"]
