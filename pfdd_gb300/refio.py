"""Reference file formats (drop-in I/O).

* ``xi.dat`` / ``xi_bc.dat``: raw native-endian FP64, layout ``[NSV][N1][N2][N3][re,im]``
  with NSV = NS + 9 virtual-strain fields (``PFDD_Final_GPU.c:4134-4135, 4366-4382,
  4777-4788``).  Virtual fields are zero and pinned (bc = 1) in every solve here.
* ``phasefield.dat``: one line per TDGL step, ``it it_plastic gamma_0 gamma_1 gamma``
  written with ``"%d       %d         %e           %e           %e\\n"``
  (``PFDD_Final_GPU.c:4672``).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

NV = 9  # virtual strain systems (PFDD_Final_GPU.c:88)


def write_xi_files(dirpath, xi: np.ndarray, bc: np.ndarray, ns_ref: int | None = None) -> None:
    """Write ``xi.dat``/``xi_bc.dat`` for a solve with ``xi`` of shape [ns, n1, n2, n3].

    ``ns_ref`` (>= ns) is the slip-system count the reading program was built with; the
    extra systems are written as zero and pinned, followed by the 9 pinned virtual fields."""
    ns = xi.shape[0]
    ns_ref = ns if ns_ref is None else ns_ref
    nsv = ns_ref + NV
    shape = (nsv,) + xi.shape[1:] + (2,)
    x = np.zeros(shape, dtype=np.float64)
    b = np.ones(shape, dtype=np.float64)
    x[:ns, ..., 0] = xi.real
    x[:ns, ..., 1] = xi.imag
    b[:ns, ..., 0] = bc
    b[:ns, ..., 1] = bc
    d = Path(dirpath)
    x.tofile(d / "xi.dat")
    b.tofile(d / "xi_bc.dat")


def read_xi_file(path, n, nsv: int) -> np.ndarray:
    """Read a raw ``[nsv][n1][n2][n3][2]`` FP64 file into a complex128 array [nsv, n1, n2, n3]."""
    a = np.fromfile(path, dtype=np.float64)
    expect = nsv * int(np.prod(n)) * 2
    if a.size != expect:
        raise ValueError(f"{path}: {a.size} doubles, expected {expect}")
    a = a.reshape((nsv,) + tuple(n) + (2,))
    return a[..., 0] + 1j * a[..., 1]


def read_gamma_full(path) -> np.ndarray:
    """Parse the patched reference's full-precision per-step log: rows of
    ``step gamma gamma_a[0..ns-1] walltime``."""
    return np.loadtxt(path, ndmin=2)


def format_phasefield_line(it: int, step: int, gamma_a0: float, gamma_a1: float, gamma: float) -> str:
    return "%d       %d         %e           %e           %e\n" % (it, step, gamma_a0, gamma_a1, gamma)
