"""Seeded synthetic PFDD workloads (initial dislocation loops + noise, stress ramps).

The reference program takes its initial order parameter either from
``initial()`` (``PFDD_Final_GPU.c:1249-1410``) or, with ``choice==2``, from the
raw FP64 files ``xi.dat``/``xi_bc.dat`` (``PFDD_Final_GPU.c:4366-4382``).
These generators produce the second form: every solve is fully described by a
:class:`SolveSpec` and is reproducible from its seeds (numpy PCG64).

Geometry follows the reference's crystal frame: slip system ``s`` of the FCC
table (``setfcc``, ``PFDD_Final_GPU.c:1812-1909``) glides on the plane whose
normal is ``theta @ n_s`` with ``theta`` from ``setorient``
(``PFDD_Final_GPU.c:1987-2057``).  For the (111) systems 0-2 that normal is the
x axis, so a loop on "plane 16" is the slab ``i == 16`` exactly as in
``initial()`` (``PFDD_Final_GPU.c:1297``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

# setfcc plane normals / Burgers directions, before normalisation (PFDD_Final_GPU.c:1826-1896)
FCC_N = np.array([[1, 1, 1]] * 3 + [[-1, 1, 1]] * 3 + [[1, -1, 1]] * 3 + [[1, 1, -1]] * 3, dtype=np.float64)
FCC_B = np.array([[-1, 1, 0], [0, -1, 1], [1, 0, -1], [-1, -1, 0], [1, 0, 1], [0, -1, 1],
                  [-1, -1, 0], [1, 0, -1], [0, -1, -1], [-1, 1, 0], [1, 0, 1], [0, -1, -1]],
                 dtype=np.float64)


def orientation() -> np.ndarray:
    """Grain orientation matrix of material 0 (``setorient``, PFDD_Final_GPU.c:1996-2056).

    Rows are [111]/sqrt3, [-110]/sqrt2, [-1-12]/sqrt6, each divided by its squared
    length, as the reference does (PFDD_Final_GPU.c:2041-2056)."""
    s3, s2, s6 = math.sqrt(3.0), math.sqrt(2.0), math.sqrt(6.0)
    th = np.array([[s3 / 3.0, s3 / 3.0, s3 / 3.0],
                   [-s2 / 2.0, s2 / 2.0, 0.0],
                   [-s6 / 6.0, -s6 / 6.0, s6 / 3.0]])
    r = (th * th).sum(axis=1)
    return th / r[:, None]


def rotated_normals() -> np.ndarray:
    """Unit slip-plane normals of the 12 FCC systems in the global frame."""
    nn = orientation() @ (FCC_N / np.sqrt(3.0)).T
    nn = nn.T
    return nn / np.linalg.norm(nn, axis=1)[:, None]


@dataclass
class Loop:
    system: int
    center: Tuple[int, int, int]
    radius: float


@dataclass
class SolveSpec:
    """One PFDD solve: grid, slip systems, material, kinetics, stress ramp and initial loops."""
    n: Tuple[int, int, int]
    ns: int
    steps: int
    sigma_max: float
    loops: List[Loop] = field(default_factory=list)
    noise_seed: int = 0
    noise_amp: float = 1e-3
    mu: float = 1.0
    nu: float = 0.3
    asf: float = 0.1          # c0 / mu
    cd2: float = 0.01         # dt * L
    dslip: float = 1.0
    d: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    name: str = ""
    pin_frac: float = 0.0     # fraction of every field's points held fixed (xi_bc = 1)
    pin_seed: int = 0
    uq2: float = 1.0          # factor of the elastic force in the update (F:3488-3489)
    c11: Optional[float] = None  # C11 of a cubic material; None: isotropic, 2 mu + lambda

    @property
    def lam(self) -> float:
        return 2.0 * self.mu * self.nu / (1.0 - 2.0 * self.nu)

    @property
    def C11(self) -> float:
        """Elastic constants (C11, C12 = lambda, C44 = mu) as the reference's
        material struct holds them."""
        return 2.0 * self.mu + self.lam if self.c11 is None else float(self.c11)

    @property
    def npts(self) -> int:
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])


def _minimum_image(x: np.ndarray, c: int, n: int) -> np.ndarray:
    return ((x - c + n // 2) % n) - n // 2


def loop_mask(n: Sequence[int], loop: Loop) -> np.ndarray:
    """Voxels of a circular slipped region: one-voxel slab of the system's rotated glide
    plane through ``center`` (minimum-image periodic distance), in-plane radius ``radius``."""
    nrm = rotated_normals()[loop.system]
    i = _minimum_image(np.arange(n[0]), loop.center[0], n[0]).astype(np.float64)
    j = _minimum_image(np.arange(n[1]), loop.center[1], n[1]).astype(np.float64)
    k = _minimum_image(np.arange(n[2]), loop.center[2], n[2]).astype(np.float64)
    di, dj, dk = np.meshgrid(i, j, k, indexing="ij")
    h = nrm[0] * di + nrm[1] * dj + nrm[2] * dk
    rho2 = di * di + dj * dj + dk * dk - h * h
    return (np.abs(h) <= 0.5) & (rho2 <= loop.radius * loop.radius)


def initial_state(spec: SolveSpec):
    """Return ``(xi, xi_bc)`` as complex128 / float64 arrays of shape ``[ns, n1, n2, n3]``.

    Re(xi) = 1 inside each loop of its system, plus U(-amp, amp) noise on Re of every
    field (PCG64, ``noise_seed``); Im(xi) = 0.  Every point evolves (xi_bc = 0) unless
    ``pin_frac`` > 0: then each point of each field is held fixed (xi_bc = 1, the
    reference's obstacle marking, skipped by plasticevolv's test at F:3482) with that
    probability (PCG64, ``pin_seed``)."""
    n1, n2, n3 = spec.n
    re = np.zeros((spec.ns, n1, n2, n3), dtype=np.float64)
    for lp in spec.loops:
        if lp.system < spec.ns:
            re[lp.system][loop_mask(spec.n, lp)] = 1.0
    if spec.noise_amp > 0:
        rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([spec.noise_seed, 1])))
        re += rng.uniform(-spec.noise_amp, spec.noise_amp, size=re.shape)
    xi = re.astype(np.complex128)
    bc = np.zeros((spec.ns, n1, n2, n3), dtype=np.float64)
    if spec.pin_frac > 0:
        rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([spec.pin_seed, 2])))
        bc[rng.random(bc.shape) < spec.pin_frac] = 1.0
    return xi, bc


def random_loops(n: Sequence[int], count: int, rmin: float, rmax: float, nsys: int, seed: int) -> List[Loop]:
    rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, 0])))
    loops = []
    for _ in range(count):
        r = float(rng.uniform(rmin, rmax))
        s = int(rng.integers(0, nsys))
        c = tuple(int(rng.integers(0, int(m))) for m in n)
        loops.append(Loop(s, c, r))
    return loops


def config0() -> SolveSpec:
    """32^3, three (111) systems, one radius-8 loop of system 0 on the slab i=16,
    sigma_xz ramp 0 -> 0.02 mu over 200 steps, noise seed 0."""
    return SolveSpec(n=(32, 32, 32), ns=3, steps=200, sigma_max=0.02,
                     loops=[Loop(0, (16, 16, 16), 8.0)], noise_seed=0, name="config0_32^3x3_fp64")


def config1(noise_seed: int = 1, sigma_max: float = 0.05, steps: int = 1000, n: int = 128) -> SolveSpec:
    """128^3, 12 FCC systems, 8 loops (radius U(8,20), system U{0..11}, centre U(grid)),
    sigma_xz ramp 0 -> 0.05 mu over 1000 steps."""
    loops = random_loops((n, n, n), 8, 8.0, 20.0, 12, seed=1)
    return SolveSpec(n=(n, n, n), ns=12, steps=steps, sigma_max=sigma_max, loops=loops,
                     noise_seed=noise_seed, name=f"config1_{n}^3x12")


def config3_replicas(count: int = 16, steps: int = 1000, n: int = 128) -> List[SolveSpec]:
    """Stress sweep: the config-1 loops, noise seeds 100.., sigma_max evenly over 0.005-0.08."""
    sig = np.linspace(0.005, 0.08, count)
    return [config1(noise_seed=100 + r, sigma_max=float(sig[r]), steps=steps, n=n) for r in range(count)]


def config4_requests(count: int = 96, seed: int = 4, scale_steps: float = 1.0) -> List[SolveSpec]:
    """Uneven serving mix: N in {32,64,128,256}^3 with p={.4,.3,.2,.1}, NS in {3,12},
    1-8 loops of radius U(4, N/6), sigma_max ~ U(0.01,0.06), 200-2000 steps."""
    rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, 2])))
    sizes = np.array([32, 64, 128, 256])
    out = []
    for q in range(count):
        n = int(rng.choice(sizes, p=[0.4, 0.3, 0.2, 0.1]))
        ns = int(rng.choice([3, 12]))
        nl = int(rng.integers(1, 9))
        sig = float(rng.uniform(0.01, 0.06))
        steps = int(rng.integers(200, 2001))
        steps = max(1, int(round(steps * scale_steps)))
        loops = random_loops((n, n, n), nl, 4.0, n / 6.0, ns, seed=1000 + q)
        out.append(SolveSpec(n=(n, n, n), ns=ns, steps=steps, sigma_max=sig, loops=loops,
                             noise_seed=2000 + q, name=f"req{q}_{n}^3x{ns}"))
    return out
