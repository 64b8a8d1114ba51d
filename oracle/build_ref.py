"""Build recipe for the patched reference program (test infrastructure only).

The reference is one C program, ``PFDD_Final_GPU.c``.  As shipped it never runs
a TDGL step (``NTD=0``), pins every slip system and has a refactoring
regression in ``virtualevolv``; to use it as an oracle for the TDGL hot path we
apply a small, line-anchored patch set to a build-time copy and compile that
copy with gcc.  Every patch is verified against the original line text, so a
different reference revision fails loudly instead of building something else.

The patched source and the binaries go to ``oracle/_ref/`` only (git-ignored).
On a machine without the reference checkout (the GPU host) the previously
generated ``oracle/_ref/pfdd_ref_patched.c`` is recompiled for the local
architecture, which is why that generated file is kept beside the binaries.

Patch set (line numbers of ``PFDD_Final_GPU.c``):

==  =========================  ====================================================
#   where                      what
==  =========================  ====================================================
1   82-86, 91                  NMAT=1, grid from -D, NS1=12 (FCC), NTD=2 (one
                               outer step runs the inner TDGL loop)
2   4315, 1903                 ``setfcc`` instead of ``set3D1sys``; Burgers vector
                               scaled by ``PFDD_BDIV`` (sqrt(2) gives |b|=1)
3   4186                       ``choice=2``: read xi.dat / xi_bc.dat
4   4205                       ``plastic_max = PFDD_K`` (fixed step count; the
                               environment variable PFDD_KRUN may run fewer)
5   4580                       ``interfacevolv`` disabled (bimaterial special case)
6   1432                       regression fix: the virtual DD term is not added to
                               slip row ``isb`` (the older program's semantics)
7   81, 302-304, 4278-4281,    mu = C44, lambda = C12, C11 (default 2 mu + lambda,
    4297                       isotropic; a cubic C11 with material type MT 2),
                               Asf2 and CD2 from -D
8   3876-3877, 3484, 3488      applied sigma_xz = PFDD_SIGMA, ramped by
                               (it_plastic+1)/K inside ``plasticevolv``
9   4442-4532, 4616-4645,      diagnostics that never feed xi (energies, strain,
    4326, 4329                 gradient term) behind ``PFDD_DIAG``
10  4325, 4157-4162            ``Bmatrix`` behind ``PFDD_SETUP_B`` (timing builds
                               only); big tables calloc'ed
11  4672                       extra full-precision per-step log (gamma_full.dat):
                               step, gamma, gamma_a[0..NS-1], wall-clock time
12  818, 927                   ``PFDD_STRAIN_OUT``: strain.txt / stress.txt of the
                               state at the start of outer step 1 (the initial xi:
                               the inner loop runs in that step) plus full-precision
                               dumps of the strain and stress fields
                               (eps_full.bin, sigma_full.bin)
13  4535, 4650                 full-precision copies of the energy lines:
                               energy_full.dat (checkEnergy.dat, one line per outer
                               step) and ebarrier_full.dat (one line per inner TDGL
                               step): the step, energy_in, energy_in2, energy_in3,
                               energy_in4, energy_Residual, energy_intotal
14  4269-4271                  grid spacing d1, d2, d3 from -D (the reference fixes
                               them at 1; frec and Bmatrix take them)
15  4209                       slip-plane spacing dslip from -D (fixed at 1; the
                               eigenstrains and tau/dslip take it)
16  4195                       uq2, the update's factor of the elastic force, from
                               -D (fixed at 1)
==  =========================  ====================================================
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
# the reference checkout: $PFDD_REFERENCE_DIR, else a checkout named `reference`
# beside this repository's parent directory
REF_ROOT = Path(os.environ.get("PFDD_REFERENCE_DIR", str(HERE.parents[1] / "reference")))
REF_SRC = REF_ROOT / "PFDD_Final_GPU.c"
PATCHED = REF_DIR / "pfdd_ref_patched.c"

DEFAULTS_BLOCK = r"""
/* ---- defaults for the build-time patch set (values come from -D) ---- */
#ifndef PFDD_N1
#define PFDD_N1 32
#endif
#ifndef PFDD_N2
#define PFDD_N2 32
#endif
#ifndef PFDD_N3
#define PFDD_N3 32
#endif
#ifndef PFDD_K
#define PFDD_K 20
#endif
#ifndef PFDD_SIGMA
#define PFDD_SIGMA 0.0
#endif
#ifndef PFDD_MU
#define PFDD_MU 1.0
#endif
#ifndef PFDD_LAMBDA
#define PFDD_LAMBDA 1.5
#endif
#ifndef PFDD_ASF
#define PFDD_ASF 0.1
#endif
#ifndef PFDD_CD2
#define PFDD_CD2 0.01
#endif
#ifndef PFDD_BDIV
#define PFDD_BDIV sqrt(2.0)
#endif
#ifndef PFDD_D1
#define PFDD_D1 1.0
#endif
#ifndef PFDD_DSLIP
#define PFDD_DSLIP 1.0
#endif
#ifndef PFDD_UQ2
#define PFDD_UQ2 1.0
#endif
#ifndef PFDD_C11
#define PFDD_C11 (2.0*PFDD_MU+PFDD_LAMBDA)
#endif
#ifndef PFDD_MT
#define PFDD_MT 1
#endif
#ifndef PFDD_D2
#define PFDD_D2 1.0
#endif
#ifndef PFDD_D3
#define PFDD_D3 1.0
#endif
#ifndef PFDD_DIAG
#define PFDD_DIAG 1
#endif
#ifndef PFDD_SETUP_B
#define PFDD_SETUP_B 1
#endif
#ifndef PFDD_STRAIN_OUT
#define PFDD_STRAIN_OUT 0
#endif
#define PFDD_DUMP(name_, arr_, n_) do { FILE *f_ = fopen(name_, "wb"); \
    fwrite((arr_), sizeof(*(arr_)), (size_t)(n_), f_); fclose(f_); } while (0)
static int pfdd_krun_(int k_) { const char *s_ = getenv("PFDD_KRUN"); return s_ ? atoi(s_) : k_; }
#define PFDD_LOG_ENERGY(file_, it_, e1_, e2_, e3_, e4_, er_, et_) do { static FILE *pfdd_ef_; \
    if (!pfdd_ef_) pfdd_ef_ = fopen(file_, "w"); \
    fprintf(pfdd_ef_, "%d %.17e %.17e %.17e %.17e %.17e %.17e\n", (it_), (double)(e1_), (double)(e2_), \
            (double)(e3_), (double)(e4_), (double)(er_), (double)(et_)); fflush(pfdd_ef_); } while (0)
#define PFDD_LOG_STEP(itp_, g_, g1_) do { static FILE *pfdd_gf_; int q_; \
    if (!pfdd_gf_) pfdd_gf_ = fopen("gamma_full.dat", "w"); \
    fprintf(pfdd_gf_, "%d %.17e", (itp_), (double)(g_)); \
    for (q_ = 0; q_ < NS; q_++) fprintf(pfdd_gf_, " %.17e", (double)(g1_)[q_]); \
    fprintf(pfdd_gf_, " %.9f\n", WTime()); fflush(pfdd_gf_); } while (0)
"""

# (1-based line, original substring, replacement substring)
PATCHES = [
    (26, "#include <sys/time.h>", "#include <sys/time.h>\n" + DEFAULTS_BLOCK),
    (81, "#define MT 1", "#define MT PFDD_MT"),
    (82, "#define NMAT 2", "#define NMAT 1"),
    (83, "#define N1 32", "#define N1 PFDD_N1"),
    (84, "#define N2 2 ", "#define N2 PFDD_N2 "),
    (85, "#define N3 32", "#define N3 PFDD_N3"),
    (86, "#define NS1 1 ", "#define NS1 12 "),
    (91, "#define NTD 0/", "#define NTD 2/"),
    (302, "mc->C11=168.4E9;", "mc->C11=PFDD_C11;"),
    (303, "mc->C12=121.4E9;", "mc->C12=PFDD_LAMBDA;"),
    (304, "mc->C44=23.5E9;", "mc->C44=PFDD_MU;"),
    (818, "if(it == NT-NTD-1){",
     "if (PFDD_STRAIN_OUT && it == 1) PFDD_DUMP(\"eps_full.bin\", dataeps, 2*N1*N2*N3*ND*ND);\n"
     "  if(it == NT-NTD-1 || (PFDD_STRAIN_OUT && it == 1)){"),
    (927, "if (it == NT-1 && itp == NP-1) {",
     "if (PFDD_STRAIN_OUT && it == 1) PFDD_DUMP(\"sigma_full.bin\", datasigma, 2*N1*N2*N3*ND*ND);\n"
     "  if ((it == NT-1 && itp == NP-1 && !PFDD_STRAIN_OUT) || (PFDD_STRAIN_OUT && it == 1)) {"),
    (1432, "if(isa >= NS) {", "if(0) {"),
    (1903, "xb[i][j] = xb[i][j]/2.0;", "xb[i][j] = xb[i][j]/PFDD_BDIV;"),
    (3484, "-tau[i][j][k][isa]/dslip2[isa]", "-tau[i][j][k][isa]*((it_plastic+1.0)/PFDD_K)/dslip2[isa]"),
    (3488, "-tau[i][j][k][isa]/dslip2[isa]", "-tau[i][j][k][isa]*((it_plastic+1.0)/PFDD_K)/dslip2[isa]"),
    (3876, "if ((u==0&&v==1) || (u==1&&v==0)) {", "if ((u==0&&v==2) || (u==2&&v==0)) {"),
    (3877, "sigma[i][j][k][u][v] = 0.0;", "sigma[i][j][k][u][v] = PFDD_SIGMA;"),
    (4157, "BB = malloc((NS)*(NSV)*(N1)*(N2)*(N3)*sizeof(double));",
     "BB = calloc((size_t)(NS)*(NSV)*(N1)*(N2)*(N3), sizeof(double));"),
    (4158, "FF = malloc((NS)*(N1)*(N2)*(N3)*(ND)*(ND)*sizeof(double));",
     "FF = calloc((size_t)(NS)*(N1)*(N2)*(N3)*(ND)*(ND), sizeof(double));"),
    (4159, "DD = malloc((NSV)*(N1)*(N2)*(N3)*(ND)*(ND)*sizeof(double));",
     "DD = calloc((size_t)(NSV)*(N1)*(N2)*(N3)*(ND)*(ND), sizeof(double));"),
    (4160, "FFv = malloc((NV)*(N1)*(N2)*(N3)*(ND)*(ND)*sizeof(double));",
     "FFv = calloc((size_t)(NV)*(N1)*(N2)*(N3)*(ND)*(ND), sizeof(double));"),
    (4162, "GG = malloc((2*(NS)*(NS)*(N1)*(N2)*(N3))*sizeof(double));",
     "GG = calloc((size_t)(2*(NS)*(NS)*(N1)*(N2)*(N3)), sizeof(double));"),
    (4186, "choice=1;", "choice=2;"),
    (4195, "uq2=1.0;", "uq2=PFDD_UQ2;"),
    (4205, "plastic_max =3000;", "plastic_max =pfdd_krun_(PFDD_K);"),
    (4209, "dslip = 1.0;", "dslip = PFDD_DSLIP;"),
    (4269, "d1 = 1;", "d1 = PFDD_D1;"),
    (4270, "d2 = 1;", "d2 = PFDD_D2;"),
    (4271, "d3 = 1;", "d3 = PFDD_D3;"),
    (4278, "Asf2[is] = 0.0262;", "Asf2[is] = PFDD_ASF;"),
    (4280, "Asf2[0] = 0.0064659518668288441;", "Asf2[0] = PFDD_ASF;"),
    (4281, "Asf2[1] = 0.0064659518668288441;", "Asf2[1] = PFDD_ASF;"),
    (4297, "CD2[is] = 0.1;", "CD2[is] = PFDD_CD2;"),
    (4315, "set3D1sys(xn,xb);", "setfcc(xn,xb);"),
    (4325, "Bmatrix(BB, fx,", "if (PFDD_SETUP_B) Bmatrix(BB, fx,"),
    (4326, "Fmatrix(FF, DD,", "if (PFDD_DIAG) Fmatrix(FF, DD,"),
    (4329, "Gmatrix (GG,", "if (PFDD_DIAG) Gmatrix (GG,"),
    (4442, "energy_in3 = avestrain(", "energy_in3 = (!PFDD_DIAG) ? 0 : avestrain("),
    (4443, "energy_in2 = Imatrix(", "energy_in2 = (!PFDD_DIAG) ? 0 : Imatrix("),
    (4458, "fft_backward(datag, NS);", "if (PFDD_DIAG) fft_backward(datag, NS);"),
    (4461, "calc_strain_stress(databeta,", "if (PFDD_DIAG) calc_strain_stress(databeta,"),
    (4530, "energy_in = Energy_calculation(", "energy_in = (!PFDD_DIAG) ? 0 : Energy_calculation("),
    (4532, "energy_Residual = ResidualEnergy(", "energy_Residual = (!PFDD_DIAG) ? 0 : ResidualEnergy("),
    (4535, "energy_Residual,energy_intotal);",
     "energy_Residual,energy_intotal); PFDD_LOG_ENERGY(\"energy_full.dat\", it, energy_in, energy_in2, "
     "energy_in3, energy_in4, energy_Residual, energy_intotal);"),
    (4580, "interfacevolv(xi,", "if(0)interfacevolv(xi,"),
    (4643, "fft_backward(datag, NS);", "if (PFDD_DIAG) fft_backward(datag, NS);"),
    (4645, "if (1) {//checkpass==1", "if (PFDD_DIAG) {//checkpass==1"),
    (4650, "fabs(energy_Residual),fabs(energy_intotal));",
     "fabs(energy_Residual),fabs(energy_intotal)); PFDD_LOG_ENERGY(\"ebarrier_full.dat\", it_checkEbarrier, "
     "energy_in, energy_in2, energy_in3, energy_in4, energy_Residual, energy_intotal);"),
    (4672, "gamma1[0],gamma1[1],gamma);", "gamma1[0],gamma1[1],gamma); PFDD_LOG_STEP(it_plastic, gamma, gamma1);"),
]
# the inner-loop gradient contraction ("if(isb<NS){" below line 4600)
INNER_DATAG = ("if(isb<NS){", "if(PFDD_DIAG && isb<NS){", 4600, 4630)


def write_patched_source(src: Path = REF_SRC, dst: Path = PATCHED) -> Path:
    """Apply the patch set to the reference source and write the result to ``dst``."""
    raw = src.read_bytes().decode("latin-1")
    lines = raw.split("\n")  # keeps the trailing '\r' of CRLF lines
    for ln, old, new in PATCHES:
        text = lines[ln - 1]
        if text.count(old) != 1:
            raise RuntimeError(f"patch at line {ln}: expected one '{old}' in {text!r}")
        lines[ln - 1] = text.replace(old, new)
    old, new, lo, hi = INNER_DATAG
    hits = [i for i in range(lo - 1, hi) if old in lines[i]]
    if len(hits) != 1:
        raise RuntimeError(f"inner datag patch: {len(hits)} matches")
    lines[hits[0]] = lines[hits[0]].replace(old, new)
    dst.parent.mkdir(parents=True, exist_ok=True)
    dst.write_bytes("\n".join(lines).encode("latin-1"))
    return dst


def binary_name(n, k, sigma, fp64=True, diag=False, setup_b=True, asf=0.1, cd2=0.01, strain=False,
                d=(1.0, 1.0, 1.0), dslip=1.0, uq2=1.0, mu=1.0, lam=1.5, c11=None) -> str:
    """A name for every value the build takes from -D (the values at their
    defaults left out), so that a cached binary is never reused for another
    configuration."""
    tag = "x".join(str(int(v)) for v in n)
    dtag = "" if tuple(map(float, d)) == (1.0, 1.0, 1.0) else "_d" + "x".join(f"{float(v):g}" for v in d)
    dtag += "" if float(dslip) == 1.0 else f"_sl{float(dslip):g}"
    dtag += "" if float(uq2) == 1.0 else f"_u{float(uq2):g}"
    dtag += "" if float(mu) == 1.0 else f"_mu{float(mu)!r}"
    dtag += "" if float(lam) == 1.5 else f"_la{float(lam)!r}"
    dtag += "" if c11 is None else f"_C11{float(c11)!r}"
    return (f"pfdd_ref_{tag}_k{k}_s{sigma:g}_a{asf:g}_c{cd2:g}{dtag}_{'fp64' if fp64 else 'fp32'}"
            f"{'_diag' if diag else ''}{'' if setup_b else '_nob'}{'_strain' if strain else ''}")


def compile_ref(n=(32, 32, 32), k=20, sigma=0.0, fp64=True, diag=False, setup_b=True,
                asf=0.1, cd2=0.01, mu=1.0, lam=1.5, force=False, strain=False, d=(1.0, 1.0, 1.0),
                dslip=1.0, uq2=1.0, c11=None) -> Path:
    """Compile one configuration of the patched reference; returns the binary path.
    strain=True (implies diag): strain.txt, stress.txt and the full-precision
    strain/stress dumps of the initial state (patch 12).  d: the grid spacing
    (patch 14); dslip: the slip-plane spacing (patch 15); uq2: the force factor
    (patch 16); c11: C11 when it is not the isotropic 2 mu + lambda (patch 7)."""
    diag = diag or strain
    if REF_SRC.exists() and (force or not PATCHED.exists()
                             or PATCHED.stat().st_mtime < Path(__file__).stat().st_mtime):
        write_patched_source()
    if not PATCHED.exists():
        raise FileNotFoundError("patched reference source missing (no reference checkout here)")
    out = REF_DIR / binary_name(n, k, sigma, fp64, diag, setup_b, asf, cd2, strain, d, dslip, uq2, mu, lam, c11)
    if out.exists() and out.stat().st_mtime >= PATCHED.stat().st_mtime and not force:
        return out
    defs = [f"-DPFDD_N1={n[0]}", f"-DPFDD_N2={n[1]}", f"-DPFDD_N3={n[2]}", f"-DPFDD_K={k}",
            f"-DPFDD_SIGMA={sigma!r}", f"-DPFDD_ASF={asf!r}", f"-DPFDD_CD2={cd2!r}",
            f"-DPFDD_MU={mu!r}", f"-DPFDD_LAMBDA={lam!r}",
            f"-DPFDD_DIAG={1 if diag else 0}", f"-DPFDD_SETUP_B={1 if setup_b else 0}",
            f"-DPFDD_STRAIN_OUT={1 if strain else 0}",
            f"-DPFDD_D1={float(d[0])!r}", f"-DPFDD_D2={float(d[1])!r}", f"-DPFDD_D3={float(d[2])!r}",
            f"-DPFDD_DSLIP={float(dslip)!r}", f"-DPFDD_UQ2={float(uq2)!r}"]
    if c11 is not None:  # a cubic material: MT 1 (isotropic) would reset C11 to 2 mu + lambda (F:4243-4244)
        defs += [f"-DPFDD_C11={float(c11)!r}", "-DPFDD_MT=2"]
    if fp64:
        defs.append("-Dfloat=double")
    cmd = ["gcc", "-O2", "-w", "-DUSE_FOURN", *defs]
    if platform.machine() == "x86_64":
        cmd.append("-mcmodel=medium")
    cmd += ["-o", str(out), str(PATCHED), "-lm"]
    subprocess.run(cmd, check=True)
    return out


def bench_variants():
    """Reference builds the CPU-baseline legs time: the stock FP32 spectral build at
    128^3 x 12 (FCC), hot path only (diagnostics off), B(k) setup skipped because
    only the per-step time is measured (the step's work does not depend on B's
    values), K = 1000 ramp as in the 128^3 workload."""
    return [dict(n=(128, 128, 128), k=1000, sigma=0.05, fp64=False, diag=False, setup_b=False),
            dict(n=(128, 128, 128), k=1000, sigma=0.05, fp64=True, diag=False, setup_b=False)]


def run_ref(binary: Path, workdir: Path, timeout=None, quiet=True, krun: int | None = None):
    """Run a patched-reference binary in ``workdir`` (which must hold xi.dat and xi_bc.dat).
    krun: run only the first ``krun`` steps of the K-step ramp (patch 4)."""
    env = dict(os.environ)
    if krun is not None:
        env["PFDD_KRUN"] = str(int(krun))
    with open(workdir / "stdout.log", "w") as fo:
        subprocess.run([str(binary)], cwd=workdir, check=True, timeout=timeout, env=env,
                       stdout=fo if quiet else None, stderr=subprocess.STDOUT)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "source":
        print(write_patched_source())
    else:
        print(compile_ref(force=True))
