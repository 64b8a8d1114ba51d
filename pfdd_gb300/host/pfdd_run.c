/*
 * pfdd_run.c -- C host driver: the reference program's TDGL loop on the GPU.
 *
 * Mirrors the hot path of `main` in PFDD_Final_GPU.c (F:4087-4847) for a
 * homogeneous FCC crystal: reads xi.dat / xi_bc.dat (F:4366-4382, choice==2),
 * builds the slip systems (setfcc F:1812-1909, setorient F:1987-2057, seteps
 * F:1912-1980), the resolved shear stress of an applied sigma_xz (resolSS
 * F:1540-1637), builds B(k) on the GPU (Bmatrix F:328-412), runs K TDGL steps
 * with a linear stress ramp (plasticevolv F:3470-3501, loop F:4574-4691),
 * and writes phasefield.dat (F:4672), gamma_full.dat (full precision) and
 * xi.dat (F:4777-4788) in the working directory.  With --strain it also
 * writes strain.txt (F:818-831) and stress.txt (F:927-944) of the state it
 * starts from, and stress-strain.dat (F:4063-4072, 4694-4698): the grid means
 * of strain and stress (over C44) of the starting state and of the final
 * state, then the final gamma_a and gamma.  With --converge the loop stops
 * where the reference's convergence test ends it (plasticconverge,
 * F:3732-3785) and the files hold the steps that ran.
 *
 * usage: pfdd_run N1 N2 N3 NS K SIGMA [--nsfile NSF] [--asf A] [--cd2 C]
 *                 [--mu MU] [--lambda LAM] [--c11 C11] [--dslip DS] [--uq2 U]
 *                 [--d D1 D2 D3] [--bdiv BD] [--fp32] [--device D]
 *                 [--strain] [--converge]
 *
 * MU, LAM: C44 and C12 (F:302-304); C11 defaults to the isotropic 2 MU + LAM
 * (F:4243-4244), --c11 gives a cubic material (the reference's MT 2).  DS: the
 * slip-plane spacing (dslip, F:4209), U: the update's force factor (uq2,
 * F:4195), D1 D2 D3: the grid spacing (d1, d2, d3, F:4269-4271); all 1 by
 * default, as the reference sets them.
 *
 * NSF (default NS) is the slip-system count of the files; systems NS..NSF-1
 * and the 9 virtual-strain fields must be zero and pinned (they contribute
 * nothing to the force and never evolve).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "pfdd_gpu.h"
#include "pfdd_setup.h"

static double wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + tv.tv_usec / 1e6;
}

static int die(const char *msg, pfdd_ctx *c, int st) {
  fprintf(stderr, "pfdd_run: %s: %s %s\n", msg, pfdd_status_string(st), c ? pfdd_last_error(c) : "");
  return 1;
}

/* strain.txt (F:818-831) and stress.txt (F:927-944, rows with j == 0); the
 * first six stress columns are the applied stress field (SIGMAV, which holds
 * it when no virtual strain evolves), the next six the stress field. */
static int write_fields(int n1, int n2, int n3, const double *e, const double *sg, const double sig[3][3]) {
  const long N = (long)n1 * n2 * n3;
  FILE *f3 = fopen("strain.txt", "w"), *f5 = fopen("stress.txt", "w");
  if (!f3 || !f5) return 1;
  fprintf(f3, "x,y,z,eps11,eps13,eps21,eps22,eps23,eps31,eps32,eps33\n");
  fprintf(f5, "x,y,z,sigma11,sigma12,sigma13,sigma22,sigma23,sigma33,datasigma11,datasigma12,datasigma13,datasigma22,"
              "datasigma23,datasigma33 \n");
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n2; ++j)
      for (int k = 0; k < n3; ++k) {
        const long pt = ((long)i * n2 + j) * n3 + k;
        fprintf(f3, "%d,%d,%d", i, j, k);
        for (int q = 0; q < 9; ++q) fprintf(f3, ",%lf", e[(long)q * N + pt]);
        fprintf(f3, " \n");
        if (j == 0) {
          fprintf(f5, "%d,%d,%d,%lf,%lf,%lf,%lf,%lf,%lf", i, j, k, sig[0][0], sig[0][1], sig[0][2], sig[1][1],
                  sig[1][2], sig[2][2]);
          const int comp[6] = {0, 1, 2, 4, 5, 8};
          for (int q = 0; q < 6; ++q) fprintf(f5, ",%lf", sg[(long)comp[q] * N + pt]);
          fprintf(f5, "\n");
        }
      }
  fclose(f3); fclose(f5);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: %s N1 N2 N3 NS K SIGMA [--nsfile NSF] [--asf A] [--cd2 C] [--mu MU] [--lambda LAM] "
                    "[--c11 C11] [--dslip DS] [--uq2 U] [--d D1 D2 D3] [--bdiv BD] [--fp32] [--device D] [--strain] "
                    "[--converge]\n", argv[0]);
    return 2;
  }
  int n1 = atoi(argv[1]), n2 = atoi(argv[2]), n3 = atoi(argv[3]), ns = atoi(argv[4]), K = atoi(argv[5]);
  double sigma_max = atof(argv[6]);
  int nsf = ns, prec = PFDD_FP64, dev = 0, strain = 0, conv = 0;
  double asf = 0.1, cd2 = 0.01, mu = 1.0, lam = 1.5, bdiv = sqrt(2.0);
  double c11 = NAN, dsl = 1.0, uq2 = 1.0, dd[3] = {1.0, 1.0, 1.0};
  for (int i = 7; i < argc; ++i) {
    if (!strcmp(argv[i], "--nsfile") && i + 1 < argc) nsf = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--asf") && i + 1 < argc) asf = atof(argv[++i]);
    else if (!strcmp(argv[i], "--cd2") && i + 1 < argc) cd2 = atof(argv[++i]);
    else if (!strcmp(argv[i], "--mu") && i + 1 < argc) mu = atof(argv[++i]);
    else if (!strcmp(argv[i], "--lambda") && i + 1 < argc) lam = atof(argv[++i]);
    else if (!strcmp(argv[i], "--c11") && i + 1 < argc) c11 = atof(argv[++i]);
    else if (!strcmp(argv[i], "--dslip") && i + 1 < argc) dsl = atof(argv[++i]);
    else if (!strcmp(argv[i], "--uq2") && i + 1 < argc) uq2 = atof(argv[++i]);
    else if (!strcmp(argv[i], "--d") && i + 3 < argc) {
      for (int q = 0; q < 3; ++q) dd[q] = atof(argv[++i]);
    }
    else if (!strcmp(argv[i], "--bdiv") && i + 1 < argc) bdiv = atof(argv[++i]);
    else if (!strcmp(argv[i], "--fp32")) prec = PFDD_FFT_FP32;
    else if (!strcmp(argv[i], "--device") && i + 1 < argc) dev = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--strain")) strain = 1;
    else if (!strcmp(argv[i], "--converge")) conv = 1;
    else { fprintf(stderr, "unknown option %s\n", argv[i]); return 2; }
  }
  if (ns < 1 || ns > 12 || nsf < ns || K < 1) { fprintf(stderr, "bad NS/K\n"); return 2; }
  if (!(dsl > 0) || !(dd[0] > 0) || !(dd[1] > 0) || !(dd[2] > 0) || !isfinite(uq2) || !isfinite(dsl) ||
      !isfinite(dd[0]) || !isfinite(dd[1]) || !isfinite(dd[2])) {
    fprintf(stderr, "bad spacing or force factor\n");
    return 2;
  }
  const long N = (long)n1 * n2 * n3;
  const int nsv = nsf + 9;
  const size_t cnt = (size_t)2 * nsv * N;
  double *xi = malloc(cnt * sizeof(double)), *bc = malloc(cnt * sizeof(double));
  if (!xi || !bc) { fprintf(stderr, "out of host memory\n"); return 1; }
  FILE *fx = fopen("xi.dat", "rb"), *fb = fopen("xi_bc.dat", "rb");
  if (!fx || !fb || fread(xi, sizeof(double), cnt, fx) != cnt || fread(bc, sizeof(double), cnt, fb) != cnt) {
    fprintf(stderr, "cannot read xi.dat / xi_bc.dat of %zu doubles\n", cnt);
    return 1;
  }
  fclose(fx); fclose(fb);
  for (size_t e = (size_t)2 * ns * N; e < cnt; ++e)
    if (xi[e] != 0.0 || bc[e - (e & 1)] == 0.0) {
      fprintf(stderr, "fields beyond the first %d slip systems must be zero and pinned\n", ns);
      return 1;
    }

  /* setup (F:4253-4330) */
  /* isotropic: C11 = 2 C44 + C12 (F:4243-4245); a cubic C11 with --c11 */
  double C44 = mu, C12 = lam, C11 = isnan(c11) ? 2. * C44 + C12 : c11;
  double xn[12][3], xb[12][3], th[3][3], dslip[12], eps[12][3][3], tau_max[12];
  for (int s = 0; s < 12; ++s) dslip[s] = dsl;
  pfdd_setfcc(xn, xb, bdiv);
  pfdd_setorient(th);
  pfdd_seteps(12, (const double(*)[3])xn, (const double(*)[3])xb, dslip, (const double(*)[3])th, eps);
  double sig[3][3] = {{0, 0, sigma_max}, {0, 0, 0}, {sigma_max, 0, 0}};
  pfdd_resolve_shear(ns, (const double(*)[3])sig, (const double(*)[3][3])eps, tau_max);
  double *tau = malloc(sizeof(double) * (size_t)K * ns);
  pfdd_ramp_tau(ns, tau_max, K, tau);
  double cdv[12], asfv[12];
  for (int s = 0; s < 12; ++s) { cdv[s] = cd2; asfv[s] = asf; }

  pfdd_ctx *c = NULL;
  int st;
  double t0 = wtime();
  if ((st = pfdd_create(&c, n1, n2, n3, ns, prec, dev)) != PFDD_OK) return die("create", c, st);
  if ((st = pfdd_build_B(c, C11, C12, C44, &eps[0][0][0], dd[0], dd[1], dd[2])) != PFDD_OK) return die("build_B", c, st);
  if ((st = pfdd_set_params(c, cdv, asfv, dslip, uq2)) != PFDD_OK) return die("set_params", c, st);
  if ((st = pfdd_set_state(c, xi, bc)) != PFDD_OK) return die("set_state", c, st);
  double *gamma = malloc(sizeof(double) * K), *gamma_a = malloc(sizeof(double) * (size_t)K * ns);
  double ave0[2][9], ave1[2][9];
  if (strain) {  /* strain and stress of the starting state (outer step before the inner loop) */
    double *e = malloc(sizeof(double) * 9 * (size_t)N), *sg = malloc(sizeof(double) * 9 * (size_t)N);
    if (!e || !sg) { fprintf(stderr, "out of host memory\n"); return 1; }
    if ((st = pfdd_strain_stress(c, 0, &sig[0][0], e, sg, ave0[0], ave0[1])) != PFDD_OK) return die("strain", c, st);
    if (write_fields(n1, n2, n3, e, sg, (const double(*)[3])sig)) { fprintf(stderr, "cannot write strain.txt\n"); return 1; }
    free(e); free(sg);
  }
  double t1 = wtime();
  int Kr = K; /* steps that ran */
  if (!conv) {
    if ((st = pfdd_step(c, K, tau, gamma, gamma_a)) != PFDD_OK) return die("step", c, st);
  } else {
    if ((st = pfdd_converge_reset(c, 0.0)) != PFDD_OK) return die("converge_reset", c, st);
    if ((st = pfdd_step_converge(c, K, tau, gamma, gamma_a, &Kr)) != PFDD_OK) return die("step_converge", c, st);
  }
  double t2 = wtime();
  if ((st = pfdd_get_state(c, xi)) != PFDD_OK) return die("get_state", c, st);

  FILE *pf = fopen("phasefield.dat", "w"), *gf = fopen("gamma_full.dat", "w");
  for (int s = 0; s < Kr; ++s) {
    /* it = 1: the single outer step that runs the inner loop; it_plastic counts from 1 */
    fprintf(pf, "%d       %d         %e           %e           %e\n", 1, s + 1, gamma_a[(size_t)s * ns],
            ns > 1 ? gamma_a[(size_t)s * ns + 1] : 0.0, gamma[s]);
    fprintf(gf, "%d %.17e", s + 1, gamma[s]);
    for (int a = 0; a < ns; ++a) fprintf(gf, " %.17e", gamma_a[(size_t)s * ns + a]);
    fprintf(gf, "\n");
  }
  fclose(pf); fclose(gf);
  if (strain) {  /* stress-strain.dat: means (stress over C44) of the start and final states, gamma */
    if ((st = pfdd_strain_stress(c, 0, &sig[0][0], NULL, NULL, ave1[0], ave1[1])) != PFDD_OK) return die("strain", c, st);
    FILE *f2 = fopen("stress-strain.dat", "w");
    if (!f2) { fprintf(stderr, "cannot write stress-strain.dat\n"); return 1; }
    for (int q = 0; q < 9; ++q) fprintf(f2, "%e %e ", ave0[0][q], ave0[1][q] / C44);
    for (int q = 0; q < 9; ++q) fprintf(f2, "%e %e ", ave1[0][q], ave1[1][q] / C44);
    for (int a = 0; a < nsf; ++a) fprintf(f2, "\t%e", a < ns ? gamma_a[(size_t)(Kr - 1) * ns + a] : 0.0);
    fprintf(f2, " %e \n", gamma[Kr - 1]);
    fclose(f2);
  }
  FILE *fo = fopen("xi.dat", "r+b");
  if (!fo || fwrite(xi, sizeof(double), cnt, fo) != cnt) { fprintf(stderr, "cannot write xi.dat\n"); return 1; }
  fclose(fo);
  printf("pfdd_run: %dx%dx%d ns=%d K=%d of %d %s setup %.3fs steps %.3fs (%.1f steps/s)\n", n1, n2, n3, ns, Kr, K,
         prec == PFDD_FP64 ? "fp64" : "fp32", t1 - t0, t2 - t1, Kr / (t2 - t1));
  pfdd_destroy(c);
  free(xi); free(bc); free(tau); free(gamma); free(gamma_a);
  return 0;
}
