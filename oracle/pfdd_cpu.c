/*
 * pfdd_cpu.c -- CPU FP64 restatement of the PFDD TDGL hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA path is checked
 * against; it is compiled into oracle/_build/libpfdd_oracle.so and is loaded
 * only by tests/, by the smoke check and by bench.py's CPU-baseline legs.
 * Nothing in the product library links or calls it.
 *
 * Every routine restates one piece of the reference program
 * PFDD_Final_GPU.c (cited as F:<line>) in plain C, double precision, with its
 * own FFT (an iterative radix-2 transform; the reference's Numerical Recipes
 * `fourn` is not used).  Parity of this restatement with the patched
 * reference binary itself is checked by tests/test_oracle.py against the
 * committed golden vectors in tests/golden/.
 *
 * Array layouts follow the reference (F:38-65): a field index is slowest,
 * then i (N1), j (N2), k (N3, fastest); complex values are interleaved
 * [re, im] doubles.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_PI_TRUNC 3.141592654 /* F:95, truncated on purpose */

/* ------------------------------------------------------------------ */
/* tiny pthread parallel-for                                           */

typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi);
struct pf_arg { range_fn fn; void *ctx; int64_t lo, hi; };

static void *pf_thread(void *p) {
  struct pf_arg *a = (struct pf_arg *)p;
  a->fn(a->ctx, a->lo, a->hi);
  return NULL;
}

static void parallel_for(int64_t n, int nthreads, range_fn fn, void *ctx) {
  if (nthreads <= 1 || n < 2) { fn(ctx, 0, n); return; }
  if (nthreads > 256) nthreads = 256;
  if (nthreads > n) nthreads = (int)n;
  pthread_t th[256];
  struct pf_arg args[256];
  int64_t chunk = (n + nthreads - 1) / nthreads;
  int started = 0;
  for (int t = 0; t < nthreads; ++t) {
    args[t].fn = fn; args[t].ctx = ctx;
    args[t].lo = t * chunk; args[t].hi = (t + 1) * chunk < n ? (t + 1) * chunk : n;
    if (args[t].lo >= args[t].hi) break;
    if (pthread_create(&th[t], NULL, pf_thread, &args[t]) != 0) { fn(ctx, args[t].lo, args[t].hi); continue; }
    started = t + 1;
  }
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* setup: frequencies, slip systems, orientation, eigenstrains         */

/* frec, F:2683-2754: f = i/N/d for 1 <= i < N/2, (i-N)/N/d for i >= N/2
 * (Nyquist maps to -1/2), evaluated in the reference's order of tests. */
void oracle_frec(int n, double d, double *f) {
  for (int i = 0; i < n; ++i) {
    double v = 0.0;
    if (i == 0) v = 0.0;
    if (i >= 1 && i < n / 2) v = (double)(i) / (double)(n) / d;
    if (i >= n / 2) v = ((double)(i) - (double)(n)) / (double)(n) / d;
    f[i] = v;
  }
}

/* setfcc, F:1812-1909: 12 FCC systems; normals use s3 = sqrt(3) held in a
 * `float` (double in the reference's FP64 build, float_s3=0); Burgers vectors
 * divided by `bdiv` (2.0 as shipped, sqrt(2) for |b| = 1). */
void oracle_setfcc(double xn[12][3], double xb[12][3], double bdiv, int float_s3) {
  double s3 = float_s3 ? (double)(float)sqrt(3) : sqrt(3);
  static const double nsgn[4][3] = {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {1, 1, -1}};
  static const double b[12][3] = {{-1, 1, 0}, {0, -1, 1}, {1, 0, -1}, {-1, -1, 0}, {1, 0, 1}, {0, -1, 1},
                                  {-1, -1, 0}, {1, 0, -1}, {0, -1, -1}, {-1, 1, 0}, {1, 0, 1}, {0, -1, -1}};
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j < 3; ++j) {
      xn[i][j] = nsgn[i / 3][j] * 1.0 / s3;
      xb[i][j] = b[i][j] / bdiv;
    }
}

/* setorient for material 0, F:1996-2056: rows divided by their squared length. */
void oracle_setorient(double th[3][3]) {
  th[0][0] = sqrt(3.) / 3.; th[0][1] = sqrt(3.) / 3.; th[0][2] = sqrt(3.) / 3.;
  th[1][0] = -sqrt(2.) / 2.; th[1][1] = sqrt(2.) / 2.; th[1][2] = 0.0;
  th[2][0] = -sqrt(6.) / 6.; th[2][1] = -sqrt(6.) / 6.; th[2][2] = sqrt(6.) / 3.;
  double r[3];
  for (int i = 0; i < 3; ++i) {
    r[i] = 0.0;
    for (int j = 0; j < 3; ++j) r[i] += th[i][j] * th[i][j];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) th[i][j] = th[i][j] / r[i];
}

/* seteps, F:1948-1980: eps_s = theta (b_s (x) n_s / dslip_s) theta^T, not symmetrised. */
void oracle_seteps(int ns, const double (*xn)[3], const double (*xb)[3], const double *dslip,
                   const double th[3][3], double (*eps)[3][3]) {
  for (int is = 0; is < ns; ++is) {
    double epst[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) epst[i][j] = xb[is][i] * xn[is][j] / dslip[is];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double e = 0.0;
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) e += th[i][k] * th[j][l] * epst[k][l];
        eps[is][i][j] = e;
      }
  }
}

/* resolSS for a uniform stress, F:1623-1634: tau_s = sigma : eps_s. */
void oracle_resolss_uniform(int ns, const double sigma[3][3], const double (*eps)[3][3], double *tau) {
  for (int is = 0; is < ns; ++is) {
    double t = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) t = t + sigma[i][j] * eps[is][i][j];
    tau[is] = t;
  }
}

/* ------------------------------------------------------------------ */
/* Bmatrix, F:328-412 (restricted to kb < ns, the slip-slip block).    */

struct bm_ctx {
  int n1, n2, n3, ns;
  const double *fx, *fy, *fz; /* per-axis frequency tables */
  double C[3][3][3][3], mu, ll, mup, mu_inv;
  const double (*eps)[3][3];
  double *B;
};

#define DLT(i, j) ((i == j) ? 1 : 0)
#define DLT4(i, j, k, l) (((i == j) && (j == k) && (k == l)) ? 1 : 0)

static void bm_range(void *p, int64_t lo, int64_t hi) {
  struct bm_ctx *c = (struct bm_ctx *)p;
  const int64_t N = (int64_t)c->n1 * c->n2 * c->n3;
  const int ns = c->ns;
  double *acc = (double *)malloc(sizeof(double) * ns * ns);
  for (int64_t pt = lo; pt < hi; ++pt) {
    int k3 = (int)(pt % c->n3), k2 = (int)((pt / c->n3) % c->n2), k1 = (int)(pt / ((int64_t)c->n3 * c->n2));
    double fk[3] = {c->fx[k1], c->fy[k2], c->fz[k3]};
    double fk2 = fk[0] * fk[0] + fk[1] * fk[1] + fk[2] * fk[2];
    for (int q = 0; q < ns * ns; ++q) acc[q] = 0.;
    if (fk2 > 0) {
      const double mu = c->mu, ll = c->ll, mup = c->mup;
      double z2[3] = {fk[0] * fk[0] / fk2, fk[1] * fk[1] / fk2, fk[2] * fk[2] / fk2};
      double kk = 1.0 + (mu + ll) * (1 / (mu + mup * z2[0]) * z2[0] + 1 / (mu + mup * z2[1]) * z2[1] +
                                     1 / (mu + mup * z2[2]) * z2[2]);
      for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n)
          for (int u = 0; u < 3; ++u)
            for (int v = 0; v < 3; ++v) {
              double A = 0.;
              for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                  for (int k = 0; k < 3; ++k) {
                    double G_ki = 1 / fk2 * (DLT(i, k) / (mu + mup * z2[k]) -
                                             fk[i] * fk[k] / fk2 / (mu + mup * z2[i]) / (mu + mup * z2[k]) * (mu + ll) / kk);
                    for (int l = 0; l < 3; ++l) A -= c->C[k][l][u][v] * c->C[i][j][m][n] * G_ki * fk[j] * fk[l];
                  }
              A += c->C[m][n][u][v];
              for (int ka = 0; ka < ns; ++ka)
                for (int kb = 0; kb < ns; ++kb) acc[kb * ns + ka] += A * c->eps[ka][m][n] * c->eps[kb][u][v] * c->mu_inv;
            }
    }
    for (int q = 0; q < ns * ns; ++q) c->B[(int64_t)q * N + pt] = acc[q];
  }
  free(acc);
}

/* B layout [kb][ka][pt] like BB(k1,k2,k3,ka,kb) = BB[I5(k1,k2,k3,ka,kb)] (F:38, 59). */
void oracle_bmatrix(int n1, int n2, int n3, double d1, double d2, double d3, double C11, double C12, double C44,
                    int ns, const double (*eps)[3][3], double *B, int nthreads) {
  struct bm_ctx c;
  c.n1 = n1; c.n2 = n2; c.n3 = n3; c.ns = ns; c.eps = eps; c.B = B;
  double *fx = (double *)malloc(sizeof(double) * n1), *fy = (double *)malloc(sizeof(double) * n2),
         *fz = (double *)malloc(sizeof(double) * n3);
  oracle_frec(n1, d1, fx); oracle_frec(n2, d2, fy); oracle_frec(n3, d3, fz);
  c.fx = fx; c.fy = fy; c.fz = fz;
  c.mu = C44; c.mu_inv = 1. / c.mu; c.ll = C12; c.mup = C11 - C12 - 2 * C44;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 3; ++m)
          c.C[i][j][k][m] = c.mu * (DLT(i, k) * DLT(j, m) + DLT(i, m) * DLT(j, k)) + c.ll * DLT(i, j) * DLT(k, m) +
                            c.mup * DLT4(i, j, k, m);
  parallel_for((int64_t)n1 * n2 * n3, nthreads, bm_range, &c);
  free(fx); free(fy); free(fz);
}

/* ------------------------------------------------------------------ */
/* 3D complex FFT: separable radix-2 line transforms, no normalisation. */
/* Sign convention of fft_forward / fft_backward, F:209-273:           */
/* forward = exp(-2 pi i n k / N), backward = exp(+2 pi i n k / N).     */

static int ilog2i(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

static void fft_line(double *x, int n, const double *tw /* n/2 cos,sin pairs for sign */, const int *rev) {
  for (int i = 0; i < n; ++i) {
    int j = rev[i];
    if (j > i) {
      double tr = x[2 * i], ti = x[2 * i + 1];
      x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
      x[2 * j] = tr; x[2 * j + 1] = ti;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1, step = n / len;
    for (int s = 0; s < n; s += len)
      for (int q = 0; q < half; ++q) {
        double wr = tw[2 * q * step], wi = tw[2 * q * step + 1];
        double *a = x + 2 * (s + q), *b = x + 2 * (s + q + half);
        double br = b[0] * wr - b[1] * wi, bi = b[0] * wi + b[1] * wr;
        b[0] = a[0] - br; b[1] = a[1] - bi;
        a[0] = a[0] + br; a[1] = a[1] + bi;
      }
  }
}

struct fft_ctx {
  double *data; int nf, n1, n2, n3, axis, sign;
  double *tw; int *rev; int len;
};

static void fft_axis_range(void *p, int64_t lo, int64_t hi) {
  struct fft_ctx *c = (struct fft_ctx *)p;
  const int64_t N = (int64_t)c->n1 * c->n2 * c->n3;
  int L = c->len;
  double *buf = (double *)malloc(sizeof(double) * 2 * L);
  int64_t stride = c->axis == 2 ? 1 : (c->axis == 1 ? c->n3 : (int64_t)c->n2 * c->n3);
  int64_t inner = stride, outer_len = (int64_t)L * stride;
  for (int64_t line = lo; line < hi; ++line) {
    /* line enumerates (field, outer, inner) with the transformed axis removed */
    int64_t f = line / (N / L), r = line % (N / L);
    int64_t o = r / inner, in = r % inner;
    double *base = c->data + 2 * (f * N + o * outer_len + in);
    for (int l = 0; l < L; ++l) { buf[2 * l] = base[2 * l * stride]; buf[2 * l + 1] = base[2 * l * stride + 1]; }
    fft_line(buf, L, c->tw, c->rev);
    for (int l = 0; l < L; ++l) { base[2 * l * stride] = buf[2 * l]; base[2 * l * stride + 1] = buf[2 * l + 1]; }
  }
  free(buf);
}

void oracle_fft3d(int n1, int n2, int n3, int nf, double *data, int sign, int nthreads) {
  int dims[3] = {n1, n2, n3};
  const int64_t N = (int64_t)n1 * n2 * n3;
  for (int axis = 0; axis < 3; ++axis) {
    int L = dims[axis];
    if (L <= 1) continue;
    double *tw = (double *)malloc(sizeof(double) * L);
    int *rev = (int *)malloc(sizeof(int) * L);
    for (int q = 0; q < L / 2; ++q) {
      double ang = 2.0 * M_PI * (double)q / (double)L;
      tw[2 * q] = cos(ang);
      tw[2 * q + 1] = sign * sin(ang);
    }
    int lb = ilog2i(L);
    for (int i = 0; i < L; ++i) {
      int r = 0;
      for (int b = 0; b < lb; ++b) if (i & (1 << b)) r |= 1 << (lb - 1 - b);
      rev[i] = r;
    }
    struct fft_ctx c = {data, nf, n1, n2, n3, axis, sign, tw, rev, L};
    parallel_for((int64_t)nf * (N / L), nthreads, fft_axis_range, &c);
    free(tw); free(rev);
  }
}

/* ------------------------------------------------------------------ */
/* force and TDGL update                                               */

struct con_ctx { const double *data; double *d2; const double *B; int ns; int64_t N; };

/* k-space contraction, F:4609-4629: data2[a] = sum_b data[b] * BB(a,b), b ascending. */
static void con_range(void *p, int64_t lo, int64_t hi) {
  struct con_ctx *c = (struct con_ctx *)p;
  for (int64_t pt = lo; pt < hi; ++pt)
    for (int a = 0; a < c->ns; ++a) {
      double re = 0., im = 0.;
      for (int b = 0; b < c->ns; ++b) {
        double bb = c->B[((int64_t)b * c->ns + a) * c->N + pt];
        re += c->data[2 * ((int64_t)b * c->N + pt)] * bb;
        im += c->data[2 * ((int64_t)b * c->N + pt) + 1] * bb;
      }
      c->d2[2 * ((int64_t)a * c->N + pt)] = re;
      c->d2[2 * ((int64_t)a * c->N + pt) + 1] = im;
    }
}

/* force(xi): copy (F:4581-4590), forward FFT (F:4599), contraction, inverse FFT (F:4638). */
void oracle_force(int n1, int n2, int n3, int ns, const double *B, const double *xi, double *data, double *d2,
                  int nthreads) {
  int64_t N = (int64_t)n1 * n2 * n3;
  memcpy(data, xi, sizeof(double) * 2 * ns * N);
  oracle_fft3d(n1, n2, n3, ns, data, -1, nthreads);
  struct con_ctx c = {data, d2, B, ns, N};
  parallel_for(N, nthreads, con_range, &c);
  oracle_fft3d(n1, n2, n3, ns, d2, +1, nthreads);
}

/* plasticevolv, F:3470-3501 (gradient term off, F:3483).  `tau` holds the
 * already-ramped resolved shear stress of this step, one value per system
 * (tau_field == NULL) or, with tau_field, tau_field[pt*ns+a] * tau[a]. */
void oracle_update(int64_t N, int ns, double *xi, const double *bc, const double *d2, const double *cd2,
                   const double *asf, const double *dslip, double uq2, const double *tau, const double *tau_field,
                   double *gamma, double *gamma_a) {
  double nsize = (double)N;
  double g = 0.0;
  for (int a = 0; a < ns; ++a) gamma_a[a] = 0.0;
  for (int a = 0; a < ns; ++a) {
    for (int64_t pt = 0; pt < N; ++pt) {
      int64_t e = 2 * ((int64_t)a * N + pt);
      if (bc[e] == 0) {
        double t = tau_field ? tau_field[pt * ns + a] * tau[a] : tau[a];
        xi[e] -= cd2[a] * (uq2 * d2[e] / nsize + asf[a] * ORACLE_PI_TRUNC * sin(2.0 * ORACLE_PI_TRUNC * xi[e]) -
                           t / dslip[a]);
        xi[e + 1] -= uq2 * cd2[a] * (d2[e + 1] / nsize);
      }
      g += xi[e] / nsize;
      gamma_a[a] += xi[e] / nsize;
    }
  }
  *gamma = g;
}

/* The inner TDGL loop, F:4574-4691: the force used by step s is that of xi_s
 * (for s = 0 it was computed by the outer step, F:4450-4452 + 1447). */
int oracle_run(int n1, int n2, int n3, int ns, const double *B, double *xi, const double *bc, const double *cd2,
               const double *asf, const double *dslip, double uq2, int nsteps, const double *tau,
               const double *tau_field, double *gamma, double *gamma_a, int nthreads) {
  int64_t N = (int64_t)n1 * n2 * n3;
  double *data = (double *)malloc(sizeof(double) * 2 * ns * N);
  double *d2 = (double *)malloc(sizeof(double) * 2 * ns * N);
  if (!data || !d2) { free(data); free(d2); return -1; }
  oracle_force(n1, n2, n3, ns, B, xi, data, d2, nthreads);
  for (int s = 0; s < nsteps; ++s) {
    oracle_update(N, ns, xi, bc, d2, cd2, asf, dslip, uq2, tau + (int64_t)s * ns, tau_field, gamma + s,
                  gamma_a + (int64_t)s * ns);
    if (s + 1 < nsteps) oracle_force(n1, n2, n3, ns, B, xi, data, d2, nthreads);
  }
  free(data); free(d2);
  return 0;
}

/* ------------------------------------------------------------------ */
/* strain and stress fields of a state (diagnostics, §8f)              */

struct fm_ctx {
  int n1, n2, n3, ns;
  const double *fx, *fy, *fz;
  double mu, ll, mup, C[3][3][3][3];
  const double (*eps)[3][3];
  const double *xhat; /* [ns][N][2], forward FFT of xi */
  double *beta;       /* [9][N][2], component i + 3 j */
};

/* k-space strain, F:414-598 (F matrix, MT = 1 so C_rotate = C, F:486) and
 * F:761-778 (databeta = sum_a F_a,ij data_a): F_a,ij = sum_klmn C_klmn G_jk
 * eps_a,mn f_i f_l, accumulated in the reference's loop order. */
static void fm_range(void *p, int64_t lo, int64_t hi) {
  struct fm_ctx *c = (struct fm_ctx *)p;
  const int64_t N = (int64_t)c->n1 * c->n2 * c->n3;
  const double mu = c->mu, ll = c->ll, mupc = c->mup;
  for (int64_t pt = lo; pt < hi; ++pt) {
    int k3 = (int)(pt % c->n3), k2 = (int)((pt / c->n3) % c->n2), k1 = (int)(pt / ((int64_t)c->n3 * c->n2));
    double fk[3] = {c->fx[k1], c->fy[k2], c->fz[k3]};
    double fk2 = fk[0] * fk[0] + fk[1] * fk[1] + fk[2] * fk[2];
    double F[12][3][3];
    memset(F, 0, sizeof F);
    if (fk2 > 0) {
      /* G of F:538-540 */
      double z2[3] = {fk[0] * fk[0] / fk2, fk[1] * fk[1] / fk2, fk[2] * fk[2] / fk2};
      double kk = 1.0 + (mu + ll) * (1 / (mu + mupc * z2[0]) * z2[0] + 1 / (mu + mupc * z2[1]) * z2[1] +
                                     1 / (mu + mupc * z2[2]) * z2[2]);
      double G[3][3];
      for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i)
          G[k][i] = 1 / fk2 * (DLT(i, k) / (mu + mupc * z2[k]) -
                               fk[i] * fk[k] / fk2 / (mu + mupc * z2[i]) / (mu + mupc * z2[k]) * (mu + ll) / kk);
      for (int ka = 0; ka < c->ns; ++ka)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
              for (int l = 0; l < 3; ++l)
                for (int m = 0; m < 3; ++m)
                  for (int n = 0; n < 3; ++n)
                    F[ka][i][j] = F[ka][i][j] + c->C[k][l][m][n] * G[j][k] * c->eps[ka][m][n] * fk[i] * fk[l];
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double re = 0., im = 0.;
        for (int a = 0; a < c->ns; ++a) {
          re += c->xhat[2 * ((int64_t)a * N + pt)] * F[a][i][j];
          im += c->xhat[2 * ((int64_t)a * N + pt) + 1] * F[a][i][j];
        }
        c->beta[2 * ((int64_t)(i + 3 * j) * N + pt)] = re;
        c->beta[2 * ((int64_t)(i + 3 * j) * N + pt) + 1] = im;
      }
  }
}

/* Strain and stress of the state xi ([ns][N][2]) under the uniform applied
 * stress sig_app[3][3] (units of C44, the reference's sigma array, F:3820-3918):
 *   avepsd_ij = sum_a eps_a,ij <Re xi_a>                        (avestrain, F:670-688)
 *   avepst_ij = sum_kl S_ijkl sig_app_kl mu + avepsd_ij          (F:726-741; S of F:661-664
 *               with S11, S12, S44 of main, F:4261-4263)
 *   beta_ij   = IFFT(sum_a F_a,ij FFT(xi_a))/N + avepst_ij      (strain, F:761-799)
 *   eps_ij    = (beta_ij + beta_ji)/2                            (F:801-812)
 *   sig_ij    = sum_kl C_ijkl (eps_kl - sum_a eps_a,kl Re xi_a)  (stress, F:885-921)
 *   aveps, avesig: means over the grid                           (F:4063-4072, F:920)
 * Outputs: eps_out[9][N], sig_out[9][N] (component 3 i + j, real parts),
 * aveps[9], avesig[9] (3 i + j). */
void oracle_strain_stress(int n1, int n2, int n3, int ns, double C11, double C12, double C44,
                          const double (*eps)[3][3], double d1, double d2, double d3, const double *xi,
                          const double sig_app[3][3], double *eps_out, double *sig_out, double *aveps,
                          double *avesig, int nthreads) {
  const int64_t N = (int64_t)n1 * n2 * n3;
  struct fm_ctx c;
  c.n1 = n1; c.n2 = n2; c.n3 = n3; c.ns = ns; c.eps = eps;
  double *fx = (double *)malloc(sizeof(double) * n1), *fy = (double *)malloc(sizeof(double) * n2),
         *fz = (double *)malloc(sizeof(double) * n3);
  oracle_frec(n1, d1, fx); oracle_frec(n2, d2, fy); oracle_frec(n3, d3, fz);
  c.fx = fx; c.fy = fy; c.fz = fz;
  const double mu = C44, ll = C12, mup = C11 - C12 - 2 * C44;
  c.mu = mu; c.ll = ll; c.mup = mup;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 3; ++m)
          c.C[i][j][k][m] = mu * (DLT(i, k) * DLT(j, m) + DLT(i, m) * DLT(j, k)) + ll * DLT(i, j) * DLT(k, m) +
                            mup * DLT4(i, j, k, m);
  double *xhat = (double *)malloc(sizeof(double) * 2 * N * ns);
  memcpy(xhat, xi, sizeof(double) * 2 * N * ns);
  oracle_fft3d(n1, n2, n3, ns, xhat, -1, nthreads);
  double *beta = (double *)malloc(sizeof(double) * 2 * N * 9);
  c.xhat = xhat; c.beta = beta;
  parallel_for(N, nthreads, fm_range, &c);
  oracle_fft3d(n1, n2, n3, 9, beta, +1, nthreads);
  /* compliance of main (F:4261-4263) and S_ijkl of avestrain (F:661-664) */
  const double S11 = 1. / 3. * (1 / (C11 + 2 * C12) + 2 / (C11 - C12));
  const double S12 = 1. / 3. * (1 / (C11 + 2 * C12) - 1 / (C11 - C12));
  const double S44 = 1 / C44;
  double avepsd[3][3] = {{0}}, avepst[3][3];
  for (int a = 0; a < ns; ++a)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int64_t pt = 0; pt < N; ++pt) avepsd[i][j] += eps[a][i][j] * xi[2 * ((int64_t)a * N + pt)] / (double)N;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          const double Sijkl = (S11 + 2 * S12) / 3.0 * DLT(i, j) * DLT(k, l) +
                               S44 / 4.0 * (DLT(i, k) * DLT(j, l) + DLT(i, l) * DLT(j, k)) - S44 / 2.0 * DLT4(i, j, k, l) +
                               (S11 - S12) * (DLT4(i, j, k, l) - DLT(i, j) * DLT(k, l) / 3.0);
          s += Sijkl * sig_app[k][l] * mu;
        }
      avepst[i][j] = s + avepsd[i][j];
    }
  for (int q = 0; q < 9; ++q) { aveps[q] = 0.; avesig[q] = 0.; }
  for (int64_t pt = 0; pt < N; ++pt) {
    double b[3][3], e[3][3], ed[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        b[i][j] = beta[2 * ((int64_t)(i + 3 * j) * N + pt)] / (double)N + avepst[i][j];
        ed[i][j] = 0.;
        for (int a = 0; a < ns; ++a) ed[i][j] += eps[a][i][j] * xi[2 * ((int64_t)a * N + pt)];
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) e[i][j] = (b[i][j] + b[j][i]) / 2.;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.;
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) s += c.C[i][j][k][l] * (e[k][l] - ed[k][l]);
        eps_out[(int64_t)(3 * i + j) * N + pt] = e[i][j];
        sig_out[(int64_t)(3 * i + j) * N + pt] = s;
        aveps[3 * i + j] += e[i][j] / (double)N;
        avesig[3 * i + j] += s / (double)N;
      }
  }
  free(fx); free(fy); free(fz); free(xhat); free(beta);
}
