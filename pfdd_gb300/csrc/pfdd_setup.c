/*
 * pfdd_setup.c -- host-side setup of a PFDD solve (see include/pfdd_setup.h).
 * Restates F:2683-2754 (frec), F:1812-1909 (setfcc), F:1987-2057 (setorient),
 * F:1912-1980 (seteps) and F:1540-1637 (resolSS) of PFDD_Final_GPU.c.
 */
#include "pfdd_setup.h"

#include <math.h>

void pfdd_frec(int n, double d, double *f) {
  for (int i = 0; i < n; ++i) {
    double v = 0.0;
    if (i >= 1 && i < n / 2) v = (double)i / (double)n / d;
    if (i >= n / 2) v = ((double)i - (double)n) / (double)n / d;
    f[i] = v;
  }
}

void pfdd_setfcc(double xn[12][3], double xb[12][3], double bdiv) {
  /* four {111} planes, three <110> directions each (F:1826-1896) */
  static const signed char planes[4][3] = {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {1, 1, -1}};
  static const signed char dirs[12][3] = {{-1, 1, 0}, {0, -1, 1}, {1, 0, -1}, {-1, -1, 0}, {1, 0, 1}, {0, -1, 1},
                                          {-1, -1, 0}, {1, 0, -1}, {0, -1, -1}, {-1, 1, 0}, {1, 0, 1}, {0, -1, -1}};
  const double s3 = sqrt(3.0);
  for (int s = 0; s < 12; ++s)
    for (int j = 0; j < 3; ++j) {
      xn[s][j] = (double)planes[s / 3][j] * 1.0 / s3;
      xb[s][j] = (double)dirs[s][j] / bdiv;
    }
}

void pfdd_setorient(double th[3][3]) {
  const double r3 = sqrt(3.), r2 = sqrt(2.), r6 = sqrt(6.);
  double t[3][3] = {{r3 / 3., r3 / 3., r3 / 3.}, {-r2 / 2., r2 / 2., 0.0}, {-r6 / 6., -r6 / 6., r6 / 3.}};
  for (int i = 0; i < 3; ++i) {
    double len2 = 0.0;
    for (int j = 0; j < 3; ++j) len2 += t[i][j] * t[i][j];
    for (int j = 0; j < 3; ++j) th[i][j] = t[i][j] / len2;
  }
}

void pfdd_seteps(int ns, const double (*xn)[3], const double (*xb)[3], const double *dslip, const double th[3][3],
                 double (*eps)[3][3]) {
  for (int s = 0; s < ns; ++s) {
    double e0[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) e0[i][j] = xb[s][i] * xn[s][j] / dslip[s];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) acc += th[i][k] * th[j][l] * e0[k][l];
        eps[s][i][j] = acc;
      }
  }
}

void pfdd_resolve_shear(int ns, const double sigma[3][3], const double (*eps)[3][3], double *tau) {
  for (int s = 0; s < ns; ++s) {
    double t = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) t = t + sigma[i][j] * eps[s][i][j];
    tau[s] = t;
  }
}

void pfdd_ramp_tau(int ns, const double *tau_max, int K, double *out) {
  for (int step = 0; step < K; ++step)
    for (int s = 0; s < ns; ++s) out[(long)step * ns + s] = tau_max[s] * ((step + 1.0) / K);
}
