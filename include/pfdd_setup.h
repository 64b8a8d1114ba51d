/*
 * pfdd_setup.h -- host-side setup of a PFDD solve (crystal geometry, stresses).
 *
 * These restate the setup routines of the reference program PFDD_Final_GPU.c
 * (cited F:<line>) that feed the TDGL hot path.  They run once per solve on the
 * host in FP64; B(k) itself is built on the device by pfdd_build_B.
 */
#ifndef PFDD_SETUP_H
#define PFDD_SETUP_H

#ifdef __cplusplus
extern "C" {
#endif

/* frec, F:2683-2754: f_i = i/N/d (1 <= i < N/2), (i-N)/N/d (i >= N/2), f_0 = 0. */
void pfdd_frec(int n, double d, double *f);

/* setfcc, F:1812-1909: the 12 FCC {111}<110> systems.  Normals are (+-1,+-1,+-1)/sqrt3;
 * Burgers vectors <110>/bdiv (bdiv = 2 as shipped, sqrt(2) for |b| = 1). */
void pfdd_setfcc(double xn[12][3], double xb[12][3], double bdiv);

/* setorient for material 0, F:1987-2057: rows [111]/sqrt3, [-110]/sqrt2,
 * [-1-12]/sqrt6, each divided by its squared length. */
void pfdd_setorient(double th[3][3]);

/* seteps, F:1912-1980: eps_s = th (b_s (x) n_s / dslip_s) th^T (not symmetrised). */
void pfdd_seteps(int ns, const double (*xn)[3], const double (*xb)[3], const double *dslip, const double th[3][3],
                 double (*eps)[3][3]);

/* resolSS for a uniform stress, F:1623-1634: tau_s = sigma : eps_s. */
void pfdd_resolve_shear(int ns, const double sigma[3][3], const double (*eps)[3][3], double *tau);

/* Per-step ramped stress of the stress-ramp convention: tau_s(step) =
 * tau_max_s * ((step + 1.0) / K), evaluated exactly as the ramp is applied
 * inside plasticevolv.  out[step][ns]. */
void pfdd_ramp_tau(int ns, const double *tau_max, int K, double *out);

#ifdef __cplusplus
}
#endif

#endif
