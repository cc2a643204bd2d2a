/*
 * g3l_oracle.h -- CPU restatement of the G3LHalo aperture-statistics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py call it to produce the reference
 * answer.  The product library (libg3lgpu.so) never links, loads or calls it.
 *
 * It restates, in plain C with the same IEEE double operation order, the
 * reference's
 *   - halo-model integrands (src/NNMap_Model.cu, src/NMapMap_Model.cu,
 *     src/generalFunctions.cu, src/HOD.cu),
 *   - h-adaptive cubature engine hcubature_v (src/hcubature.cpp,
 *     src/converged.h): Genz-Malik 7/5 rule for dim>=2, 15-point
 *     Gauss-Kronrod for dim 1, max-heap of regions, Gladwell batch refinement,
 *   - per-term prefactors and n-bar(z) precompute.
 * Parity is pinned against a build of the reference's own CPU path (see
 * oracle/build_ref.sh, oracle/ref_harness.cu) and against committed golden
 * vectors under tests/golden/.
 *
 * Generalisation: the reference uses one Nbins for the z, m and k axes; this
 * restatement takes Nz, Nm, Nk separately (equal values reproduce the
 * reference exactly).  An optional clamp of the P_lin k index at Nk-1 replaces
 * the reference's out-of-bounds read (src/NNMap_Model.cu:826-839).
 */
#ifndef G3L_ORACLE_H
#define G3L_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* HOD parameters in the reference's device order [f, alpha, Mth, sigma, M', beta]
 * (src/HOD.cu:15-20). */
typedef struct {
    double f, alpha, mth, sigma, mprime, beta;
} orc_hod;

/* Flat LCDM parameters used by the model (src/Cosmology.h:18-29). */
typedef struct {
    double Om, OL, Ob, s8, H0, ns;
} orc_cosmo;

/* Tables, binning and HOD state of one model (NNMap_Model / NMapMap_Model). */
typedef struct {
    int Nz, Nm, Nk;
    double zmin, zmax, mmin, mmax, kmin, kmax;
    const double *g, *p1, *p2, *w, *dwdz; /* [Nz] */
    const double *hmf, *b_h, *conc;       /* [Nz*Nm], z-major */
    const double *P_lin;                  /* [Nz*Nk], z-major */
    double *rho_bar, *nbar1, *nbar2;      /* [Nz], filled by orc_model_init */
    orc_hod hod1, hod2;
    int same_pop;   /* 1 if hod1 and hod2 are the same population object */
    double A, eps;  /* satellite-pair correlation parameters */
    orc_cosmo cosmo;
    int clamp_k;    /* 1: clamp P_lin k index at Nk-1 */
    int nthreads;   /* OpenMP threads for integrand evaluation (0 = default) */
    /* satellite-variance rescaling of the reference's SCALING build
     * (src/NNMap_Model.h:59-62): [Nm] per mass bin, or NULL for none */
    const double *scaling1, *scaling2;
} orc_model;

typedef int (*orc_integrand_v)(unsigned ndim, size_t npt, const double *x,
                               void *fdata, unsigned fdim, double *fval);

/* ---- physics primitives (scalar) ---- */
void   orc_sici(double x, double *si, double *ci);
double orc_u_nfw(const orc_model *M, double k, double m, double z, double f);
double orc_aperture(double eta);
double orc_ncen(const orc_hod *h, double m);
double orc_nsat(const orc_hod *h, double m);
double orc_bi_lin(const orc_model *M, double k1, double k2, double cosphi, double z);

/* ---- integrand kernels at one physical point (after the 10^x transform) ----
 * kind: 0 = NNMap, 1 = NMapMap.  term: 1, 2, 3.
 * pt = {l1, l2, phi, m1[, m2[, m3]], z}; type1/type2 select the HOD slots
 * for NNMap (1 or 2); ignored for NMapMap (uses hod1 / nbar1). */
double orc_kernel(const orc_model *M, int kind, int term, const double th[3],
                  const double *pt, int type1, int type2);

/* ---- cubature engine (restated hcubature_v) ---- */
int orc_hcubature_v(unsigned fdim, orc_integrand_v f, void *fdata, unsigned dim,
                    const double *xmin, const double *xmax, size_t maxEval,
                    double reqAbsError, double reqRelError, int norm,
                    double *val, double *err, size_t *numEval);

/* ---- model-level API ---- */
/* rho_bar(z) and nbar1/nbar2(z) for the current HODs (src/NNMap_Model.cu:244-297). */
int  orc_model_init(orc_model *M);
/* Integration bounds of a term (src/NNMap_Model.cu:46-49, 313-314, 338-339, 363-364). */
int  orc_term_bounds(const orc_model *M, int term, double *xmin, double *xmax);
/* Prefactor chain applied to the raw integral, left to right as the reference
 * writes it (src/NNMap_Model.cu:321-322, src/NMapMap_Model.cu:189-191). */
double orc_apply_prefactor(const orc_model *M, int kind, int term, double raw);
/* One term: raw integral val/err, number of evaluations, and the scaled result. */
int  orc_term(const orc_model *M, int kind, int term, const double th[3], int type1,
              int type2, size_t maxEval, double rtol, double *val, double *err,
              size_t *neval, double *result);
/* Vectorised integrand over log-coordinates (the reference's integrand_v callbacks). */
int  orc_integrand_points(const orc_model *M, int kind, int term, const double th[3],
                          int type1, int type2, size_t npt, const double *x, double *fval);
/* Genz-Malik rule of one region: point list, value, error and split dimension. */
int  orc_rule75_region(const orc_model *M, int kind, int term, const double th[3],
                       int type1, int type2, const double *center, const double *halfwidth,
                       double vol, double *val, double *err, int *split);

/* ---- table precomputation (precompute.c; src/doPrecomputations.cpp) ---- */
typedef struct {
    double Om, OL, Ob, s8, H0, ns, rho_crit;
    /* Eisenstein & Hu transfer-function parameters (src/Powerspectrum.h:14-36) */
    double omhh, obhh, theta_cmb, z_equality, k_equality, z_drag, R_drag, R_equality,
        sound_horizon, k_silk, alpha_c, beta_c, alpha_b, beta_b, beta_node;
    double amplitude; /* P(k) normalisation to sigma8 [Mpc^3] */
} orc_pk;

int    orc_pk_init(orc_pk *P, const double cosmo[6]); /* {Om, OL, Ob, sigma8, H0, ns} */
double orc_transfer(const orc_pk *P, double k);
double orc_spectrum(const orc_pk *P, double k, double z);
double orc_sigma2(const orc_pk *P, double m, double z);
double orc_dsigma2dm(const orc_pk *P, double m, double z);
double orc_delta_c(const orc_pk *P, double z);
double orc_mstar(const orc_pk *P, double z);
double orc_concentration(double m, double mstar, double z);
double orc_hmf(const orc_pk *P, double m, double z);
double orc_halo_bias(const orc_pk *P, double m, double z);
double orc_comoving(const orc_pk *P, double z);
double orc_dcomoving(const orc_pk *P, double z);
/* the whole of doPrecomputations.x on N bins; 2-D outputs z-major [N*N] */
int orc_precompute(const double cosmo[6], const double *zs_src, const double *nz_src, int Ns,
                   double zmin, double zmax, double mmin, double mmax, double kmin, double kmax,
                   int N, double *g, double *w, double *dwdz, double *P_lin, double *conc,
                   double *hmf, double *b_h);

#ifdef __cplusplus
}
#endif
#endif
