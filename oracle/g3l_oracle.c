/*
 * g3l_oracle.c -- CPU restatement of the G3LHalo hot path (TEST INFRASTRUCTURE).
 *
 * This file is the oracle used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py.  The product library never links it.
 *
 * Every function follows the reference's IEEE double expression order so
 * that, compiled with -ffp-contract=off against the same libm, it reproduces
 * the reference CPU build bit for bit (pinned by tests/test_oracle_pin.py).
 * Citations are path:line inside the reference project.
 */
#include "g3l_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* constants (src/constants.h:15-21,36-39; src/Cosmology.h:26-28)            */
/* ------------------------------------------------------------------------ */
static const double G3L_PI = 3.14159;          /* truncated pi, src/constants.h:15 */
static const double G3L_C = 2.99792e5;         /* km/s, src/constants.h:39 */
static const double COSMO_MPC_IN_KM = 3.086e19;/* src/Cosmology.h:28 */
static const double COSMO_G = 1.327e11;        /* src/Cosmology.h:27 */
static const double L_MIN = 0.1, L_MAX = 1e6;  /* src/NNMap_Model.h:47-48 */

static double ln10(void) { return log(10.0); } /* src/constants.h:21 */

/* ------------------------------------------------------------------------ */
/* Si / Ci rational approximation (src/generalFunctions.cu:44-87).          */
/* The coefficients are the published Pade approximants of Rowe et al.      */
/* (2015, GalSim, Appendix B); the reference evaluates explicit powers      */
/* left to right, which this restatement keeps for bit parity.              */
/* ------------------------------------------------------------------------ */
static const double SI_NUM[7] = {-4.54393409816329991e-2, 1.15457225751016682e-3,
    -1.41018536821330254e-5, 9.43280809438713025e-8, -3.53201978997168357e-10,
    7.08240282274875911e-13, -6.05338212010422477e-16};
static const double SI_DEN[6] = {1.01162145739225565e-2, 4.99175116169755106e-5,
    1.55654986308745614e-7, 3.28067571055789734e-10, 4.5049097575386581e-13,
    3.21107051193712168e-16};
static const double CI_NUM[6] = {7.51851524438898291e-3, -1.27528342240267686e-4,
    1.05297363846239184e-6, -4.68889508144848019e-9, 1.06480802891189243e-11,
    -9.93728488857585407e-15};
static const double CI_DEN[7] = {1.1592605689110735e-2, 6.72126800814254432e-5,
    2.55533277086129636e-7, 6.97071295760958946e-10, 1.38536352772778619e-12,
    1.89106054713059759e-15, 1.39759616731376855e-18};
static const double FA_NUM[10] = {7.44437068161936700618e2, 1.96396372895146869801e5,
    2.37750310125431834034e7, 1.43073403821274636888e9, 4.33736238870432522765e10,
    6.40533830574022022911e11, 4.20968180571076940208e12, 1.00795182980368574617e13,
    4.94816688199951963482e12, -4.94701168645415959931e11};
static const double FA_DEN[9] = {7.46437068161927678031e2, 1.97865247031583951450e5,
    2.41535670165126845144e7, 1.47478952192985464958e9, 4.58595115847765779830e10,
    7.08501308149515401563e11, 5.06084464593475076774e12, 1.43468549171581016479e13,
    1.11535493509914254097e13};
static const double GA_NUM[10] = {8.1359520115168615e2, 2.35239181626478200e5,
    3.12557570795778731e7, 2.06297595146763354e9, 6.83052205423625007e10,
    1.09049528450362786e12, 7.57664583257834349e12, 1.81004487464664575e13,
    6.43291613143049485e12, -1.36517137670871689e12};
static const double GA_DEN[9] = {8.19595201151451564e2, 2.40036752835578777e5,
    3.26026661647090822e7, 2.23355543278099360e9, 7.87465017341829930e10,
    1.39866710696414565e12, 1.17164723371736605e13, 4.01839087307656620e13,
    3.99653257887490811e13};

void orc_sici(double x, double *si, double *ci)
{
    double p[11]; /* p[i] = x^(2i) built as the reference does */
    p[1] = x * x;
    p[2] = p[1] * p[1];
    p[3] = p[1] * p[2];
    p[4] = p[2] * p[2];
    p[5] = p[4] * p[1];
    p[6] = p[3] * p[3];
    p[7] = p[6] * p[1];
    if (x < 4) {
        double a = 1, b = 1;
        for (int i = 0; i < 7; ++i) a = a + SI_NUM[i] * p[i + 1];
        for (int i = 0; i < 6; ++i) b = b + SI_DEN[i] * p[i + 1];
        *si = x * a / b;
        a = -0.25;
        b = 1;
        for (int i = 0; i < 6; ++i) a = a + CI_NUM[i] * p[i + 1];
        for (int i = 0; i < 7; ++i) b = b + CI_DEN[i] * p[i + 1];
        *ci = 0.5772156649 + log(x) + p[1] * a / b;
    } else {
        p[8] = p[4] * p[4];
        p[9] = p[8] * p[1];
        p[10] = p[5] * p[5];
        double cx = cos(x), sx = sin(x);
        double fn = 1, fd = 1, gn = 1, gd = 1;
        for (int i = 0; i < 10; ++i) fn = fn + FA_NUM[i] / p[i + 1];
        for (int i = 0; i < 9; ++i) fd = fd + FA_DEN[i] / p[i + 1];
        for (int i = 0; i < 10; ++i) gn = gn + GA_NUM[i] / p[i + 1];
        for (int i = 0; i < 9; ++i) gd = gd + GA_DEN[i] / p[i + 1];
        double f = fn / fd / x;
        double g = gn / gd / p[1];
        *si = 0.5 * M_PI - f * cx - g * sx;
        *ci = f * sx - g * cx;
    }
}

/* ------------------------------------------------------------------------ */
/* table indices                                                             */
/* ------------------------------------------------------------------------ */
static inline double z_arg(const orc_model *M, double z)
{
    return (z - M->zmin) * M->Nz / (M->zmax - M->zmin);
}
static inline double m_arg(const orc_model *M, double m)
{
    return log(m / M->mmin) * M->Nm / log(M->mmax / M->mmin);
}
static inline double k_arg(const orc_model *M, double k)
{
    return log(k / M->kmin) * M->Nk / log(M->kmax / M->kmin);
}

/* r_200 (src/generalFunctions.cu:32-37): truncated z index. */
static double r200(const orc_model *M, double m, double z)
{
    int z_ix = (int)z_arg(M, z);
    return pow(0.239 * m / M->rho_bar[z_ix] / 200, 1. / 3.);
}

/* NFW Fourier profile (src/generalFunctions.cu:6-30): truncated indices. */
double orc_u_nfw(const orc_model *M, double k, double m, double z, double f)
{
    int z_ix = (int)z_arg(M, z);
    int m_ix = (int)m_arg(M, m);
    double c = f * M->conc[z_ix * M->Nm + m_ix];
    double arg1 = k * r200(M, m, z) / c;
    double arg2 = arg1 * (1 + c);
    double si1, ci1, si2, ci2;
    orc_sici(arg1, &si1, &ci1);
    orc_sici(arg2, &si2, &ci2);
    double term1 = sin(arg1) * (si2 - si1);
    double term2 = cos(arg1) * (ci2 - ci1);
    double term3 = -sin(arg1 * c) / arg2;
    double F = log(1. + c) - c / (1. + c);
    return (term1 + term2 + term3) / F;
}

/* exponential aperture filter (src/generalFunctions.cu:39-42) */
double orc_aperture(double eta) { return 0.5 * eta * eta * exp(-0.5 * eta * eta); }

/* HOD occupations (src/HOD.cu:35-76) */
double orc_nsat(const orc_hod *h, double m)
{
    return 0.5 * (1 + erf(log(m / h->mth) / h->sigma / 1.414213562)) * pow(m / h->mprime, h->beta);
}
double orc_ncen(const orc_hod *h, double m)
{
    return 0.5 * h->alpha * (1 + erf(log(m / h->mth) / h->sigma / 1.414213562));
}
/* satellite pairs (src/HOD.cu:78-94); same_type mirrors the pointer test.  scale1 is
 * the satellite-variance rescaling (1 without one); the reference never reads scale2. */
static double nsat_nsat(double m, const orc_hod *h1, const orc_hod *h2, int same_type,
                        double A, double eps, double scale1)
{
    double Ns1 = orc_nsat(h1, m);
    if (same_type) return (Ns1 + scale1 * scale1 - 1) * Ns1;
    double Ns2 = orc_nsat(h2, m);
    double result = Ns1 * Ns2 + A * pow(m, eps) * sqrt(Ns1 * Ns2);
    if (result < 0) return 0;
    return result;
}

/* tree-level kernel with the reference's k2/k2 term (src/generalFunctions.cu:89-92) */
static double F2(double k1, double k2, double cosphi)
{
    return 0.7143 + 0.2857 * cosphi * cosphi + 0.5 * cosphi * (k1 / k2 + k2 / k2);
}

/* linear power spectrum lookup with the small-k linear extrapolation
 * (src/NNMap_Model.cu:819-839, src/generalFunctions.cu:112-143) */
static double plin(const orc_model *M, int z_ix, double k)
{
    int k_ix = (int)round(k_arg(M, k));
    if (k_ix >= 0) {
        /* clamp_k: stay in the z row.  Otherwise read the flat array as the
         * reference does, stopping at its last element instead of past it. */
        if (M->clamp_k && k_ix > M->Nk - 1) k_ix = M->Nk - 1;
        long flat = (long)z_ix * M->Nk + k_ix;
        if (flat > (long)M->Nz * M->Nk - 1) flat = (long)M->Nz * M->Nk - 1;
        return M->P_lin[flat];
    }
    return M->P_lin[z_ix * M->Nk] / M->kmin * k;
}

/* tree-level bispectrum (src/generalFunctions.cu:94-147) */
double orc_bi_lin(const orc_model *M, double k1, double k2, double cosphi, double z)
{
    double k3 = sqrt(k1 * k1 + k2 * k2 + 2 * k1 * k2 * cosphi);
    double c_phi12 = cosphi;
    double c_phi13 = (k2 * k2 - k3 * k3 - k1 * k1) / (2 * k1 * k3);
    double c_phi23 = (k1 * k1 - k2 * k2 - k3 * k3) / (2 * k3 * k2);
    int z_ix = (int)round(z_arg(M, z));
    double Pk1 = plin(M, z_ix, k1);
    double Pk2 = plin(M, z_ix, k2);
    double Pk3 = plin(M, z_ix, k3);
    return 2 * (F2(k1, k2, c_phi12) * Pk1 * Pk2 + F2(k1, k3, c_phi13) * Pk1 * Pk3 +
                F2(k2, k3, c_phi23) * Pk2 * Pk3);
}

/* G_g and G_gg (src/NNMap_Model.cu:1071-1108) */
static double G_g(const orc_model *M, double k, double m, double z, const orc_hod *h)
{
    double Nc = orc_ncen(h, m);
    double Ns = orc_nsat(h, m);
    return Nc + Ns * orc_u_nfw(M, k, m, z, h->f);
}
static double G_gg(const orc_model *M, double k1, double k2, double m, double z,
                   const orc_hod *h1, const orc_hod *h2, int same_type, double scale1)
{
    double Nc1 = orc_ncen(h1, m);
    double Nc2 = orc_ncen(h2, m);
    double Ns1 = orc_nsat(h1, m);
    double Ns2 = orc_nsat(h2, m);
    double Nss = nsat_nsat(m, h1, h2, same_type, M->A, M->eps, scale1);
    double f1 = h1->f, f2 = h2->f;
    return Nc1 * Ns2 * orc_u_nfw(M, k2, m, z, f2) + Nc2 * Ns1 * orc_u_nfw(M, k1, m, z, f1) +
           Nss * orc_u_nfw(M, k1, m, z, f1) * orc_u_nfw(M, k2, m, z, f2);
}

/* ------------------------------------------------------------------------ */
/* integrand kernels                                                          */
/* ------------------------------------------------------------------------ */
static double nnm_1h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m, double z, const orc_hod *h1, const orc_hod *h2,
                     const double *n_bar1, const double *n_bar2, int same_type)
{   /* src/NNMap_Model.cu:544-593 */
    int z_ix = (int)round(z_arg(M, z));
    int m_ix = (int)round(m_arg(M, m));
    /* SCALING build: scale1 = scaling1[m_ix] (src/NNMap_Model.cu:563) */
    double scale1 = M->scaling1 ? M->scaling1[m_ix] : 1;
    double nbar1 = n_bar1[z_ix];
    double nbar2 = n_bar2[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    double Bggd = 1. / nbar1 / nbar2 / M->rho_bar[z_ix] * M->hmf[z_ix * M->Nm + m_ix] * m *
                  orc_u_nfw(M, k3, m, z, 1);
    Bggd *= G_gg(M, k1, k2, m, z, h1, h2, same_type, scale1);
    double bggk = Bggd / M->dwdz[z_ix] * M->g[z_ix] * M->p1[z_ix] * M->p2[z_ix] / w_ / w_ / w_ *
                  (1. + z);
    return l1 * l2 * m * l1 * l2 * orc_aperture(th[0] * l1) * orc_aperture(th[1] * l2) *
           orc_aperture(th[2] * l3) * bggk;
}

static double nnm_2h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m1, double m2, double z, const orc_hod *h1, const orc_hod *h2,
                     const double *n_bar1, const double *n_bar2, int same_type)
{   /* src/NNMap_Model.cu:787-856 */
    int z_ix = (int)round(z_arg(M, z));
    int m1_ix = (int)round(m_arg(M, m1));
    int m2_ix = (int)round(m_arg(M, m2));
    /* SCALING build: scale1 = scaling1[m2_ix] (src/NNMap_Model.cu:808) */
    double scale1 = M->scaling1 ? M->scaling1[m2_ix] : 1;
    double nbar1 = n_bar1[z_ix];
    double nbar2 = n_bar2[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    double Pk1 = plin(M, z_ix, k1);
    double Pk2 = plin(M, z_ix, k2);
    double Pk3 = plin(M, z_ix, k3);
    const int Nm = M->Nm;
    double Bggd = 1. / nbar1 / nbar2 / M->rho_bar[z_ix] * M->hmf[z_ix * Nm + m1_ix] *
                  M->hmf[z_ix * Nm + m2_ix] * M->b_h[z_ix * Nm + m1_ix] * M->b_h[z_ix * Nm + m2_ix] *
                  (m1 * orc_u_nfw(M, k3, m1, z, 1) * G_gg(M, k1, k2, m2, z, h1, h2, same_type, scale1) * Pk3 +
                   m2 * orc_u_nfw(M, k3, m2, z, 1) * G_g(M, k1, m1, z, h1) * G_g(M, k2, m2, z, h2) * Pk1 +
                   m2 * orc_u_nfw(M, k3, m2, z, 1) * G_g(M, k2, m1, z, h2) * G_g(M, k1, m2, z, h1) * Pk2);
    double bggk = 1. / M->dwdz[z_ix] * M->g[z_ix] * M->p1[z_ix] * M->p2[z_ix] / w_ / w_ / w_ *
                  (1. + z) * Bggd;
    return l1 * l2 * m1 * m2 * l1 * l2 * orc_aperture(th[0] * l1) * orc_aperture(th[1] * l2) *
           orc_aperture(th[2] * l3) * bggk;
}

static double nnm_3h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m1, double m2, double m3, double z, const orc_hod *h1,
                     const orc_hod *h2, const double *n_bar1, const double *n_bar2)
{   /* src/NNMap_Model.cu:1003-1037 */
    int z_ix = (int)round(z_arg(M, z));
    int m1_ix = (int)round(m_arg(M, m1));
    int m2_ix = (int)round(m_arg(M, m2));
    int m3_ix = (int)round(m_arg(M, m3));
    double nbar1 = n_bar1[z_ix];
    double nbar2 = n_bar2[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    const int Nm = M->Nm;
    double Bggd = 1. / nbar1 / nbar2 / M->rho_bar[z_ix] * M->hmf[z_ix * Nm + m1_ix] *
                  M->hmf[z_ix * Nm + m2_ix] * M->hmf[z_ix * Nm + m3_ix] * m3 *
                  orc_u_nfw(M, k3, m3, z, 1) * G_g(M, k1, m1, z, h1) * G_g(M, k2, m2, z, h2) *
                  orc_bi_lin(M, k1, k2, cos(phi), z) * M->b_h[z_ix * Nm + m1_ix] *
                  M->b_h[z_ix * Nm + m2_ix] * M->b_h[z_ix * Nm + m3_ix];
    double bggk = Bggd / M->dwdz[z_ix] * M->g[z_ix] * M->p1[z_ix] * M->p2[z_ix] / w_ / w_ / w_ *
                  (1. + z);
    return l1 * l2 * m1 * m2 * m3 * l1 * l2 * orc_aperture(th[0] * l1) * orc_aperture(th[1] * l2) *
           orc_aperture(th[2] * l3) * bggk;
}

static double nmm_1h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m, double z)
{   /* src/NMapMap_Model.cu:263-301 */
    const orc_hod *h = &M->hod1;
    int z_ix = (int)round(z_arg(M, z));
    int m_ix = (int)round(m_arg(M, m));
    double nbar = M->nbar1[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    double Nc = orc_ncen(h, m);
    double Ns = orc_nsat(h, m);
    double f = h->f;
    double rho = M->rho_bar[z_ix];
    double Bgdd = 1. / nbar / rho / rho * M->hmf[z_ix * M->Nm + m_ix] * m * m *
                  (Nc + Ns * orc_u_nfw(M, k1, m, z, f)) * orc_u_nfw(M, k2, m, z, 1) *
                  orc_u_nfw(M, k3, m, z, 1);
    double bgkk = Bgdd / M->dwdz[z_ix] * M->g[z_ix] * M->g[z_ix] * M->p1[z_ix] / w_ / w_ *
                  (1. + z) * (1. + z);
    return l1 * l2 * m * l1 * l2 * orc_aperture(th[0] * l1) * orc_aperture(th[1] * l2) *
           orc_aperture(th[2] * l3) * bgkk / nbar;
}

static double nmm_2h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m1, double m2, double z)
{   /* src/NMapMap_Model.cu:402-468 */
    const orc_hod *h = &M->hod1;
    int z_ix = (int)round(z_arg(M, z));
    int m1_ix = (int)round(m_arg(M, m1));
    int m2_ix = (int)round(m_arg(M, m2));
    double nbar = M->nbar1[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    double Pk1 = plin(M, z_ix, k1);
    double Pk2 = plin(M, z_ix, k2);
    double Pk3 = plin(M, z_ix, k3);
    double Nc1 = orc_ncen(h, m1);
    double Ns1 = orc_nsat(h, m1);
    double Nc2 = orc_ncen(h, m2);
    double Ns2 = orc_nsat(h, m2);
    double f = h->f;
    double rho = M->rho_bar[z_ix];
    const int Nm = M->Nm;
    double Bgdd = 1. / nbar / rho / rho * M->hmf[z_ix * Nm + m1_ix] * M->hmf[z_ix * Nm + m2_ix] *
                  M->b_h[z_ix * Nm + m1_ix] * M->b_h[z_ix * Nm + m2_ix] *
                  (m1 * m2 * orc_u_nfw(M, k2, m1, z, 1) * orc_u_nfw(M, k3, m2, z, 1) *
                       (Nc2 + Ns2 * orc_u_nfw(M, k1, m2, z, f)) * Pk2 +
                   m1 * m2 * orc_u_nfw(M, k3, m1, z, 1) * orc_u_nfw(M, k2, m2, z, 1) *
                       (Nc2 + Ns2 * orc_u_nfw(M, k1, m2, z, f)) * Pk3 +
                   m2 * m2 * orc_u_nfw(M, k2, m1, z, 1) * orc_u_nfw(M, k3, m2, z, 1) *
                       (Nc1 + Ns1 * orc_u_nfw(M, k1, m1, z, f)) * Pk1);
    double bgkk = Bgdd / M->dwdz[z_ix] * M->g[z_ix] * M->g[z_ix] * M->p1[z_ix] / w_ / w_ *
                  (1. + z) * (1. + z);
    return l1 * l2 * m1 * m2 * l1 * l2 * orc_aperture(th[0] * l1) * orc_aperture(th[1] * l2) *
           orc_aperture(th[2] * l3) * bgkk / nbar;
}

static double nmm_3h(const orc_model *M, const double th[3], double l1, double l2, double phi,
                     double m1, double m2, double m3, double z)
{   /* src/NMapMap_Model.cu:592-632 (Nc/Ns at m3 but u_NFW(k1, m2, f) as in the reference) */
    const orc_hod *h = &M->hod1;
    int z_ix = (int)round(z_arg(M, z));
    int m1_ix = (int)round(m_arg(M, m1));
    int m2_ix = (int)round(m_arg(M, m2));
    int m3_ix = (int)round(m_arg(M, m3));
    double nbar = M->nbar1[z_ix];
    double w_ = M->w[z_ix];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    double k1 = l1 / w_;
    double k2 = l2 / w_;
    double k3 = l3 / w_;
    double Nc = orc_ncen(h, m3);
    double Ns = orc_nsat(h, m3);
    double f = h->f;
    double rho = M->rho_bar[z_ix];
    const int Nm = M->Nm;
    double Bgdd = 1. / nbar / rho / rho * M->hmf[z_ix * Nm + m1_ix] * M->hmf[z_ix * Nm + m2_ix] *
                  M->hmf[z_ix * Nm + m3_ix] * M->b_h[z_ix * Nm + m1_ix] *
                  M->b_h[z_ix * Nm + m2_ix] * M->b_h[z_ix * Nm + m3_ix] * m1 * m2 *
                  orc_u_nfw(M, k2, m1, z, 1) * orc_u_nfw(M, k3, m2, z, 1) *
                  (Nc + Ns * orc_u_nfw(M, k1, m2, z, f)) * orc_bi_lin(M, k1, k2, cos(phi), z);
    double bgkk = Bgdd / M->dwdz[z_ix] * M->g[z_ix] * M->g[z_ix] * M->p1[z_ix] / w_ / w_ *
                  (1. + z) * (1. + z);
    return l1 * l2 * m1 * m2 * m3 * l1 * l2 * orc_aperture(th[0] * l1) *
           orc_aperture(th[1] * l2) * orc_aperture(th[2] * l3) * bgkk / nbar;
}

/* HOD / nbar choice per type (src/NNMap_Model.cu:437-475) */
static void pick_types(const orc_model *M, int type1, int type2, const orc_hod **h1,
                       const orc_hod **h2, const double **nb1, const double **nb2, int *same)
{
    *h1 = (type1 == 1) ? &M->hod1 : &M->hod2;
    *nb1 = (type1 == 1) ? M->nbar1 : M->nbar2;
    *h2 = (type2 == 1) ? &M->hod1 : &M->hod2;
    *nb2 = (type2 == 1) ? M->nbar1 : M->nbar2;
    *same = (type1 == type2) || M->same_pop;
}

double orc_kernel(const orc_model *M, int kind, int term, const double th[3], const double *pt,
                  int type1, int type2)
{
    if (kind == 0) {
        const orc_hod *h1, *h2;
        const double *nb1, *nb2;
        int same;
        pick_types(M, type1, type2, &h1, &h2, &nb1, &nb2, &same);
        if (term == 1) return nnm_1h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4], h1, h2, nb1, nb2, same);
        if (term == 2)
            return nnm_2h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], h1, h2, nb1, nb2, same);
        return nnm_3h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], pt[6], h1, h2, nb1, nb2);
    }
    if (term == 1) return nmm_1h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4]);
    if (term == 2) return nmm_2h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4], pt[5]);
    return nmm_3h(M, th, pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], pt[6]);
}

/* ------------------------------------------------------------------------ */
/* vectorised integrands over log coordinates (src/NNMap_Model.cu:519-538)   */
/* ------------------------------------------------------------------------ */
typedef struct {
    const orc_model *M;
    int kind, term, type1, type2;
    double th[3];
} term_ctx;

static int term_integrand(unsigned ndim, size_t npt, const double *x, void *fdata,
                          unsigned fdim, double *fval)
{
    const term_ctx *T = (const term_ctx *)fdata;
    if (fdim != 1) return 1;
    const long n = (long)npt;
    const int nth = T->M->nthreads;
#pragma omp parallel for schedule(static) num_threads(nth > 0 ? nth : omp_get_max_threads())
    for (long i = 0; i < n; ++i) {
        const double *xi = x + (size_t)i * ndim;
        double pt[7];
        pt[0] = pow(10, xi[0]);
        pt[1] = pow(10, xi[1]);
        pt[2] = xi[2];
        for (unsigned d = 3; d + 1 < ndim; ++d) pt[d] = pow(10, xi[d]);
        pt[ndim - 1] = xi[ndim - 1];
        fval[i] = orc_kernel(T->M, T->kind, T->term, T->th, pt, T->type1, T->type2);
    }
    return 0;
}

int orc_integrand_points(const orc_model *M, int kind, int term, const double th[3], int type1,
                         int type2, size_t npt, const double *x, double *fval)
{
    term_ctx T = {M, kind, term, type1, type2, {th[0], th[1], th[2]}};
    return term_integrand((unsigned)(term + 4), npt, x, &T, 1, fval);
}

/* n-bar integrand (src/generalFunctions.cu:149-211, 233-245) */
typedef struct {
    const orc_model *M;
    const orc_hod *h;
    double z;
} nbar_ctx;

static int nbar_integrand(unsigned ndim, size_t npt, const double *x, void *fdata, unsigned fdim,
                          double *fval)
{
    const nbar_ctx *C = (const nbar_ctx *)fdata;
    const orc_model *M = C->M;
    if (fdim != 1) return 1;
    for (size_t i = 0; i < npt; ++i) {
        double m = pow(10, x[i * ndim]);
        double Nc = orc_ncen(C->h, m);
        double Ns = orc_nsat(C->h, m);
        int m_ix = (int)round(m_arg(M, m));
        int z_ix = (int)round(z_arg(M, C->z));
        fval[i] = m * M->hmf[(int)(z_ix * M->Nm + m_ix)] * (Nc + Ns);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* cubature engine (restatement of src/hcubature.cpp:115-1067)               */
/* ------------------------------------------------------------------------ */
typedef struct {
    double *c;     /* center[dim] followed by halfwidth[dim] */
    double vol;
    double val, err;
    unsigned split;
} orc_region;

static double region_volume(const double *hw, unsigned dim)
{   /* compute_vol, src/hcubature.cpp:134-141 */
    double vol = 1;
    for (unsigned i = 0; i < dim; ++i) vol *= 2 * hw[i];
    return vol;
}

/* Genz-Malik degree 7/5 constants (Genz & Malik 1983; src/hcubature.cpp:458-466, 600-606) */
static const double GM_L2 = 0.3585685828003180919906451539079374954541;
static const double GM_L4 = 0.9486832980505137995996680633298155601160;
static const double GM_L5 = 0.6882472016116852977216287342936235251269;

typedef struct {
    unsigned dim, npts;
    double w1, w3, w5, wE1, wE3;
} gm_rule;

static gm_rule gm_make(unsigned dim)
{
    gm_rule r;
    int d = (int)dim;
    r.dim = dim;
    r.npts = 1 + 2 * 2 * dim + 2 * dim * (dim - 1) + (1u << dim);
    r.w1 = (double)(12824 - 9120 * d + 400 * d * d) / (double)19683;
    r.w3 = (double)(1820 - 400 * d) / (double)19683;
    r.w5 = (double)6859 / (double)19683 / (double)(1u << dim);
    r.wE1 = (double)(729 - 950 * d + 50 * d * d) / (double)729;
    r.wE3 = (double)(265 - 100 * d) / (double)1458;
    return r;
}

/* Point set of one region in the reference's order (src/hcubature.cpp:343-414, 476-503). */
static void gm_points(const gm_rule *r, const double *c, const double *hw, double *pts)
{
    const unsigned dim = r->dim;
    double r2[32], r4[32], r5[32], p[32];
    for (unsigned i = 0; i < dim; ++i) {
        p[i] = c[i];
        r2[i] = hw[i] * GM_L2;
        r4[i] = hw[i] * GM_L4;
        r5[i] = hw[i] * GM_L5;
    }
    double *o = pts;
    /* center and the +-lambda2 / +-lambda4 axis points */
    memcpy(o, p, sizeof(double) * dim); o += dim;
    for (unsigned i = 0; i < dim; ++i) {
        p[i] = c[i] - r2[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
        p[i] = c[i] + r2[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
        p[i] = c[i] - r4[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
        p[i] = c[i] + r4[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
        p[i] = c[i];
    }
    /* (+-lambda4, +-lambda4) pairs */
    for (unsigned i = 0; i + 1 < dim; ++i) {
        p[i] = c[i] - r4[i];
        for (unsigned j = i + 1; j < dim; ++j) {
            p[j] = c[j] - r4[j]; memcpy(o, p, sizeof(double) * dim); o += dim;
            p[i] = c[i] + r4[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
            p[j] = c[j] + r4[j]; memcpy(o, p, sizeof(double) * dim); o += dim;
            p[i] = c[i] - r4[i]; memcpy(o, p, sizeof(double) * dim); o += dim;
            p[j] = c[j];
        }
        p[i] = c[i];
    }
    /* (+-lambda5)^dim corners in reflected-Gray-code order */
    for (unsigned n = 0; n < (1u << dim); ++n) {
        unsigned gray = n ^ (n >> 1);
        for (unsigned d = 0; d < dim; ++d)
            o[d] = (gray >> d & 1u) ? c[d] - r5[d] : c[d] + r5[d];
        o += dim;
    }
}

/* Rule sums of one region from its point values (src/hcubature.cpp:512-576). */
static void gm_combine(const gm_rule *r, const double *v, double vol, double *val, double *err,
                       unsigned *split)
{
    const unsigned dim = r->dim;
    const double w2 = 980. / 6561., w4 = 200. / 19683.;
    const double wE2 = 245. / 486., wE4 = 25. / 729.;
    const double ratio = (GM_L2 * GM_L2) / (GM_L4 * GM_L4);
    double val0 = v[0], sum2 = 0, sum3 = 0, sum4 = 0, sum5 = 0;
    double diff[32];
    unsigned k, k0 = 1;
    for (k = 0; k < dim; ++k) {
        double v0 = v[k0 + 4 * k], v1 = v[k0 + 4 * k + 1];
        double v2 = v[k0 + 4 * k + 2], v3 = v[k0 + 4 * k + 3];
        sum2 += v0 + v1;
        sum3 += v2 + v3;
        diff[k] = 0;
        diff[k] += fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
    }
    k0 += 4 * dim;
    const unsigned nrr = 2 * dim * (dim - 1);
    for (k = 0; k < nrr; ++k) sum4 += v[k0 + k];
    k0 += nrr;
    for (k = 0; k < (1u << dim); ++k) sum5 += v[k0 + k];
    double result = vol * (r->w1 * val0 + w2 * sum2 + r->w3 * sum3 + w4 * sum4 + r->w5 * sum5);
    double res5th = vol * (r->wE1 * val0 + wE2 * sum2 + r->wE3 * sum3 + wE4 * sum4);
    *val = result;
    *err = fabs(res5th - result);
    double maxdiff = 0;
    unsigned dimDiffMax = 0;
    for (unsigned i = 0; i < dim; ++i)
        if (diff[i] > maxdiff) {
            maxdiff = diff[i];
            dimDiffMax = i;
        }
    *split = dimDiffMax;
}

/* 15-point Gauss-Kronrod (QUADPACK qk15 nodes/weights; src/hcubature.cpp:620-757) */
static const double GK_XGK[8] = {0.991455371120812639206854697526329,
    0.949107912342758524526189684047851, 0.864864423359769072789712788640926,
    0.741531185599394439863864773280788, 0.586087235467691130294144838258730,
    0.405845151377397166906606412076961, 0.207784955007898467600689403773245, 0.0};
static const double GK_WG[4] = {0.129484966168869693270611432679082,
    0.279705391489276667901467771423780, 0.381830050505118944950369775488975,
    0.417959183673469387755102040816327};
static const double GK_WGK[8] = {0.022935322010529224963732008058970,
    0.063092092629978553290700663189204, 0.104790010322250183839876322541518,
    0.140653259715525918745189590510238, 0.169004726639267902826583426598550,
    0.190350578064785409913256402421014, 0.204432940075298892414161999234649,
    0.209482141084727828012999174891714};

static void gk_points(double c, double hw, double *pts)
{
    int n = 0;
    pts[n++] = c;
    for (int j = 0; j < 3; ++j) {
        double w = hw * GK_XGK[2 * j + 1];
        pts[n++] = c - w;
        pts[n++] = c + w;
    }
    for (int j = 0; j < 4; ++j) {
        double w = hw * GK_XGK[2 * j];
        pts[n++] = c - w;
        pts[n++] = c + w;
    }
}

static void gk_combine(const double *vk, double hw, double *val, double *err)
{
    double result_gauss = vk[0] * GK_WG[3];
    double result_kronrod = vk[0] * GK_WGK[7];
    double result_abs = fabs(result_kronrod);
    double result_asc, mean, e;
    int n = 1;
    for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        double v = vk[n] + vk[n + 1];
        result_gauss += GK_WG[j] * v;
        result_kronrod += GK_WGK[j2] * v;
        result_abs += GK_WGK[j2] * (fabs(vk[n]) + fabs(vk[n + 1]));
        n += 2;
    }
    for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        result_kronrod += GK_WGK[j2] * (vk[n] + vk[n + 1]);
        result_abs += GK_WGK[j2] * (fabs(vk[n]) + fabs(vk[n + 1]));
        n += 2;
    }
    *val = result_kronrod * hw;
    mean = result_kronrod * 0.5;
    result_asc = GK_WGK[7] * fabs(vk[0] - mean);
    n = 1;
    for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        result_asc += GK_WGK[j2] * (fabs(vk[n] - mean) + fabs(vk[n + 1] - mean));
        n += 2;
    }
    for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        result_asc += GK_WGK[j2] * (fabs(vk[n] - mean) + fabs(vk[n + 1] - mean));
        n += 2;
    }
    e = fabs(result_kronrod - result_gauss) * hw;
    result_abs *= hw;
    result_asc *= hw;
    if (result_asc != 0 && e != 0) {
        double scale = pow((200 * e / result_asc), 1.5);
        e = (scale < 1) ? result_asc * scale : result_asc;
    }
    if (result_abs > DBL_MIN / (50 * DBL_EPSILON)) {
        double min_err = 50 * DBL_EPSILON * result_abs;
        if (min_err > e) e = min_err;
    }
    *err = e;
}

/* binary max-heap keyed on err with running totals (src/hcubature.cpp:772-890) */
typedef struct {
    size_t n, nalloc;
    orc_region *items;
    double val, err;
} orc_heap;

static int heap_push(orc_heap *h, orc_region r)
{
    h->val += r.val;
    h->err += r.err;
    size_t ins = h->n;
    if (++h->n > h->nalloc) {
        size_t na = h->n * 2;
        orc_region *ni = (orc_region *)realloc(h->items, sizeof(orc_region) * na);
        if (!ni) return 1;
        h->items = ni;
        h->nalloc = na;
    }
    while (ins) {
        size_t parent = (ins - 1) / 2;
        if (r.err <= h->items[parent].err) break;
        h->items[ins] = h->items[parent];
        ins = parent;
    }
    h->items[ins] = r;
    return 0;
}

static orc_region heap_pop(orc_heap *h)
{
    orc_region ret = h->items[0];
    size_t i = 0, n = --h->n, child;
    h->items[0] = h->items[n];
    while ((child = i * 2 + 1) < n) {
        size_t largest = (h->items[child].err <= h->items[i].err) ? i : child;
        if (++child < n && h->items[largest].err < h->items[child].err) largest = child;
        if (largest == i) break;
        orc_region sw = h->items[i];
        h->items[i] = h->items[largest];
        h->items[largest] = sw;
        i = largest;
    }
    h->val -= ret.val;
    h->err -= ret.err;
    return ret;
}

/* converged() for one integrand (src/converged.h:10-14) */
static int converged1(double err, double val, double reqAbs, double reqRel)
{
    return !(err > reqAbs && err > fabs(val) * reqRel);
}

/* evaluate a batch of regions with one integrand call (src/hcubature.cpp:285-294) */
static int eval_batch(unsigned dim, const gm_rule *gm, orc_integrand_v f, void *fdata,
                      size_t nR, orc_region *R, double **pts_buf, size_t *pts_cap)
{
    const unsigned npts = (dim == 1) ? 15u : gm->npts;
    size_t need = nR * npts * (dim + 1);
    if (need > *pts_cap) {
        free(*pts_buf);
        *pts_cap = need * 2;
        *pts_buf = (double *)malloc(sizeof(double) * *pts_cap);
        if (!*pts_buf) return 1;
    }
    double *pts = *pts_buf, *vals = pts + nR * npts * dim;
    for (size_t i = 0; i < nR; ++i) {
        if (dim == 1) gk_points(R[i].c[0], R[i].c[1], pts + i * npts);
        else gm_points(gm, R[i].c, R[i].c + dim, pts + i * npts * dim);
    }
    if (f(dim, nR * npts, pts, fdata, 1, vals)) return 1;
    for (size_t i = 0; i < nR; ++i) {
        if (dim == 1) {
            gk_combine(vals + i * npts, R[i].c[1], &R[i].val, &R[i].err);
            R[i].split = 0;
        } else {
            gm_combine(gm, vals + i * npts, R[i].vol, &R[i].val, &R[i].err, &R[i].split);
        }
    }
    return 0;
}

int orc_hcubature_v(unsigned fdim, orc_integrand_v f, void *fdata, unsigned dim,
                    const double *xmin, const double *xmax, size_t maxEval, double reqAbsError,
                    double reqRelError, int norm, double *val, double *err, size_t *numEvalOut)
{
    (void)norm; /* fdim == 1: every norm reduces to the individual criterion */
    if (fdim != 1 || dim == 0 || dim > 20) return 1;
    gm_rule gm = gm_make(dim < 2 ? 2 : dim);
    const unsigned npts = (dim == 1) ? 15u : gm.npts;
    orc_heap H = {0, 0, NULL, 0, 0};
    size_t numEval = 0, nR_alloc = 2, pts_cap = 0;
    double *pts_buf = NULL;
    orc_region *R = (orc_region *)malloc(sizeof(orc_region) * nR_alloc);
    int status = 1;
    if (!R) goto done;
    /* root region (src/hcubature.cpp:160-172, 928-936) */
    R[0].c = (double *)malloc(sizeof(double) * 2 * dim);
    for (unsigned i = 0; i < dim; ++i) {
        R[0].c[i] = 0.5 * (xmin[i] + xmax[i]);
        R[0].c[i + dim] = 0.5 * (xmax[i] - xmin[i]);
    }
    R[0].vol = region_volume(R[0].c + dim, dim);
    if (eval_batch(dim, &gm, f, fdata, 1, R, &pts_buf, &pts_cap)) goto done;
    if (heap_push(&H, R[0])) goto done;
    numEval += npts;
    /* Gladwell batch refinement (src/hcubature.cpp:938-989) */
    while (numEval < maxEval || !maxEval) {
        if (converged1(H.err, H.val, reqAbsError, reqRelError)) break;
        size_t nR = 0;
        double ee_err = H.err, ee_val = H.val;
        do {
            if (nR + 2 > nR_alloc) {
                nR_alloc = (nR + 2) * 2;
                orc_region *nr = (orc_region *)realloc(R, nR_alloc * sizeof(orc_region));
                if (!nr) goto done;
                R = nr;
            }
            R[nR] = heap_pop(&H);
            ee_err -= R[nR].err;
            /* cut_region (src/hcubature.cpp:206-218) */
            {
                orc_region *L = &R[nR], *Rt = &R[nR + 1];
                unsigned d = L->split;
                *Rt = *L;
                L->c[d + dim] *= 0.5;
                L->vol *= 0.5;
                Rt->c = (double *)malloc(sizeof(double) * 2 * dim);
                memcpy(Rt->c, L->c, sizeof(double) * 2 * dim);
                Rt->vol = region_volume(Rt->c + dim, dim);
                L->c[d] -= L->c[d + dim];
                Rt->c[d] += L->c[d + dim];
            }
            numEval += (size_t)npts * 2;
            nR += 2;
            if (converged1(ee_err, ee_val, reqAbsError, reqRelError)) break;
        } while (H.n > 0 && (numEval < maxEval || !maxEval));
        if (eval_batch(dim, &gm, f, fdata, nR, R, &pts_buf, &pts_cap)) goto done;
        for (size_t i = 0; i < nR; ++i)
            if (heap_push(&H, R[i])) goto done;
    }
    /* re-sum in heap order (src/hcubature.cpp:1000-1008) */
    *val = 0;
    *err = 0;
    for (size_t i = 0; i < H.n; ++i) {
        *val += H.items[i].val;
        *err += H.items[i].err;
    }
    status = 0;
done:
    for (size_t i = 0; i < H.n; ++i) free(H.items[i].c);
    free(H.items);
    free(R);
    free(pts_buf);
    if (numEvalOut) *numEvalOut = numEval;
    return status;
}

/* ------------------------------------------------------------------------ */
/* model-level API                                                            */
/* ------------------------------------------------------------------------ */
static double mmax_integral(const orc_model *M)
{
    return exp(log(M->mmin) + log(M->mmax / M->mmin) * (M->Nm - 1) / M->Nm);
}

int orc_model_init(orc_model *M)
{   /* updateDensities (src/NNMap_Model.cu:244-297; src/Cosmology.cpp:71-87) */
    const orc_cosmo *C = &M->cosmo;
    /* one population object in both slots (src/HOD.cu:82 compares pointers) */
    if (M->same_pop) M->hod2 = M->hod1;
    double rho_crit = 3 * C->H0 * C->H0 * COSMO_MPC_IN_KM / 8 / G3L_PI / COSMO_G;
    double m_min[1] = {log10(M->mmin)};
    double m_max[1] = {log10(mmax_integral(M))};
    for (int i = 0; i < M->Nz; ++i) {
        double z = M->zmin + i * (M->zmax - M->zmin) / M->Nz;
        double E = C->Om * (1 + z) * (1 + z) * (1 + z) + C->OL;
        double Om_z = C->Om * (1 + z) * (1 + z) * (1 + z) / E;
        M->rho_bar[i] = Om_z * rho_crit;
        double result, error;
        nbar_ctx nc = {M, &M->hod1, z};
        if (orc_hcubature_v(1, nbar_integrand, &nc, 1, m_min, m_max, 0, 0, 1e-4, 3, &result, &error,
                            NULL))
            return 1;
        M->nbar1[i] = ln10() * result;
        nc.h = &M->hod2;
        if (orc_hcubature_v(1, nbar_integrand, &nc, 1, m_min, m_max, 0, 0, 1e-4, 3, &result, &error,
                            NULL))
            return 1;
        M->nbar2[i] = ln10() * result;
    }
    return 0;
}

int orc_term_bounds(const orc_model *M, int term, double *xmin, double *xmax)
{
    const double zmax_int = M->zmax - (M->zmax - M->zmin) / M->Nz;
    const double lm0 = log10(M->mmin), lm1 = log10(mmax_integral(M));
    int dim = term + 4, d = 0;
    xmin[d] = log10(L_MIN); xmax[d++] = log10(L_MAX);
    xmin[d] = log10(L_MIN); xmax[d++] = log10(L_MAX);
    xmin[d] = 0; xmax[d++] = 2 * G3L_PI;
    for (int j = 0; j < term; ++j) { xmin[d] = lm0; xmax[d++] = lm1; }
    xmin[d] = M->zmin; xmax[d++] = zmax_int;
    return dim;
}

/* prefactor chain, left to right as in src/NNMap_Model.cu:321-322,346-347,371-372 and
 * src/NMapMap_Model.cu:189-191,214,237 */
double orc_apply_prefactor(const orc_model *M, int kind, int term, double result)
{
    const double H0 = M->cosmo.H0, Om = M->cosmo.Om, l10 = ln10();
    double r;
    if (kind == 0) r = result * 3 * H0 * H0 * Om / 2 / G3L_C / G3L_C;
    else r = result * 9 * pow(H0, 4) * pow(Om, 2) / 4 / pow(G3L_C, 4);
    for (int i = 0; i < term + 2; ++i) r = r * l10;
    r = r / (2 * G3L_PI) / (2 * G3L_PI) / (2 * G3L_PI);
    return r;
}

int orc_term(const orc_model *M, int kind, int term, const double th[3], int type1, int type2,
             size_t maxEval, double rtol, double *val, double *err, size_t *neval, double *result)
{
    double xmin[7], xmax[7];
    int dim = orc_term_bounds(M, term, xmin, xmax);
    term_ctx T = {M, kind, term, type1, type2, {th[0], th[1], th[2]}};
    int st = orc_hcubature_v(1, term_integrand, &T, (unsigned)dim, xmin, xmax, maxEval, 0, rtol, 3,
                             val, err, neval);
    if (result) *result = orc_apply_prefactor(M, kind, term, *val);
    return st;
}

int orc_rule75_region(const orc_model *M, int kind, int term, const double th[3], int type1,
                      int type2, const double *center, const double *halfwidth, double vol,
                      double *val, double *err, int *split)
{
    const unsigned dim = (unsigned)(term + 4);
    gm_rule gm = gm_make(dim);
    double *pts = (double *)malloc(sizeof(double) * gm.npts * (dim + 1));
    if (!pts) return 1;
    double *vals = pts + gm.npts * dim;
    gm_points(&gm, center, halfwidth, pts);
    term_ctx T = {M, kind, term, type1, type2, {th[0], th[1], th[2]}};
    int st = term_integrand(dim, gm.npts, pts, &T, 1, vals);
    unsigned s = 0;
    if (!st) gm_combine(&gm, vals, vol, val, err, &s);
    *split = (int)s;
    free(pts);
    return st;
}
