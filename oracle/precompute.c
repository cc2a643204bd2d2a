/* precompute.c -- CPU restatement of the reference's table precomputation
 * (TEST INFRASTRUCTURE ONLY: the oracle of the device precompute, never shipped).
 *
 * Follows doPrecomputations.x (src/doPrecomputations.cpp:40-134): the lensing
 * efficiency, comoving distance and its derivative on the z grid
 * (src/Cosmology.cpp:74-193), the Eisenstein & Hu transfer function and the linear
 * power spectrum normalised to sigma8 (src/Powerspectrum.cpp:9-196), sigma^2(m, z)
 * and dsigma^2/dm (:198-293), the concentration through M*(z) (:117-150, 296-313),
 * and the Sheth-Tormen mass function and halo bias (src/HMF.cpp:7-84).  The same
 * IEEE operations in the same order (compiled with -ffp-contract=off), and the
 * reference's adaptive 1-D integrals through orc_hcubature_v, which restates its
 * hcubature_v.  Every (z, m) integral is independent; OpenMP spreads them.
 *
 * One deviation: dsigma2dm never sets the redshift of its integrand container
 * (src/Powerspectrum.cpp:249-258; the integrand reads container->z at :281), so the
 * reference evaluates P(k, z) at an unspecified z there.  This restatement uses the
 * z of the call; the pin against the reference build shows which z that build used.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "g3l_oracle.h"

/* the reference's constants (src/constants.h:15,39; src/Cosmology.h:27-28) */
static const double kPiTrunc = 3.14159;
static const double kC = 2.99792e5;
static const double kG = 1.327e11;
static const double kMpcInKm = 3.086e19;
static const double kPi = 3.14159265358979323846; /* std::numbers::pi */

static double E_of(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:84-87 */
    return P->Om * (1 + z) * (1 + z) * (1 + z) + P->OL;
}
static double Om_of(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:79-82 */
    return P->Om * (1 + z) * (1 + z) * (1 + z) / E_of(P, z);
}
double orc_delta_c(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:74-77 */
    return 1.686 * (1 + 0.0123 * log10(Om_of(P, z)));
}
static double growth(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:125-129 */
    double om_m = Om_of(P, z);
    return 2.5 / (z + 1) * om_m /
           (pow(om_m, 4. / 7.) - P->OL + (1. + 0.5 * om_m) * (1 + P->OL / 70));
}

static double tophat(double k, double R)
{   /* src/Powerspectrum.cpp:104-108 */
    double x = k * R;
    return 3 / x / x / x * (sin(x) - x * cos(x));
}
static double d_tophat(double k, double R)
{   /* src/Powerspectrum.cpp:110-114 */
    double x = k * R;
    return ((x * x - 3.) * sin(x) + 3. * x * cos(x)) * 3 * k / x / x / x / x;
}

double orc_transfer(const orc_pk *P, double k)
{   /* src/Powerspectrum.cpp:153-186 */
    if (k == 0.0) return 1.0;
    double q = k / 13.41 / P->k_equality;
    double xx = k * P->sound_horizon;
    double T_c_ln_beta = log(2.718282 + 1.8 * P->beta_c * q);
    double T_c_ln_nobeta = log(2.718282 + 1.8 * q);
    double T_c_C_alpha = 14.2 / P->alpha_c + 386.0 / (1.0 + 69.9 * pow(q, 1.08));
    double T_c_C_noalpha = 14.2 + 386.0 / (1 + 69.9 * pow(q, 1.08));
    double T_c_f = 1.0 / (1.0 + pow(xx / 5.4, 4));
    double T_c = T_c_f * T_c_ln_beta / (T_c_ln_beta + T_c_C_noalpha * q * q) +
                 (1. - T_c_f) * T_c_ln_beta / (T_c_ln_beta + T_c_C_alpha * q * q);
    double s_tilde = P->sound_horizon * pow(1. + pow(P->beta_node / xx, 3), -1. / 3.);
    double xx_tilde = k * s_tilde;
    double T_b_T0 = T_c_ln_nobeta / (T_c_ln_nobeta + T_c_C_noalpha * q * q);
    double T_b = sin(xx_tilde) / (xx_tilde) *
                 (T_b_T0 / (1. + pow(xx / 5.2, 2)) +
                  P->alpha_b / (1. + pow(P->beta_b / xx, 3)) * exp(-pow(k / P->k_silk, 1.4)));
    double f_baryon = P->obhh / P->omhh;
    return f_baryon * T_b + (1. - f_baryon) * T_c;
}

double orc_spectrum(const orc_pk *P, double k, double z)
{   /* src/Powerspectrum.cpp:189-196 */
    double g = growth(P, z) / growth(P, 0.0);
    double trans = orc_transfer(P, k);
    return P->amplitude * trans * trans * g * g * pow(k, P->ns);
}

typedef struct {
    const orc_pk *P;
    double R, dR, z;
} sig_ctx;

static int integrand_amplitude(unsigned ndim, size_t npt, const double *k, void *fd,
                               unsigned fdim, double *v)
{   /* src/Powerspectrum.cpp:79-102 */
    (void)fdim;
    const orc_pk *P = ((const sig_ctx *)fd)->P;
    double R = 8. / P->H0 * 100;
    for (size_t i = 0; i < npt; ++i) {
        double k_ = k[i * ndim];
        double W = tophat(k_, R);
        double T = orc_transfer(P, k_);
        v[i] = W * W * T * T * pow(k_, P->ns + 2);
    }
    return 0;
}

static int integrand_sigma2(unsigned ndim, size_t npt, const double *k, void *fd, unsigned fdim,
                            double *v)
{   /* src/Powerspectrum.cpp:219-243 */
    (void)fdim;
    const sig_ctx *C = (const sig_ctx *)fd;
    for (size_t i = 0; i < npt; ++i) {
        double k_ = k[i * ndim];
        double W = tophat(k_, C->R);
        v[i] = k_ * k_ * W * W * orc_spectrum(C->P, k_, C->z);
    }
    return 0;
}

static int integrand_dsigma2(unsigned ndim, size_t npt, const double *k, void *fd, unsigned fdim,
                             double *v)
{   /* src/Powerspectrum.cpp:267-293 */
    (void)fdim;
    const sig_ctx *C = (const sig_ctx *)fd;
    for (size_t i = 0; i < npt; ++i) {
        double k_ = k[i * ndim];
        double W = tophat(k_, C->R);
        double Wprime = d_tophat(k_, C->R);
        v[i] = k_ * k_ * W * Wprime * C->dR * orc_spectrum(C->P, k_, C->z);
    }
    return 0;
}

static double integrate_k(orc_integrand_v f, sig_ctx *C)
{
    double lo[1] = {0}, hi[1] = {1e12}, r = 0, e = 0;
    size_t ne;
    orc_hcubature_v(1, f, C, 1, lo, hi, 0, 0, 1e-4, 0, &r, &e, &ne);
    return r;
}

int orc_pk_init(orc_pk *P, const double cosmo[6])
{
    memset(P, 0, sizeof *P);
    P->Om = cosmo[0];
    P->OL = cosmo[1];
    P->Ob = cosmo[2];
    P->s8 = cosmo[3];
    P->H0 = cosmo[4];
    P->ns = cosmo[5];
    /* src/Cosmology.h:41-47 */
    P->rho_crit = 3 * P->H0 * P->H0 * kMpcInKm / 8 / kPiTrunc / kG;
    /* set_transfer_parameters, src/Powerspectrum.cpp:15-69 */
    double h = P->H0 / 100;
    P->omhh = P->Om * h * h;
    P->obhh = P->Ob * h * h;
    double f_baryon = P->obhh / P->omhh;
    double Tcmb = 2.72548;
    P->theta_cmb = Tcmb / 2.7;
    double theta_cmbSq = P->theta_cmb * P->theta_cmb;
    double theta_cmb4 = theta_cmbSq * theta_cmbSq;
    double omhh = P->omhh, obhh = P->obhh;
    P->z_equality = 2.50e4 * omhh / theta_cmb4;
    P->k_equality = 0.0746 * omhh / theta_cmbSq;
    double z_drag_b1 = 0.313 * pow(omhh, -0.419) * (1.0 + 0.607 * pow(omhh, 0.674));
    double z_drag_b2 = 0.238 * pow(omhh, 0.223);
    P->z_drag = 1291.0 * pow(omhh, 0.251) / (1.0 + 0.659 * pow(omhh, 0.828)) *
                (1.0 + z_drag_b1 * pow(obhh, z_drag_b2));
    P->R_drag = 31.5 * obhh / (theta_cmb4) * (1000.0 / (1.0 + P->z_drag));
    P->R_equality = 31.5 * obhh / (theta_cmb4) * (1000.0 / P->z_equality);
    P->sound_horizon = 2.0 / 3.0 / P->k_equality * sqrt(6.0 / P->R_equality) *
                       log((sqrt(1.0 + P->R_drag) + sqrt(P->R_drag + P->R_equality)) /
                           (1.0 + sqrt(P->R_equality)));
    P->k_silk = 1.6 * pow(obhh, 0.52) * pow(omhh, 0.73) * (1.0 + pow(10.4 * omhh, -0.95));
    double alpha_c_a1 = pow(46.9 * omhh, 0.670) * (1.0 + pow(32.1 * omhh, -0.532));
    double alpha_c_a2 = pow(12.0 * omhh, 0.424) * (1.0 + pow(45.0 * omhh, -0.582));
    P->alpha_c = pow(alpha_c_a1, -f_baryon) * pow(alpha_c_a2, -pow(f_baryon, 3));
    double beta_c_b1 = 0.944 / (1.0 + pow(458.0 * omhh, -0.708));
    double beta_c_b2 = pow(0.395 * omhh, -0.0266);
    P->beta_c = 1.0 / (1.0 + beta_c_b1 * (pow(1.0 - f_baryon, beta_c_b2) - 1.0));
    double y = P->z_equality / (1.0 + P->z_drag);
    double alpha_b_G =
        y * (-6.0 * sqrt(1.0 + y) + (2.0 + 3.0 * y) * log((sqrt(1.0 + y) + 1.0) / (sqrt(1.0 + y) - 1.0)));
    P->alpha_b = 2.07 * P->k_equality * P->sound_horizon * pow(1.0 + P->R_drag, -0.75) * alpha_b_G;
    P->beta_node = 8.41 * pow(omhh, 0.435);
    P->beta_b = 0.5 + f_baryon + (3.0 - 2.0 * f_baryon) * sqrt(pow(17.2 * omhh, 2.0) + 1.0);
    /* set_amplitude, src/Powerspectrum.cpp:67-77 */
    double factor = kPi * P->s8;
    sig_ctx C = {P, 0, 0, 0};
    double result = integrate_k(integrand_amplitude, &C);
    P->amplitude = 2 * factor * factor / result;
    return 0;
}

double orc_sigma2(const orc_pk *P, double m, double z)
{   /* src/Powerspectrum.cpp:198-216 */
    double om = Om_of(P, z);
    sig_ctx C = {P, pow(0.75 / kPi * m / P->rho_crit / om, 1. / 3.), 0, z};
    return integrate_k(integrand_sigma2, &C) / 2 / kPi / kPi;
}

double orc_dsigma2dm(const orc_pk *P, double m, double z)
{   /* src/Powerspectrum.cpp:246-264 */
    double rho_m = P->rho_crit * Om_of(P, z);
    sig_ctx C = {P, 0.6204 * pow(m / rho_m, 1. / 3.), 0.2068 * pow(rho_m * m * m, -1. / 3.), z};
    return integrate_k(integrand_dsigma2, &C) / kPi / kPi;
}

double orc_mstar(const orc_pk *P, double z)
{   /* src/Powerspectrum.cpp:117-140: the first of 256 log-spaced masses in [1e10, 1e18)
       closest to sigma(m) = delta_c */
    double dc = orc_delta_c(P, z);
    const double m_min = 1e10, m_max = 1e18;
    const int Nb = 256;
    double m_bin = log(m_max / m_min) / Nb, best = 0, bm = 0;
    for (int i = 0; i < Nb; ++i) {
        double m = exp(log(m_min) + m_bin * i);
        double diff = dc - sqrt(orc_sigma2(P, m, z));
        double d = sqrt(diff * diff);
        if (i == 0 || d < best) {
            best = d;
            bm = m;
        }
    }
    return bm;
}

double orc_concentration(double m, double mstar, double z)
{   /* src/Powerspectrum.cpp:143-150 */
    return 9 / (1. + z) * pow(m / mstar, -0.13);
}

double orc_hmf(const orc_pk *P, double m, double z)
{   /* src/HMF.cpp:7-33 */
    double A = 0.322, q = 0.707, p = 0.3;
    double sigma2 = orc_sigma2(P, m, z);
    double dsigma2 = orc_dsigma2dm(P, m, z);
    double delta_c = orc_delta_c(P, z);
    double rho_mean = Om_of(P, z) * P->rho_crit;
    double nuSq = delta_c * delta_c / sigma2;
    return -rho_mean / m / sigma2 * dsigma2 * A * (1 + pow(q * nuSq, -p)) *
           sqrt(q * nuSq / 2 / kPiTrunc) * exp(-0.5 * q * nuSq);
}

double orc_halo_bias(const orc_pk *P, double m, double z)
{   /* src/HMF.cpp:36-49 */
    double q = 0.707, p = 0.3;
    double sigma2 = orc_sigma2(P, m, z);
    double delta_c = orc_delta_c(P, z);
    return 1 + 1. / delta_c *
                   (q * delta_c * delta_c / sigma2 - 1 + 2 * p / (1 + pow(q * delta_c * delta_c / sigma2, p)));
}

static int integrand_chi(unsigned ndim, size_t npt, const double *z, void *fd, unsigned fdim,
                         double *v)
{   /* src/Cosmology.cpp:106-122 */
    (void)fdim;
    const orc_pk *P = (const orc_pk *)fd;
    for (size_t i = 0; i < npt; ++i) v[i] = kC / P->H0 / sqrt(E_of(P, z[i * ndim]));
    return 0;
}

double orc_comoving(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:89-98 */
    double lo[1] = {0}, hi[1] = {z}, r = 0, e = 0;
    size_t ne;
    orc_hcubature_v(1, integrand_chi, (void *)P, 1, lo, hi, 0, 0, 1e-4, 0, &r, &e, &ne);
    return r;
}

double orc_dcomoving(const orc_pk *P, double z)
{   /* src/Cosmology.cpp:101-104 */
    return kC / P->H0 / sqrt(E_of(P, z));
}

int orc_precompute(const double cosmo[6], const double *zs_src, const double *nz_src, int Ns,
                   double zmin, double zmax, double mmin, double mmax, double kmin, double kmax,
                   int N, double *g, double *w, double *dwdz, double *P_lin, double *conc,
                   double *hmf, double *b_h)
{   /* src/doPrecomputations.cpp:40-134 */
    orc_pk P;
    orc_pk_init(&P, cosmo);
    double z_bin = (zmax - zmin) / N, m_bin = log(mmax / mmin) / N, k_bin = log(kmax / kmin) / N;
    double *zs = malloc(sizeof(double) * N), *ms = malloc(sizeof(double) * N),
           *ks = malloc(sizeof(double) * N), *wsrc = malloc(sizeof(double) * (Ns > 0 ? Ns : 1)),
           *mst = malloc(sizeof(double) * N);
    for (int i = 0; i < N; ++i) {
        zs[i] = zmin + i * z_bin;
        ms[i] = exp(log(mmin) + m_bin * i);
        ks[i] = exp(log(kmin) + k_bin * i);
    }
    /* lensing efficiency (src/Cosmology.cpp:132-166): the source distances are the
       same for every z, computed once here */
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < Ns; ++j) wsrc[j] = orc_comoving(&P, zs_src[j]);
    double deltaZ = Ns > 0 ? (zs_src[Ns - 1] - zs_src[0]) / Ns : 0;
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < N; ++i) {
        double wi = orc_comoving(&P, zs[i]), r = 0;
        for (int j = 0; j < Ns; ++j)
            if (zs_src[j] >= zs[i]) r += nz_src[j] * (wsrc[j] - wi) / wsrc[j];
        g[i] = r * deltaZ;
        w[i] = wi;
        dwdz[i] = orc_dcomoving(&P, zs[i]);
        mst[i] = orc_mstar(&P, zs[i]);
    }
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            P_lin[i * N + j] = orc_spectrum(&P, ks[j], zs[i]);
            conc[i * N + j] = orc_concentration(ms[j], mst[i], zs[i]);
            hmf[i * N + j] = orc_hmf(&P, ms[j], zs[i]);
            b_h[i * N + j] = orc_halo_bias(&P, ms[j], zs[i]);
        }
    free(zs);
    free(ms);
    free(ks);
    free(wsrc);
    free(mst);
    return 0;
}
