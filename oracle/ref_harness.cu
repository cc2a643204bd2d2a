// ref_harness.cu -- in-memory driver for the reference's own CPU build (TEST INFRASTRUCTURE).
//
// Compiled by oracle/build_ref.sh together with the reference's unmodified
// sources (HOD.cu, generalFunctions.cu, NNMap_Model.cu, NMapMap_Model.cu,
// hcubature.cpp, Cosmology.cpp, Params.cpp) WITHOUT -DGPU, i.e. the OpenMP CPU
// path.  It constructs NNMap_Model / NMapMap_Model from arrays (bypassing the
// ASCII table readers) and exposes a C ABI so that the oracle restatement can
// be pinned against the reference bit for bit.  Output lives in oracle/_ref/.
//
// Compiled a second time with -DSCALING=1 (the reference's satellite-variance
// rescaling, src/Makefile:17-21) together with a SCALING build of
// NNMap_Model.cu into libg3lref_scaling.so.  That build has only the NNMap model:
// the scaled constructor replaces ref_nnmap_create, and the NMapMap entry points
// are left out (NMapMap_Model.cu does not compile with SCALING set).
#include "Cosmology.h"
#include "Function.h"
#include "Function2D.h"
#include "HMF.h"
#include "HOD.h"
#include "NMapMap_Model.h"
#include "NNMap_Model.h"
#include "Params.h"
#include "Powerspectrum.h"
#include "cubature.h"
#include "generalFunctions.h"

#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct RefTables {
    std::vector<double> g, p1, p2, w, dwdz, hmf, P_lin, b_h, conc;
};

struct RefNNMap {
    RefTables T;
    g3lhalo::Cosmology *cosmo;
    g3lhalo::Params *par1, *par2;
    g3lhalo::HOD *hod1, *hod2;
    g3lhalo::NNMap_Model *model;
};

struct RefNMapMap {
    RefTables T;
    g3lhalo::Cosmology *cosmo;
    g3lhalo::Params *par;
    g3lhalo::HOD *hod;
    g3lhalo::NMapMap_Model *model;
};

void fill_tables(RefTables &T, int N, const double *g, const double *p1, const double *p2,
                 const double *w, const double *dwdz, const double *hmf, const double *P_lin,
                 const double *b_h, const double *conc)
{
    T.g.assign(g, g + N);
    T.p1.assign(p1, p1 + N);
    T.p2.assign(p2, p2 + N);
    T.w.assign(w, w + N);
    T.dwdz.assign(dwdz, dwdz + N);
    T.hmf.assign(hmf, hmf + N * N);
    T.P_lin.assign(P_lin, P_lin + N * N);
    T.b_h.assign(b_h, b_h + N * N);
    T.conc.assign(conc, conc + N * N);
}

// hod[6] = {f, alpha, Mth, sigma, M', beta}
g3lhalo::Params *make_params(const double *h)
{
    return new g3lhalo::Params(h[0], h[1], h[2], h[3], h[4], h[5]);
}

struct Counter {
    integrand_v f;
    void *fdata;
    size_t n;
};

int counting(unsigned ndim, size_t npt, const double *x, void *d, unsigned fdim, double *fval)
{
    Counter *c = (Counter *)d;
    c->n += npt;
    return c->f(ndim, npt, x, c->fdata, fdim, fval);
}

}  // namespace

extern "C" {

#if SCALING
// The reference's SCALING constructor (src/NNMap_Model.cu:103-200).  Its destructor
// free()s the two arrays (src/NNMap_Model.cu:231-234), so they are handed over as
// malloc'd copies.  scaling1/2: [N] per mass bin.
void *ref_nnmap_create_scaled(const double *cosmo, double zmin, double zmax, double kmin,
                              double kmax, double mmin, double mmax, int N, const double *g,
                              const double *p1, const double *p2, const double *w,
                              const double *dwdz, const double *hmf, const double *P_lin,
                              const double *b_h, const double *conc, const double *scaling1,
                              const double *scaling2, const double *hod1, const double *hod2,
                              int same_pop, double A, double eps)
{
    RefNNMap *R = new RefNNMap;
    fill_tables(R->T, N, g, p1, p2, w, dwdz, hmf, P_lin, b_h, conc);
    double *s1 = (double *)malloc(sizeof(double) * N);
    double *s2 = (double *)malloc(sizeof(double) * N);
    std::memcpy(s1, scaling1, sizeof(double) * N);
    std::memcpy(s2, scaling2, sizeof(double) * N);
    R->cosmo = new g3lhalo::Cosmology(cosmo[0], cosmo[1], cosmo[2], cosmo[3], cosmo[4], cosmo[5]);
    R->par1 = make_params(hod1);
    R->par2 = make_params(hod2);
    R->hod1 = new g3lhalo::HOD(R->par1);
    R->hod2 = same_pop ? R->hod1 : new g3lhalo::HOD(R->par2);
    R->model = new g3lhalo::NNMap_Model(R->cosmo, zmin, zmax, kmin, kmax, mmin, mmax, N,
                                        R->T.g.data(), R->T.p1.data(), R->T.p2.data(),
                                        R->T.w.data(), R->T.dwdz.data(), R->T.hmf.data(),
                                        R->T.P_lin.data(), R->T.b_h.data(), R->T.conc.data(), s1,
                                        s2, R->hod1, R->hod2, A, eps);
    return R;
}
#else
// cosmo[6] = {Om, OL, Ob, s8, H0, ns}
void *ref_nnmap_create(const double *cosmo, double zmin, double zmax, double kmin, double kmax,
                       double mmin, double mmax, int N, const double *g, const double *p1,
                       const double *p2, const double *w, const double *dwdz, const double *hmf,
                       const double *P_lin, const double *b_h, const double *conc,
                       const double *hod1, const double *hod2, int same_pop, double A, double eps)
{
    RefNNMap *R = new RefNNMap;
    fill_tables(R->T, N, g, p1, p2, w, dwdz, hmf, P_lin, b_h, conc);
    R->cosmo = new g3lhalo::Cosmology(cosmo[0], cosmo[1], cosmo[2], cosmo[3], cosmo[4], cosmo[5]);
    R->par1 = make_params(hod1);
    R->par2 = make_params(hod2);
    R->hod1 = new g3lhalo::HOD(R->par1);
    R->hod2 = same_pop ? R->hod1 : new g3lhalo::HOD(R->par2);
    R->model = new g3lhalo::NNMap_Model(R->cosmo, zmin, zmax, kmin, kmax, mmin, mmax, N,
                                        R->T.g.data(), R->T.p1.data(), R->T.p2.data(),
                                        R->T.w.data(), R->T.dwdz.data(), R->T.hmf.data(),
                                        R->T.P_lin.data(), R->T.b_h.data(), R->T.conc.data(),
                                        R->hod1, R->hod2, A, eps);
    return R;
}
#endif

void ref_nnmap_destroy(void *h)
{
    RefNNMap *R = (RefNNMap *)h;
    delete R->model;
    if (R->hod2 != R->hod1) delete R->hod2;
    delete R->hod1;
    delete R->par1;
    delete R->par2;
    delete R->cosmo;
    delete R;
}

void ref_nnmap_densities(void *h, double *rho_bar, double *nbar1, double *nbar2)
{
    RefNNMap *R = (RefNNMap *)h;
    int N = R->model->Nbins;
    std::memcpy(rho_bar, R->model->rho_bar, sizeof(double) * N);
    std::memcpy(nbar1, R->model->n_bar1, sizeof(double) * N);
    std::memcpy(nbar2, R->model->n_bar2, sizeof(double) * N);
}

// Raw integral of one term through hcubature_v with the stock integrand callback.
int ref_nnmap_term(void *h, int term, const double *th, int type1, int type2, size_t maxEval,
                   double rtol, double *val, double *err, size_t *neval)
{
    RefNNMap *R = (RefNNMap *)h;
    g3lhalo::NNMap_Model *M = R->model;
    g3lhalo::nnmap_container c;
    c.nnmap = M;
    c.theta1 = th[0];
    c.theta2 = th[1];
    c.theta3 = th[2];
    c.type1 = type1;
    c.type2 = type2;
    double lo[7], hi[7];
    int d = 0;
    lo[d] = std::log10(M->lmin_integral); hi[d++] = std::log10(M->lmax_integral);
    lo[d] = std::log10(M->lmin_integral); hi[d++] = std::log10(M->lmax_integral);
    lo[d] = M->phimin_integral; hi[d++] = M->phimax_integral;
    for (int j = 0; j < term; ++j) {
        lo[d] = std::log10(M->mmin_integral);
        hi[d++] = std::log10(M->mmax_integral);
    }
    lo[d] = M->zmin_integral; hi[d++] = M->zmax_integral;
    Counter cnt;
    cnt.f = term == 1 ? g3lhalo::NNM::integrand_1halo
          : term == 2 ? g3lhalo::NNM::integrand_2halo
                      : g3lhalo::NNM::integrand_3halo;
    cnt.fdata = &c;
    cnt.n = 0;
    int st = hcubature_v(1, counting, &cnt, d, lo, hi, maxEval, 0, rtol, ERROR_L1, val, err);
    *neval = cnt.n;
    return st;
}

// The stock per-term method (hard-coded maxEval and rtol, prefactor applied).
double ref_nnmap_method(void *h, int term, const double *th, int type1, int type2)
{
    RefNNMap *R = (RefNNMap *)h;
    if (term == 1) return R->model->NNMap_1h(th[0], th[1], th[2], type1, type2);
    if (term == 2) return R->model->NNMap_2h(th[0], th[1], th[2], type1, type2);
    return R->model->NNMap_3h(th[0], th[1], th[2], type1, type2);
}

// Integrand kernel at physical point pt = {l1, l2, phi, m..., z}.  The SCALING build
// passes the model's scaling arrays, as its integrands do (src/NNMap_Model.cu:527-531).
#if SCALING
#define SCALING_ARGS M->scaling1, M->scaling2
#else
#define SCALING_ARGS NULL, NULL
#endif
double ref_nnmap_kernel(void *h, int term, const double *th, const double *pt, int type1,
                        int type2)
{
    RefNNMap *R = (RefNNMap *)h;
    g3lhalo::NNMap_Model *M = R->model;
    g3lhalo::HOD *h1 = type1 == 1 ? M->hod1 : M->hod2;
    g3lhalo::HOD *h2 = type2 == 1 ? M->hod1 : M->hod2;
    const double *nb1 = type1 == 1 ? M->n_bar1 : M->n_bar2;
    const double *nb2 = type2 == 1 ? M->n_bar1 : M->n_bar2;
    if (term == 1)
        return g3lhalo::NNM::kernel_function_1halo(
            th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], M->zmin, M->zmax, M->mmin,
            M->mmax, M->Nbins, h1, h2, NULL, NULL, M->A, M->epsilon, M->g, M->p_lens1, M->p_lens2,
            M->w, M->dwdz, M->hmf, M->concentration, M->rho_bar, nb1, nb2, SCALING_ARGS);
    if (term == 2)
        return g3lhalo::NNM::kernel_function_2halo(
            th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], M->zmin, M->zmax,
            M->mmin, M->mmax, M->kmin, M->kmax, M->Nbins, h1, h2, NULL, NULL, M->A, M->epsilon,
            M->g, M->p_lens1, M->p_lens2, M->w, M->dwdz, M->hmf, M->P_lin, M->b_h,
            M->concentration, M->rho_bar, nb1, nb2, SCALING_ARGS);
    return g3lhalo::NNM::kernel_function_3halo(
        th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], pt[6], M->zmin, M->zmax,
        M->mmin, M->mmax, M->kmin, M->kmax, M->Nbins, h1, h2, NULL, NULL, M->g, M->p_lens1,
        M->p_lens2, M->w, M->dwdz, M->hmf, M->P_lin, M->b_h, M->concentration, M->rho_bar, nb1,
        nb2);
}

#if !SCALING
void *ref_nmapmap_create(const double *cosmo, double zmin, double zmax, double kmin,
                         double kmax, double mmin, double mmax, int N, const double *g,
                         const double *p, const double *w, const double *dwdz, const double *hmf,
                         const double *P_lin, const double *b_h, const double *conc,
                         const double *hod)
{
    RefNMapMap *R = new RefNMapMap;
    fill_tables(R->T, N, g, p, p, w, dwdz, hmf, P_lin, b_h, conc);
    R->cosmo = new g3lhalo::Cosmology(cosmo[0], cosmo[1], cosmo[2], cosmo[3], cosmo[4], cosmo[5]);
    R->par = make_params(hod);
    R->hod = new g3lhalo::HOD(R->par);
    R->model = new g3lhalo::NMapMap_Model(R->cosmo, zmin, zmax, kmin, kmax, mmin, mmax, N,
                                          R->T.g.data(), R->T.p1.data(), R->T.w.data(),
                                          R->T.dwdz.data(), R->T.hmf.data(), R->T.P_lin.data(),
                                          R->T.b_h.data(), R->T.conc.data(), R->hod);
    return R;
}

void ref_nmapmap_destroy(void *h)
{
    RefNMapMap *R = (RefNMapMap *)h;
    delete R->model;
    delete R->hod;
    delete R->par;
    delete R->cosmo;
    delete R;
}

void ref_nmapmap_densities(void *h, double *rho_bar, double *nbar)
{
    RefNMapMap *R = (RefNMapMap *)h;
    int N = R->model->Nbins;
    std::memcpy(rho_bar, R->model->rho_bar, sizeof(double) * N);
    std::memcpy(nbar, R->model->n_bar, sizeof(double) * N);
}

int ref_nmapmap_term(void *h, int term, const double *th, size_t maxEval, double rtol,
                     double *val, double *err, size_t *neval)
{
    RefNMapMap *R = (RefNMapMap *)h;
    g3lhalo::NMapMap_Model *M = R->model;
    g3lhalo::nmapmap_container c;
    c.nmapmap = M;
    c.theta1 = th[0];
    c.theta2 = th[1];
    c.theta3 = th[2];
    double lo[7], hi[7];
    int d = 0;
    lo[d] = std::log10(M->lmin_integral); hi[d++] = std::log10(M->lmax_integral);
    lo[d] = std::log10(M->lmin_integral); hi[d++] = std::log10(M->lmax_integral);
    lo[d] = M->phimin_integral; hi[d++] = M->phimax_integral;
    for (int j = 0; j < term; ++j) {
        lo[d] = std::log10(M->mmin_integral);
        hi[d++] = std::log10(M->mmax_integral);
    }
    lo[d] = M->zmin_integral; hi[d++] = M->zmax_integral;
    Counter cnt;
    cnt.f = term == 1 ? g3lhalo::NMM::integrand_1halo
          : term == 2 ? g3lhalo::NMM::integrand_2halo
                      : g3lhalo::NMM::integrand_3halo;
    cnt.fdata = &c;
    cnt.n = 0;
    int st = hcubature_v(1, counting, &cnt, d, lo, hi, maxEval, 0, rtol, ERROR_L1, val, err);
    *neval = cnt.n;
    return st;
}

double ref_nmapmap_method(void *h, int term, const double *th)
{
    RefNMapMap *R = (RefNMapMap *)h;
    if (term == 1) return R->model->NMapMap_1h(th[0], th[1], th[2]);
    if (term == 2) return R->model->NMapMap_2h(th[0], th[1], th[2]);
    return R->model->NMapMap_3h(th[0], th[1], th[2]);
}

double ref_nmapmap_kernel(void *h, int term, const double *th, const double *pt)
{
    RefNMapMap *R = (RefNMapMap *)h;
    g3lhalo::NMapMap_Model *M = R->model;
    if (term == 1)
        return g3lhalo::NMM::kernel_function_1halo(
            th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], M->zmin, M->zmax, M->mmin,
            M->mmax, M->Nbins, M->hod, NULL, M->g, M->p_lens, M->w, M->dwdz, M->hmf,
            M->concentration, M->rho_bar, M->n_bar);
    if (term == 2)
        return g3lhalo::NMM::kernel_function_2halo(
            th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], M->zmin, M->zmax,
            M->mmin, M->mmax, M->kmin, M->kmax, M->Nbins, M->hod, NULL, M->g, M->p_lens, M->w,
            M->dwdz, M->hmf, M->P_lin, M->b_h, M->concentration, M->rho_bar, M->n_bar);
    return g3lhalo::NMM::kernel_function_3halo(
        th[0], th[1], th[2], pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], pt[6], M->zmin, M->zmax,
        M->mmin, M->mmax, M->kmin, M->kmax, M->Nbins, M->hod, NULL, M->g, M->p_lens, M->w,
        M->dwdz, M->hmf, M->P_lin, M->b_h, M->concentration, M->rho_bar, M->n_bar);
}

#endif  // !SCALING

// The reference's cubature engine with a caller-supplied integrand.
int ref_hcubature_v(unsigned fdim, integrand_v f, void *fdata, unsigned dim, const double *xmin,
                    const double *xmax, size_t maxEval, double reqAbs, double reqRel, int norm,
                    double *val, double *err, size_t *neval)
{
    Counter cnt;
    cnt.f = f;
    cnt.fdata = fdata;
    cnt.n = 0;
    int st = hcubature_v(fdim, counting, &cnt, dim, xmin, xmax, maxEval, reqAbs, reqRel,
                         (error_norm)norm, val, err);
    *neval = cnt.n;
    return st;
}

#if !SCALING
// doPrecomputations.x without its file I/O (src/doPrecomputations.cpp:40-134): the
// same objects and calls, in the same order, on the same grids.  nz_z / nz_v: the
// source redshift distribution as the driver holds it (Function x / y values).
// 2-D outputs are z-major [N*N].  Also returns the power-spectrum amplitude.
void ref_precompute(const double *cosmo, const double *nz_z, const double *nz_v, int Ns,
                    double z_min, double z_max, double m_min, double m_max, double k_min,
                    double k_max, int Nbins, double *g, double *w, double *dwdz, double *P_lin,
                    double *conc, double *hmf_out, double *b_h, double *amplitude)
{
    double z_bin = (z_max - z_min) / Nbins;
    double m_bin = log(m_max / m_min) / Nbins;
    double k_bin = log(k_max / k_min) / Nbins;
    std::vector<double> zs, ms, ks;
    for (int i = 0; i < Nbins; i++) {
        zs.push_back(z_min + i * z_bin);
        ms.push_back(exp(log(m_min) + m_bin * i));
        ks.push_back(exp(log(k_min) + k_bin * i));
    }
    std::vector<double> nzx(nz_z, nz_z + Ns), nzy(nz_v, nz_v + Ns);
    g3lhalo::Cosmology cosmology(cosmo[0], cosmo[1], cosmo[2], cosmo[3], cosmo[4], cosmo[5]);
    std::vector<double> v;
    cosmology.getLensingEfficiency(zs, nzy, nzx, v);
    std::memcpy(g, v.data(), sizeof(double) * Nbins);
    v.clear();
    cosmology.getComovingDistance(zs, v);
    std::memcpy(w, v.data(), sizeof(double) * Nbins);
    v.clear();
    cosmology.getDerivativeComovingDistance(zs, v);
    std::memcpy(dwdz, v.data(), sizeof(double) * Nbins);
    g3lhalo::Powerspectrum powerspectrum(&cosmology);
    *amplitude = powerspectrum.amplitude;
    v.clear();
    powerspectrum.getSpectrum(zs, ks, v);
    std::memcpy(P_lin, v.data(), sizeof(double) * Nbins * Nbins);
    v.clear();
    powerspectrum.getConcentration(zs, ms, v);
    std::memcpy(conc, v.data(), sizeof(double) * Nbins * Nbins);
    g3lhalo::Halomassfunction hmf(&cosmology, &powerspectrum);
    v.clear();
    hmf.getHMF(zs, ms, v);
    std::memcpy(hmf_out, v.data(), sizeof(double) * Nbins * Nbins);
    v.clear();
    hmf.getHaloBias(zs, ms, v);
    std::memcpy(b_h, v.data(), sizeof(double) * Nbins * Nbins);
}

// single pieces, for point-level pinning
double ref_pk_piece(const double *cosmo, int what, double a, double b)
{
    g3lhalo::Cosmology c(cosmo[0], cosmo[1], cosmo[2], cosmo[3], cosmo[4], cosmo[5]);
    g3lhalo::Powerspectrum p(&c);
    g3lhalo::Halomassfunction h(&c, &p);
    switch (what) {
    case 0: return p.amplitude;
    case 1: return p.transfer(a);
    case 2: return p.spectrum(a, b);
    case 3: return p.sigma2(a, b);
    case 4: return p.mStar(a);
    case 5: return h.b_h(a, b);
    case 6: return c.comovingDistance(a);
    default: return 0;
    }
}
#endif

// The reference's ASCII readers as its drivers use them (src/calculateNNMap.cu:42-72).
// They exit() or throw on bad input, so callers pass valid files only.
int ref_function_read(const char *path, double def, int N, double min, double max, int log_bins,
                      double *out)
{
    g3lhalo::Function f(path, def);
    std::vector<double> v;
    int st = log_bins ? f.readLog(N, min, max, v) : f.read(N, min, max, v);
    std::memcpy(out, v.data(), sizeof(double) * v.size());
    return st;
}

int ref_function2d_read(const char *path, double def, int N, double min1, double max1,
                        double min2, double max2, double *out)
{
    g3lhalo::Function2D f(path, def);
    std::vector<double> v;
    int st = f.read(N, min1, max1, min2, max2, v);
    std::memcpy(out, v.data(), sizeof(double) * v.size());
    return st;
}

// {f, alpha, Mth, sigma, M', beta}
void ref_params_read(const char *path, double *out)
{
    g3lhalo::Params p(path);
    out[0] = p.f;
    out[1] = p.alpha;
    out[2] = p.mmin;
    out[3] = p.sigma;
    out[4] = p.mprime;
    out[5] = p.beta;
}

// {Om, OL, Ob, sigma8, H0, ns}
void ref_cosmology_read(const char *path, double *out)
{
    g3lhalo::Cosmology c(path);
    out[0] = c.Omega_m;
    out[1] = c.Omega_Lambda;
    out[2] = c.Omega_b;
    out[3] = c.sigma8;
    out[4] = c.H0;
    out[5] = c.ns;
}

// Physics primitives, for point-level pinning.
void ref_sici(double x, double *si, double *ci) { g3lhalo::SiCi(x, *si, *ci); }

}  // extern "C"
