// precompute.cu -- the reference's table precomputation on the device.
//
// doPrecomputations.x (src/doPrecomputations.cpp:40-134) fills the model's lookup
// tables from a cosmology and a source redshift distribution: the lensing efficiency,
// comoving distance and its derivative on the z grid (src/Cosmology.cpp:74-193), the
// linear power spectrum (Eisenstein & Hu transfer function normalised to sigma8,
// src/Powerspectrum.cpp:9-196), the concentration through M*(z) (:117-150, 296-313)
// and the Sheth-Tormen mass function and halo bias (src/HMF.cpp:7-84).  Its cost is
// ~28k adaptive 1-D integrals over k in [0, 1e12] for N = 64 bins (sigma^2 and
// dsigma^2/dm at every (z, m), sigma^2 at 256 masses per z for M*), each one run by
// the reference's hcubature_v on the host.
//
// Here every integral runs on the device.  One block integrates one integral at a
// time (grid-stride over the integrals): thread 0 keeps the reference's max-heap of
// regions with its running value/error sums, its Gladwell batch (pop the largest
// errors until the rest is within tolerance), its cut and its push order, so the
// refinement follows the reference's; the block's half-warps evaluate the 15-point
// Gauss-Kronrod rule of one region each, and lane 0 of each half-warp forms the
// rule's value and QUADPACK error in the reference's operation order
// (src/hcubature.cpp:620-765, 772-1021).  The heap and the batch live in shared memory.
// Integral parameters (radii, growth factors, grids) are computed on the host with
// the reference's expressions; the integrands and the tables are evaluated here.
// Compiled with -fmad=false, so results differ from the reference only by the
// device libm's last-ulp differences in sin, cos, exp, log and pow.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <new>
#include <string>
#include <vector>

#include "g3l_gpu.h"
#include "host_internal.h"

namespace g3l {
namespace {

constexpr int PC_THREADS = 128;
// live regions of one integral (the heap) and regions of one round (the batch, at most
// twice the heap): a first pass with 512 (48 KB of shared memory, 4 blocks per SM)
// integrates almost everything; integrals that need more run again with 2048.
constexpr int PC_CAP_SMALL = 512, PC_CAP_LARGE = 2048;
// G3L_PC_FIRST_CAP=64 makes the first pass hold only 64 regions, so that most
// integrals take the 2048-region pass (its results are the same: an integral that
// overflows starts again from its root region); used to test that pass.
constexpr int PC_CAP_TINY = 64;
constexpr int PC_MAX_ROUNDS = 4096;
constexpr size_t pc_smem(int cap) { return sizeof(double) * 4 * (cap + 2 * cap); }
constexpr size_t nbar_smem(int cap) { return pc_smem(cap) + sizeof(int) * cap; }

// QUADPACK qk15 nodes and weights (the reference's rule15gauss, src/hcubature.cpp:626-660)
__constant__ double cXgk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                               0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                               0.586087235467691130294144838258730, 0.405845151377397166906606412076961,
                               0.207784955007898467600689403773245, 0.0};
__constant__ double cWg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                              0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
__constant__ double cWgk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                               0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                               0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                               0.204432940075298892414161999234649, 0.209482141084727828012999174891714};

constexpr double kPiTrunc = 3.14159;   // src/constants.h:15
constexpr double kC = 2.99792e5;       // src/constants.h:39
constexpr double kPi = 3.14159265358979323846;  // std::numbers::pi (src/Powerspectrum.cpp:69)

// cosmology and Eisenstein & Hu transfer-function parameters (src/Powerspectrum.h:14-36)
struct PkDev {
    double Om, OL, H0, ns, rho_crit, amplitude;
    double omhh, obhh, k_equality, sound_horizon, k_silk, alpha_c, beta_c, alpha_b, beta_b,
        beta_node;
};

enum PcType { PC_AMP = 0, PC_SIGMA2 = 1, PC_DSIGMA2 = 2, PC_CHI = 3 };

struct PcTask {
    int type, pad;
    double R, dR, gz;  // top-hat radius, dR/dm, growth(z)/growth(0)
    double lo, hi;     // integration range
};

struct PcOut {
    double val, err;
    unsigned long long neval;
    int status, rounds;
};

__device__ __forceinline__ double E_of(const PkDev &P, double z)
{   // src/Cosmology.cpp:84-87
    return P.Om * (1 + z) * (1 + z) * (1 + z) + P.OL;
}
__device__ __forceinline__ double Om_of(const PkDev &P, double z)
{   // src/Cosmology.cpp:79-82
    return P.Om * (1 + z) * (1 + z) * (1 + z) / E_of(P, z);
}
__device__ __forceinline__ double delta_c(const PkDev &P, double z)
{   // src/Cosmology.cpp:74-77
    return 1.686 * (1 + 0.0123 * log10(Om_of(P, z)));
}
__device__ __forceinline__ double tophat(double k, double R)
{   // src/Powerspectrum.cpp:104-108
    double x = k * R;
    return 3 / x / x / x * (sin(x) - x * cos(x));
}
__device__ __forceinline__ double d_tophat(double k, double R)
{   // src/Powerspectrum.cpp:110-114
    double x = k * R;
    return ((x * x - 3.) * sin(x) + 3. * x * cos(x)) * 3 * k / x / x / x / x;
}

// The Eisenstein & Hu (1998, ApJ 496, 605) transfer function with baryon acoustic
// terms: eqs. 17-21 (CDM part T_c with the ln/C fitting forms), eqs. 21-24 (baryon part
// T_b with the node shift s_tilde and Silk damping), weighted by the baryon fraction.
// The names of its intermediate quantities are those of the paper's published code, and
// the operation order is the reference's (src/Powerspectrum.cpp:153-186), which the
// table parity (<= 1e-13 relative) depends on.
__device__ double transfer(const PkDev &P, double k)
{   // src/Powerspectrum.cpp:153-186
    if (k == 0.0) return 1.0;
    double q = k / 13.41 / P.k_equality;
    double xx = k * P.sound_horizon;
    double T_c_ln_beta = log(2.718282 + 1.8 * P.beta_c * q);
    double T_c_ln_nobeta = log(2.718282 + 1.8 * q);
    double T_c_C_alpha = 14.2 / P.alpha_c + 386.0 / (1.0 + 69.9 * pow(q, 1.08));
    double T_c_C_noalpha = 14.2 + 386.0 / (1 + 69.9 * pow(q, 1.08));
    double T_c_f = 1.0 / (1.0 + pow(xx / 5.4, 4));
    double T_c = T_c_f * T_c_ln_beta / (T_c_ln_beta + T_c_C_noalpha * q * q) +
                 (1. - T_c_f) * T_c_ln_beta / (T_c_ln_beta + T_c_C_alpha * q * q);
    double s_tilde = P.sound_horizon * pow(1. + pow(P.beta_node / xx, 3), -1. / 3.);
    double xx_tilde = k * s_tilde;
    double T_b_T0 = T_c_ln_nobeta / (T_c_ln_nobeta + T_c_C_noalpha * q * q);
    double T_b = sin(xx_tilde) / (xx_tilde) *
                 (T_b_T0 / (1. + pow(xx / 5.2, 2)) +
                  P.alpha_b / (1. + pow(P.beta_b / xx, 3)) * exp(-pow(k / P.k_silk, 1.4)));
    double f_baryon = P.obhh / P.omhh;
    return f_baryon * T_b + (1. - f_baryon) * T_c;
}

// P_lin(k, z) with gz = growth(z)/growth(0) (src/Powerspectrum.cpp:189-196)
__device__ __forceinline__ double spectrum(const PkDev &P, double k, double gz)
{
    double trans = transfer(P, k);
    return P.amplitude * trans * trans * gz * gz * pow(k, P.ns);
}

__device__ double integrand(const PkDev &P, const PcTask &t, double x)
{
    switch (t.type) {
    case PC_AMP: {  // src/Powerspectrum.cpp:79-102
        double R = 8. / P.H0 * 100;
        double W = tophat(x, R);
        double T = transfer(P, x);
        return W * W * T * T * pow(x, P.ns + 2);
    }
    case PC_SIGMA2: {  // src/Powerspectrum.cpp:219-243
        double W = tophat(x, t.R);
        return x * x * W * W * spectrum(P, x, t.gz);
    }
    case PC_DSIGMA2: {  // src/Powerspectrum.cpp:267-293
        double W = tophat(x, t.R);
        double Wprime = d_tophat(x, t.R);
        return x * x * W * Wprime * t.dR * spectrum(P, x, t.gz);
    }
    default:  // comoving distance integrand c/H0/sqrt(E(z)) (src/Cosmology.cpp:101-122)
        return kC / P.H0 / sqrt(E_of(P, x));
    }
}

// 15-point Gauss-Kronrod value and QUADPACK error of one region from its point values
// in the reference's order (centre, then the Gauss pairs, then the Kronrod pairs)
__device__ void rule_gk15(const double *vk, double hw, double &val, double &err)
{
    double rg = vk[0] * cWg[3], rk = vk[0] * cWgk[7];
    double rabs = fabs(rk);
    int n = 1;
    for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        double v = vk[n] + vk[n + 1];
        rg += cWg[j] * v;
        rk += cWgk[j2] * v;
        rabs += cWgk[j2] * (fabs(vk[n]) + fabs(vk[n + 1]));
        n += 2;
    }
    for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rk += cWgk[j2] * (vk[n] + vk[n + 1]);
        rabs += cWgk[j2] * (fabs(vk[n]) + fabs(vk[n + 1]));
        n += 2;
    }
    val = rk * hw;
    double mean = rk * 0.5;
    double rasc = cWgk[7] * fabs(vk[0] - mean);
    n = 1;
    for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        rasc += cWgk[j2] * (fabs(vk[n] - mean) + fabs(vk[n + 1] - mean));
        n += 2;
    }
    for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rasc += cWgk[j2] * (fabs(vk[n] - mean) + fabs(vk[n + 1] - mean));
        n += 2;
    }
    double e = fabs(rk - rg) * hw;
    rabs *= hw;
    rasc *= hw;
    if (rasc != 0 && e != 0) {
        double scale = pow((200 * e / rasc), 1.5);
        e = (scale < 1) ? rasc * scale : rasc;
    }
    if (rabs > DBL_MIN / (50 * DBL_EPSILON)) {
        double min_err = 50 * DBL_EPSILON * rabs;
        if (min_err > e) e = min_err;
    }
    err = e;
}

// the i-th Gauss-Kronrod abscissa of the region (c, hw), in the reference's order
__device__ __forceinline__ double gk_point(double c, double hw, int i)
{
    if (i == 0) return c;
    const int j = (i - 1) >> 1;  // pair index
    const double w = i < 7 ? hw * cXgk[2 * j + 1] : hw * cXgk[2 * (j - 3)];
    return (i & 1) ? c - w : c + w;
}

struct Heap {
    double *c, *hw, *val, *err;
};

__device__ __forceinline__ bool converged(double err, double val)
{   // src/converged.h:10-14 with reqAbs = 0, reqRel = 1e-4
    return !(err > 0 && err > fabs(val) * 1e-4);
}

// the reference's heap discipline (src/hcubature.cpp:772-890), on shared arrays
__device__ void heap_push(Heap H, int &n, double &hv, double &he, double c, double hw, double v,
                          double e)
{
    hv += v;
    he += e;
    int ins = n++;
    while (ins) {
        int parent = (ins - 1) / 2;
        if (e <= H.err[parent]) break;
        H.c[ins] = H.c[parent];
        H.hw[ins] = H.hw[parent];
        H.val[ins] = H.val[parent];
        H.err[ins] = H.err[parent];
        ins = parent;
    }
    H.c[ins] = c;
    H.hw[ins] = hw;
    H.val[ins] = v;
    H.err[ins] = e;
}

__device__ void heap_pop(Heap H, int &nn, double &hv, double &he, double &c, double &hw, double &v,
                         double &e)
{
    c = H.c[0];
    hw = H.hw[0];
    v = H.val[0];
    e = H.err[0];
    const int n = nn - 1;
    H.c[0] = H.c[n];
    H.hw[0] = H.hw[n];
    H.val[0] = H.val[n];
    H.err[0] = H.err[n];
    nn = n;
    int i = 0, child;
    while ((child = i * 2 + 1) < n) {
        int largest = (H.err[child] <= H.err[i]) ? i : child;
        if (++child < n && H.err[largest] < H.err[child]) largest = child;
        if (largest == i) break;
        double t;
        t = H.c[i]; H.c[i] = H.c[largest]; H.c[largest] = t;
        t = H.hw[i]; H.hw[i] = H.hw[largest]; H.hw[largest] = t;
        t = H.val[i]; H.val[i] = H.val[largest]; H.val[largest] = t;
        t = H.err[i]; H.err[i] = H.err[largest]; H.err[largest] = t;
        i = largest;
    }
    hv -= v;
    he -= e;
}

// One adaptive 15-point Gauss-Kronrod integral over [lo, hi] by the whole block, with
// the reference's refinement: thread 0 keeps the heap, the Gladwell batch and the cut;
// ev(nb, bc, bh, bv, be) is called by every thread and evaluates the batch's regions
// (centres bc, half-widths bh) into their values bv and errors be.  Status: 0 ok,
// G3L_ERR_POOL (more than CAP live regions), G3L_ERR_ROUNDS (more than PC_MAX_ROUNDS
// rounds).  The result is valid in thread 0; the block is synchronised on return.
template <int CAP, class Eval>
__device__ PcOut gk_integrate(double lo, double hi, double *sm, const Eval &ev)
{
    constexpr int PC_CAP = CAP, PC_BATCH = 2 * CAP;
    Heap H{sm, sm + PC_CAP, sm + 2 * PC_CAP, sm + 3 * PC_CAP};
    double *bc = sm + 4 * PC_CAP, *bh = bc + PC_BATCH, *bv = bh + PC_BATCH, *be = bv + PC_BATCH;
    __shared__ int s_nb, s_done;
    // thread 0's state: heap size, running sums, counters
    int n = 0, status = 0, rounds = 0;
    double hv = 0, he = 0;
    unsigned long long neval = 15;
    if (threadIdx.x == 0) {
        bc[0] = 0.5 * (lo + hi);
        bh[0] = 0.5 * (hi - lo);
        s_nb = 1;
        s_done = 0;
    }
    __syncthreads();
    while (true) {
        ev(s_nb, bc, bh, bv, be);
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nb = s_nb;
            for (int b = 0; b < nb; ++b) heap_push(H, n, hv, he, bc[b], bh[b], bv[b], be[b]);
            int nbn = 0;
            if (converged(he, hv)) {
                s_done = 1;
            } else if (++rounds > PC_MAX_ROUNDS) {
                status = G3L_ERR_ROUNDS;
                s_done = 1;
            } else {
                // Gladwell batch: pop until the error left is within tolerance
                double eErr = he;
                const double eVal = hv;
                do {
                    // after this pop and the pushes the heap holds n + nbn + 1 regions
                    if (n + nbn + 1 > PC_CAP) {
                        status = G3L_ERR_POOL;
                        s_done = 1;
                        break;
                    }
                    double c, hw, v, e;
                    heap_pop(H, n, hv, he, c, hw, v, e);
                    eErr -= e;
                    const double h2 = hw * 0.5;  // cut (src/hcubature.cpp:206-218)
                    bc[nbn] = c - h2;
                    bh[nbn] = h2;
                    bc[nbn + 1] = c + h2;
                    bh[nbn + 1] = h2;
                    nbn += 2;
                    neval += 30;
                    if (converged(eErr, eVal)) break;
                } while (n > 0);
            }
            s_nb = nbn;
        }
        __syncthreads();
        if (s_done) break;
    }
    PcOut o{0, 0, neval, status, rounds};
    if (threadIdx.x == 0) {
        double v = 0, e = 0;
        for (int i = 0; i < n; ++i) {
            v += H.val[i];
            e += H.err[i];
        }
        o.val = v;
        o.err = e;
    }
    __syncthreads();
    return o;
}

// The same refinement with the live regions in plain arrays instead of a heap, for
// integrals whose result needs agree with the reference's to ~1e-12 rather than in the
// last bit (n_bar): each round the whole block sorts the live regions by error
// (bitonic, descending) and thread 0 walks that order with the reference's Gladwell
// rule (pop the largest errors until the rest is within tolerance), so the regions cut
// are the heap's; only the order among exactly equal errors and the summation order of
// the totals differ.  Shared memory: pc_smem(CAP) plus CAP ints.
template <int CAP, class Eval>
__device__ PcOut gk_integrate_sorted(double lo, double hi, double *sm, const Eval &ev)
{
    constexpr int PC_BATCH = 2 * CAP;
    double *lc = sm, *lh = sm + CAP, *lv = sm + 2 * CAP, *le = sm + 3 * CAP;
    double *bc = sm + 4 * CAP, *bh = bc + PC_BATCH, *bv = bh + PC_BATCH, *be = bv + PC_BATCH;
    int *ord = (int *)(be + PC_BATCH);
    __shared__ int s_nb, s_done, s_n, s_K, s_status, s_rounds;
    __shared__ double s_red[2][32];
    __shared__ unsigned long long s_neval;
    const int tid = threadIdx.x, nth = blockDim.x;
    if (tid == 0) {
        bc[0] = 0.5 * (lo + hi);
        bh[0] = 0.5 * (hi - lo);
        s_nb = 1;
        s_done = 0;
        s_n = 0;
        s_status = 0;
        s_rounds = 0;
        s_neval = 15;
    }
    __syncthreads();
    // deterministic block sums of val and err over the live regions
    auto totals = [&](int n, double &V, double &E) {
        double v = 0, e = 0;
        for (int i = tid; i < n; i += nth) {
            v += lv[i];
            e += le[i];
        }
        for (int o = 16; o > 0; o >>= 1) {
            v += __shfl_down_sync(0xffffffffu, v, o);
            e += __shfl_down_sync(0xffffffffu, e, o);
        }
        if ((tid & 31) == 0) {
            s_red[0][tid >> 5] = v;
            s_red[1][tid >> 5] = e;
        }
        __syncthreads();
        V = 0;
        E = 0;
        for (int w = 0; w < nth / 32; ++w) {
            V += s_red[0][w];
            E += s_red[1][w];
        }
        __syncthreads();
    };
    while (true) {
        ev(s_nb, bc, bh, bv, be);
        __syncthreads();
        // the batch joins the live regions
        const int n0 = s_n, nb = s_nb;
        for (int b = tid; b < nb; b += nth) {
            lc[n0 + b] = bc[b];
            lh[n0 + b] = bh[b];
            lv[n0 + b] = bv[b];
            le[n0 + b] = be[b];
        }
        const int n = n0 + nb;
        __syncthreads();
        if (tid == 0) s_n = n;  // every thread has read n0 (barrier above)
        double hv, he;
        totals(n, hv, he);
        if (converged(he, hv)) break;
        // largest errors first
        int P2 = 1;
        while (P2 < n) P2 <<= 1;
        for (int i = tid; i < P2; i += nth) ord[i] = i;
        __syncthreads();
        for (int k = 2; k <= P2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = tid; t < P2; t += nth) {
                    const int u = t ^ j;
                    if (u > t) {
                        const int a = ord[t], b = ord[u];
                        // errors are >= 0: their bit patterns order as integers (integer
                        // compares; FP64 ones run at 1/64 of the FP32 rate)
                        const long long ka = a < n ? __double_as_longlong(le[a]) : -1ll;
                        const long long kb = b < n ? __double_as_longlong(le[b]) : -1ll;
                        // descending overall: the first half of each k-block descending
                        const bool desc = (t & k) == 0;
                        if (desc ? (ka < kb || (ka == kb && a > b)) : (ka > kb || (ka == kb && a < b))) {
                            ord[t] = b;
                            ord[u] = a;
                        }
                    }
                }
                __syncthreads();
            }
        if (tid == 0) {
            int K = 0;
            if (++s_rounds > PC_MAX_ROUNDS) {
                s_status = G3L_ERR_ROUNDS;
                s_done = 1;
            } else {
                double eErr = he;
                const double eVal = hv;
                do {
                    if (n + K + 1 > CAP) {  // live regions and children after this pop
                        s_status = G3L_ERR_POOL;
                        s_done = 1;
                        break;
                    }
                    eErr -= le[ord[K]];
                    ++K;
                    if (converged(eErr, eVal)) break;
                } while (K < n);
            }
            s_K = K;
        }
        __syncthreads();
        if (s_done) break;
        const int K = s_K;
        // children of the popped regions (cut, src/hcubature.cpp:206-218)
        for (int k = tid; k < K; k += nth) {
            const int r = ord[k];
            const double h2 = lh[r] * 0.5;
            bc[2 * k] = lc[r] - h2;
            bh[2 * k] = h2;
            bc[2 * k + 1] = lc[r] + h2;
            bh[2 * k + 1] = h2;
        }
        // the rest stays live (gathered through the batch's value arrays)
        const int m = n - K;
        for (int k = tid; k < m; k += nth) {
            const int r = ord[K + k];
            bv[k] = lc[r];
            bv[CAP + k] = lh[r];
            be[k] = lv[r];
            be[CAP + k] = le[r];
        }
        __syncthreads();
        for (int k = tid; k < m; k += nth) {
            lc[k] = bv[k];
            lh[k] = bv[CAP + k];
            lv[k] = be[k];
            le[k] = be[CAP + k];
        }
        if (tid == 0) {
            s_n = m;
            s_nb = 2 * K;
            s_neval += 30ull * (unsigned long long)K;
        }
        __syncthreads();
    }
    double V, E;
    totals(s_n, V, E);
    PcOut o{V, E, s_neval, s_status, s_rounds};
    __syncthreads();
    return o;
}

// The batch of one precompute integral: one region per half-warp, one point per lane.
struct PcEval {
    const PkDev &P;
    const PcTask &t;
    __device__ void operator()(int nb, const double *bc, const double *bh, double *bv,
                               double *be) const
    {
        const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x / 32;
        for (int r0 = 2 * warp; r0 < nb; r0 += 2 * nwarps) {
            const int r = r0 + half;
            double f = 0;
            if (r < nb && hl < 15) f = integrand(P, t, gk_point(bc[r], bh[r], hl));
            double vk[15];
#pragma unroll
            for (int k = 0; k < 15; ++k) vk[k] = __shfl_sync(0xffffffffu, f, k, 16);
            if (r < nb && hl == 0) rule_gk15(vk, bh[r], bv[r], be[r]);
        }
    }
};

// One block per integral at a time (grid-stride).  idx: the integrals to run (null:
// all ntask).
template <int CAP>
__global__ void __launch_bounds__(PC_THREADS) k_pc_integrate(const PkDev *__restrict__ Pp,
                                                             const PcTask *__restrict__ tasks,
                                                             const int *__restrict__ idx,
                                                             int ntask, PcOut *__restrict__ out)
{
    extern __shared__ double sm[];
    const PkDev P = *Pp;
    for (int tj = blockIdx.x; tj < ntask; tj += gridDim.x) {
        const int ti = idx ? idx[tj] : tj;
        const PcTask t = tasks[ti];
        const PcOut o = gk_integrate<CAP>(t.lo, t.hi, sm, PcEval{P, t});
        if (threadIdx.x == 0) out[ti] = o;
    }
}

// ------------------------------------------------------------------ n_bar(z) per HOD
// The galaxy number density of each HOD vector at every z bin, the reference's
// updateDensities (src/NNMap_Model.cu:244-297): n_bar(z) = ln10 * integral over
// log10 m of m n(m, z) (N_c + N_s) with the nearest mass bin of the FP64 mass function,
// each z bin one adaptive Gauss-Kronrod integral at rtol 1e-4
// (src/generalFunctions.cu:149-245, src/hcubature.cpp:620-765).
//
// The mass factors (m, N_c + N_s, mass bin) do not depend on z, and every region of
// every z bin is a node of the same bisection tree of [log10 mmin, log10 mmax'): depth
// d and index k, with half-width hw0 2^-d (exact) and the centre the cut arithmetic
// c -+ h/2 produces along the path from the root.  k_nbar_factors evaluates the factors
// of all 15 abscissae of every node down to depth NBAR_DEPTH, for every HOD vector of
// the call, spread over the whole device and reproducing that arithmetic bit for bit;
// the integrals then read them by node index and evaluate only deeper regions
// themselves.  Either way a factor is the same expression of the same abscissa.
constexpr int NBAR_DEPTH = 12;
constexpr int NBAR_NODES = (2 << NBAR_DEPTH) - 1;  // depths 0..NBAR_DEPTH
// Below depth NBAR_DEPTH the refinement follows the mass-bin edges (the nearest-bin
// lookup makes n(m, z) jump there; elsewhere the integrand is smooth): at every depth the
// two children of the node that contains an edge.  k_nbar_deep evaluates those, for the
// Nm - 1 edges and depths NBAR_DEPTH + 1 .. NBAR_DEEP, by the same path arithmetic.
constexpr int NBAR_DEEP = 44;
constexpr int NBAR_NDEEP = NBAR_DEEP - NBAR_DEPTH;

struct NbarTask {
    double lo, hi;
    int z_ix, hod;
};

struct NbarArgs {
    const double *hmf;   // FP64 mass function [Nz][Nm]
    const double *hods;  // [hod][6] f, alpha, Mth, sigma, M', beta
    int Nm;
    double mmin, ln_mratio;  // mass bin = round(log(m / mmin) Nm / ln_mratio)
    double lo, hi;           // integration range in log10 m
    double inv_hw0;          // 1 / root half-width
    // factors of node n of HOD h at abscissa i: [(h * NBAR_NODES + n) * 15 + i]
    double *fm, *fS;
    int *fmix;
    // deep nodes: edge e (e + 1 = the index whose bin starts there) at x = xm0 + (e + 0.5) dx,
    // depth NBAR_DEPTH + 1 + dd, side s: entry q = ((h * ne + e) * NBAR_NDEEP + dd) * 2 + s,
    // its node index at that depth dkey[q], factors [q * 15 + i]
    double xm0, dx, inv_dx;
    int ne;
    long long *dkey;
    double *dm, *dS;
    int *dmix;
};

constexpr size_t kNbarNodeBytes = 15 * (8 + 8 + 4);
constexpr size_t kNbarDeepBytes = 8 + kNbarNodeBytes;  // key + factors

// N_c + N_s (src/HOD.cu:35-76; erf taken once, the same argument in both) and the
// nearest mass bin (src/NNMap_Model.cu:556) at x = log10 m
__device__ __forceinline__ void nbar_factors(const NbarArgs &A, const double *h, double x,
                                             double &m, double &S, int &mix)
{
    m = pow(10.0, x);
    const double e = erf(log(m / h[2]) / h[3] / 1.414213562);
    const double Nc = 0.5 * h[1] * (1 + e);
    const double Ns = 0.5 * (1 + e) * pow(m / h[4], h[5]);
    S = Nc + Ns;
    mix = (int)round(log(m / A.mmin) * A.Nm / A.ln_mratio);
    mix = min(max(mix, 0), A.Nm - 1);  // in range for every abscissa of the interval
}

// centre and half-width of node n (heap numbering: root 0, children 2n+1 and 2n+2 the
// lower and upper half), by the cut arithmetic of the integrators (src/hcubature.cpp:
// 206-218): h2 = hw / 2, children c - h2 and c + h2
__device__ __forceinline__ void nbar_node(double lo, double hi, int n, double &c, double &hw)
{
    c = 0.5 * (lo + hi);
    hw = 0.5 * (hi - lo);
    int d = 31 - __clz(n + 1);  // depth
    for (int l = d - 1; l >= 0; --l) {
        const double h2 = hw * 0.5;
        c = (((n + 1) >> l) & 1) ? c + h2 : c - h2;
        hw = h2;
    }
}

// one thread per (HOD, node, abscissa)
__global__ void __launch_bounds__(256) k_nbar_factors(NbarArgs A, int nh)
{
    const long long total = (long long)nh * NBAR_NODES * 15;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % 15);
        const long long hn = t / 15;
        const int n = (int)(hn % NBAR_NODES), h = (int)(hn / NBAR_NODES);
        double c, hw;
        nbar_node(A.lo, A.hi, n, c, hw);
        double m, S;
        int mix;
        nbar_factors(A, A.hods + 6 * h, gk_point(c, hw, i), m, S, mix);
        A.fm[t] = m;
        A.fS[t] = S;
        A.fmix[t] = mix;
    }
}

// The 15-point Gauss-Kronrod value and QUADPACK error of rule_gk15, formed across the
// 16 lanes of a half-warp (lane i holds the value at abscissa i of gk_point's order;
// lane 15 holds nothing) instead of by one lane: the same sums in another order.
// Valid in lane 0 of the half-warp.
__device__ __forceinline__ void rule_gk15_hw(double f, int hl, double hw, double &val, double &err)
{
    // abscissa i: 0 centre, then pairs (2j+1, 2j+2): Gauss-Kronrod pair j (Kronrod-only
    // nodes for j = 0, 2, 4, 6 of cXgk; Gauss nodes for odd j)
    double wk = 0, wg = 0;
    if (hl == 0) {
        wk = cWgk[7];
        wg = cWg[3];
    } else if (hl < 7) {  // pairs j = 0..2: Gauss nodes cXgk[2j+1]
        const int j = (hl - 1) >> 1;
        wk = cWgk[2 * j + 1];
        wg = cWg[j];
    } else if (hl < 15) {  // pairs j = 3..6: Kronrod nodes cXgk[2(j-3)]
        const int j = (hl - 1) >> 1;
        wk = cWgk[2 * (j - 3)];
    }
    double rk = wk * f, rg = wg * f, ra = wk * fabs(f);
    for (int o = 8; o > 0; o >>= 1) {
        rk += __shfl_xor_sync(0xffffffffu, rk, o, 16);
        rg += __shfl_xor_sync(0xffffffffu, rg, o, 16);
        ra += __shfl_xor_sync(0xffffffffu, ra, o, 16);
    }
    const double mean = rk * 0.5;
    double rs = wk * fabs(f - mean);
    for (int o = 8; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o, 16);
    val = rk * hw;
    double e = fabs(rk - rg) * hw;
    const double rabs = ra * hw, rasc = rs * hw;
    if (rasc != 0 && e != 0) {
        const double scale = pow((200 * e / rasc), 1.5);
        e = (scale < 1) ? rasc * scale : rasc;
    }
    if (rabs > DBL_MIN / (50 * DBL_EPSILON)) {
        const double min_err = 50 * DBL_EPSILON * rabs;
        if (min_err > e) e = min_err;
    }
    err = e;
}

// one thread per (HOD, edge, depth, side, abscissa): walk from the root towards the edge
// (upper half when the edge is at or above the centre), then take the child on side s
__global__ void __launch_bounds__(256) k_nbar_deep(NbarArgs A, int nh)
{
    const long long total = (long long)nh * A.ne * NBAR_NDEEP * 2 * 15;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % 15);
        const long long q = t / 15;
        const int side = (int)(q & 1);
        const int dd = (int)((q >> 1) % NBAR_NDEEP);
        const long long he = (q >> 1) / NBAR_NDEEP;
        const int e = (int)(he % A.ne), h = (int)(he / A.ne);
        const double xe = A.xm0 + (e + 0.5) * A.dx;
        const int d = NBAR_DEPTH + 1 + dd;
        double c = 0.5 * (A.lo + A.hi), hw = 0.5 * (A.hi - A.lo);
        long long k = 0;
        for (int l = 1; l < d; ++l) {  // to the depth-(d-1) node containing the edge
            const double h2 = hw * 0.5;
            const bool up = xe >= c;
            c = up ? c + h2 : c - h2;
            hw = h2;
            k = 2 * k + (up ? 1 : 0);
        }
        const double h2 = hw * 0.5;
        c = side ? c + h2 : c - h2;
        hw = h2;
        k = 2 * k + side;
        double m, S;
        int mix;
        nbar_factors(A, A.hods + 6 * h, gk_point(c, hw, i), m, S, mix);
        A.dm[t] = m;
        A.dS[t] = S;
        A.dmix[t] = mix;
        if (i == 0) A.dkey[q] = k;
    }
}

// The batch of one n_bar integral: one region per half-warp, one point per lane.
struct NbarEval {
    const NbarArgs &A;
    const NbarTask &t;
    double hw0;  // root half-width
    __device__ void operator()(int nb, const double *bc, const double *bh, double *bv,
                               double *be) const
    {
        const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x / 32;
        const double *h = A.hods + 6 * t.hod;
        const double *row = A.hmf + (size_t)t.z_ix * A.Nm;
        for (int r0 = 2 * warp; r0 < nb; r0 += 2 * nwarps) {
            const int r = r0 + half;
            const bool live = r < nb;
            double f = 0;
            const double c = live ? bc[r] : 0.0, hw = live ? bh[r] : 1.0;
            if (live && hl < 15) {
                // node of the region: depth from the exponent of the exact half-width
                // hw0 2^-d, index from the centre (within a few ulp of lo + (2k + 1) hw):
                // k = floor((c - lo) / (2 hw)) with 1 / (2 hw) = 2^(d-1) / hw0
                const int d = (int)((__double_as_longlong(hw0) >> 52) & 0x7ff) -
                              (int)((__double_as_longlong(hw) >> 52) & 0x7ff);
                double m, S;
                int mix;
                bool have = false;
                if (d >= 0 && d <= NBAR_DEPTH) {
                    const long long k = (long long)floor((c - A.lo) * ldexp(A.inv_hw0, d - 1));
                    const long long n = (1ll << d) - 1 + k;
                    const size_t q = ((size_t)t.hod * NBAR_NODES + n) * 15 + hl;
                    m = A.fm[q];
                    S = A.fS[q];
                    mix = A.fmix[q];
                    have = true;
                } else if (d > NBAR_DEPTH && d <= NBAR_DEEP) {
                    // a node on the path to the nearest mass-bin edge, if it is one
                    const long long k = (long long)floor((c - A.lo) * ldexp(A.inv_hw0, d - 1));
                    const int e = (int)floor((c - A.xm0) * A.inv_dx);
                    if (e >= 0 && e < A.ne) {
                        const long long q =
                            (((long long)t.hod * A.ne + e) * NBAR_NDEEP + (d - NBAR_DEPTH - 1)) * 2 +
                            (k & 1);
                        if (A.dkey[q] == k) {
                            m = A.dm[q * 15 + hl];
                            S = A.dS[q * 15 + hl];
                            mix = A.dmix[q * 15 + hl];
                            have = true;
                        }
                    }
                }
                if (!have) nbar_factors(A, h, gk_point(c, hw, hl), m, S, mix);
                f = m * row[mix] * S;  // src/generalFunctions.cu:233-245
            }
            double v, e;
            rule_gk15_hw(f, hl, hw, v, e);
            if (live && hl == 0) {
                bv[r] = v;
                be[r] = e;
            }
        }
    }
};

// 16 warps per integral: the batch of a round (up to ~800 regions) takes a few passes
constexpr int NBAR_THREADS = 512;

template <int CAP>
__global__ void __launch_bounds__(NBAR_THREADS) k_nbar(NbarArgs A, const NbarTask *__restrict__ tasks,
                                                     const int *__restrict__ idx, int ntask,
                                                     PcOut *__restrict__ out)
{
    extern __shared__ double sm[];
    for (int tj = blockIdx.x; tj < ntask; tj += gridDim.x) {
        const int ti = idx ? idx[tj] : tj;
        const NbarTask t = tasks[ti];
        const PcOut o = gk_integrate_sorted<CAP>(t.lo, t.hi, sm, NbarEval{A, t, 0.5 * (t.hi - t.lo)});
        if (threadIdx.x == 0) out[ti] = o;
    }
}

// The tables from the integrals (one thread per (z, m/k) bin):
//   g, w, dwdz [N]; P_lin, conc, hmf, b_h [N*N], z-major.
struct TableArgs {
    int N, Ns, Nstar;
    const double *zs, *ms, *ks;         // grids [N]
    const double *gz;                   // growth(z)/growth(0) [N]
    const double *zsrc, *nzsrc;         // source n(z) [Ns]
    const PcOut *chi_z, *chi_src;       // comoving distances [N], [Ns]
    const PcOut *sig, *dsig, *sig_star; // [N*N], [N*N], [N*Nstar]
    const double *mstar_grid;           // [Nstar]
    double deltaZ;
    double *g, *w, *dwdz, *P_lin, *conc, *hmf, *b_h;
    int *mstar_ix;                      // [N]
};

__global__ void k_pc_zrow(const PkDev *__restrict__ Pp, TableArgs A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const PkDev P = *Pp;
    const double z = A.zs[i];
    // lensing efficiency (src/Cosmology.cpp:132-150)
    const double wz = A.chi_z[i].val;
    double r = 0;
    for (int j = 0; j < A.Ns; ++j) {
        const double zp = A.zsrc[j];
        const double wp = A.chi_src[j].val;
        if (zp >= z) r += A.nzsrc[j] * (wp - wz) / wp;
    }
    A.g[i] = r * A.deltaZ;
    A.w[i] = wz;
    A.dwdz[i] = kC / P.H0 / sqrt(E_of(P, z));  // src/Cosmology.cpp:101-104
    // M*(z): the first of the masses closest to sigma = delta_c (src/Powerspectrum.cpp:117-140)
    const double dc = delta_c(P, z);
    int best = 0;
    double bd = 0;
    for (int j = 0; j < A.Nstar; ++j) {
        const double s2 = A.sig_star[(size_t)i * A.Nstar + j].val / 2 / kPi / kPi;
        const double diff = dc - sqrt(s2);
        const double d = sqrt(diff * diff);
        if (j == 0 || d < bd) {
            bd = d;
            best = j;
        }
    }
    A.mstar_ix[i] = best;
}

__global__ void k_pc_table(const PkDev *__restrict__ Pp, TableArgs A)
{
    const int ij = blockIdx.x * blockDim.x + threadIdx.x;
    if (ij >= A.N * A.N) return;
    const int i = ij / A.N, j = ij % A.N;
    const PkDev P = *Pp;
    const double z = A.zs[i], m = A.ms[j];
    A.P_lin[ij] = spectrum(P, A.ks[j], A.gz[i]);
    const double mstar = A.mstar_grid[A.mstar_ix[i]];
    A.conc[ij] = 9 / (1. + z) * pow(m / mstar, -0.13);  // src/Powerspectrum.cpp:143-150
    // Sheth-Tormen n(m, z) and b_h (src/HMF.cpp:7-49)
    const double sigma2 = A.sig[ij].val / 2 / kPi / kPi;
    const double dsigma2 = A.dsig[ij].val / kPi / kPi;
    const double dc = delta_c(P, z);
    {
        const double Af = 0.322, q = 0.707, p = 0.3;
        const double rho_mean = Om_of(P, z) * P.rho_crit;
        const double nuSq = dc * dc / sigma2;
        A.hmf[ij] = -rho_mean / m / sigma2 * dsigma2 * Af * (1 + pow(q * nuSq, -p)) *
                    sqrt(q * nuSq / 2 / kPiTrunc) * exp(-0.5 * q * nuSq);
    }
    {
        const double q = 0.707, p = 0.3;
        A.b_h[ij] = 1 + 1. / dc * (q * dc * dc / sigma2 - 1 + 2 * p / (1 + pow(q * dc * dc / sigma2, p)));
    }
}

#define PC_CK(call)                                                                      \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            host::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
            return G3L_ERR_CUDA;                                                         \
        }                                                                                \
    } while (0)

// host-side Om(z), growth and the transfer-function parameters, with the reference's
// expressions (src/Cosmology.cpp:79-129, src/Powerspectrum.cpp:15-65)
double h_E(const PkDev &P, double z) { return P.Om * (1 + z) * (1 + z) * (1 + z) + P.OL; }
double h_Om(const PkDev &P, double z) { return P.Om * (1 + z) * (1 + z) * (1 + z) / h_E(P, z); }
double h_growth(const PkDev &P, double z)
{
    double om_m = h_Om(P, z);
    return 2.5 / (z + 1) * om_m / (std::pow(om_m, 4. / 7.) - P.OL + (1. + 0.5 * om_m) * (1 + P.OL / 70));
}

void transfer_parameters(PkDev &P, double Ob)
{
    const double h = P.H0 / 100;
    const double omhh = P.Om * h * h, obhh = Ob * h * h;
    P.omhh = omhh;
    P.obhh = obhh;
    const double f_baryon = obhh / omhh;
    const double Tcmb = 2.72548;
    const double theta_cmb = Tcmb / 2.7;
    const double theta_cmbSq = theta_cmb * theta_cmb;
    const double theta_cmb4 = theta_cmbSq * theta_cmbSq;
    const double z_equality = 2.50e4 * omhh / theta_cmb4;
    P.k_equality = 0.0746 * omhh / theta_cmbSq;
    const double z_drag_b1 = 0.313 * std::pow(omhh, -0.419) * (1.0 + 0.607 * std::pow(omhh, 0.674));
    const double z_drag_b2 = 0.238 * std::pow(omhh, 0.223);
    const double z_drag = 1291.0 * std::pow(omhh, 0.251) / (1.0 + 0.659 * std::pow(omhh, 0.828)) *
                          (1.0 + z_drag_b1 * std::pow(obhh, z_drag_b2));
    const double R_drag = 31.5 * obhh / (theta_cmb4) * (1000.0 / (1.0 + z_drag));
    const double R_equality = 31.5 * obhh / (theta_cmb4) * (1000.0 / z_equality);
    P.sound_horizon = 2.0 / 3.0 / P.k_equality * std::sqrt(6.0 / R_equality) *
                      std::log((std::sqrt(1.0 + R_drag) + std::sqrt(R_drag + R_equality)) /
                               (1.0 + std::sqrt(R_equality)));
    P.k_silk = 1.6 * std::pow(obhh, 0.52) * std::pow(omhh, 0.73) * (1.0 + std::pow(10.4 * omhh, -0.95));
    const double alpha_c_a1 = std::pow(46.9 * omhh, 0.670) * (1.0 + std::pow(32.1 * omhh, -0.532));
    const double alpha_c_a2 = std::pow(12.0 * omhh, 0.424) * (1.0 + std::pow(45.0 * omhh, -0.582));
    P.alpha_c = std::pow(alpha_c_a1, -f_baryon) * std::pow(alpha_c_a2, -std::pow(f_baryon, 3));
    const double beta_c_b1 = 0.944 / (1.0 + std::pow(458.0 * omhh, -0.708));
    const double beta_c_b2 = std::pow(0.395 * omhh, -0.0266);
    P.beta_c = 1.0 / (1.0 + beta_c_b1 * (std::pow(1.0 - f_baryon, beta_c_b2) - 1.0));
    const double y = z_equality / (1.0 + z_drag);
    const double alpha_b_G =
        y * (-6.0 * std::sqrt(1.0 + y) +
             (2.0 + 3.0 * y) * std::log((std::sqrt(1.0 + y) + 1.0) / (std::sqrt(1.0 + y) - 1.0)));
    P.alpha_b = 2.07 * P.k_equality * P.sound_horizon * std::pow(1.0 + R_drag, -0.75) * alpha_b_G;
    P.beta_node = 8.41 * std::pow(omhh, 0.435);
    P.beta_b = 0.5 + f_baryon + (3.0 - 2.0 * f_baryon) * std::sqrt(std::pow(17.2 * omhh, 2.0) + 1.0);
}

template <typename T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc((void **)&p, (n ? n : 1) * sizeof(T)); }
};

template <typename T>
cudaError_t upload(DevBuf<T> &b, const std::vector<T> &v, cudaStream_t s)
{
    cudaError_t e = b.alloc(v.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

int run_tasks(const PkDev *dP, const std::vector<PcTask> &tasks, std::vector<PcOut> &res,
              DevBuf<PcOut> &dres, cudaStream_t s, int nsm)
{
    DevBuf<PcTask> dt;
    PC_CK(upload(dt, tasks, s));
    PC_CK(dres.alloc(tasks.size()));
    const int n = (int)tasks.size();
    const char *fc = std::getenv("G3L_PC_FIRST_CAP");
    if (fc && std::atoi(fc) == PC_CAP_TINY)
        k_pc_integrate<PC_CAP_TINY><<<std::min(n, nsm * 8), PC_THREADS, pc_smem(PC_CAP_TINY), s>>>(
            dP, dt.p, nullptr, n, dres.p);
    else
        k_pc_integrate<PC_CAP_SMALL><<<std::min(n, nsm * 4), PC_THREADS, pc_smem(PC_CAP_SMALL),
                                       s>>>(dP, dt.p, nullptr, n, dres.p);
    PC_CK(cudaGetLastError());
    res.resize(n);
    PC_CK(cudaMemcpyAsync(res.data(), dres.p, n * sizeof(PcOut), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaStreamSynchronize(s));
    std::vector<int> big;
    for (int i = 0; i < n; ++i)
        if (res[i].status == G3L_ERR_POOL) big.push_back(i);
    if (!big.empty()) {
        DevBuf<int> di;
        PC_CK(upload(di, big, s));
        const int nb = (int)big.size();
        k_pc_integrate<PC_CAP_LARGE><<<std::min(nb, nsm), PC_THREADS, pc_smem(PC_CAP_LARGE), s>>>(
            dP, dt.p, di.p, nb, dres.p);
        PC_CK(cudaGetLastError());
        PC_CK(cudaMemcpyAsync(res.data(), dres.p, n * sizeof(PcOut), cudaMemcpyDeviceToHost, s));
        PC_CK(cudaStreamSynchronize(s));
    }
    for (const PcOut &o : res)
        if (o.status) {
            host::set_error(o.status == G3L_ERR_POOL
                                ? "g3l_precompute_tables: an integral needed more than 2048 regions"
                                : "g3l_precompute_tables: an integral exceeded 4096 rounds");
            return o.status;
        }
    return G3L_OK;
}

}  // namespace

namespace host {

void free_nbar_device(NbarDevice &W)
{
    for (void *p : {W.tasks, W.out, W.idx, W.cache, (void *)W.hods})
        if (p) cudaFree(p);
    W = NbarDevice{};
}

namespace {
constexpr int kNbarChunk = 64;  // HOD vectors per launch (157 MB of factor tables)
constexpr int kNbarCapSmall = 1024;      // live regions of the first pass
}  // namespace

int n_bar_device(NbarDevice &W, const Binning &B, const double *d_hmf, const double *hods,
                 int nh, void *stream, int nsm, double *out)
{
    cudaStream_t s = (cudaStream_t)stream;
    const int Nz = B.Nz;
    const double lo = std::log10(B.mmin), hi = std::log10(B.mmax_integral());
    const double ln10 = std::log(10.0);
    PC_CK(cudaFuncSetAttribute(k_nbar<kNbarCapSmall>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbar_smem(kNbarCapSmall)));
    PC_CK(cudaFuncSetAttribute(k_nbar<PC_CAP_LARGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbar_smem(PC_CAP_LARGE)));
    std::vector<NbarTask> tasks;
    std::vector<PcOut> res;
    std::vector<int> big;
    for (int h0 = 0; h0 < nh; h0 += kNbarChunk) {
        const int nk = std::min(kNbarChunk, nh - h0);
        const int ntask = nk * Nz;
        tasks.resize(ntask);
        for (int k = 0; k < nk; ++k)
            for (int i = 0; i < Nz; ++i) {
                const double z = B.zmin + i * (B.zmax - B.zmin) / B.Nz;
                const int z_ix = (int)std::round((z - B.zmin) * B.Nz / (B.zmax - B.zmin));
                tasks[(size_t)k * Nz + i] = NbarTask{lo, hi, z_ix, k};
            }
        if ((size_t)ntask > W.ntask_cap) {
            for (void **p : {&W.tasks, &W.out, &W.idx})
                if (*p) cudaFree(*p), *p = nullptr;
            W.ntask_cap = 0;
            PC_CK(cudaMalloc(&W.tasks, sizeof(NbarTask) * ntask));
            PC_CK(cudaMalloc(&W.out, sizeof(PcOut) * ntask));
            PC_CK(cudaMalloc(&W.idx, sizeof(int) * ntask));
            W.ntask_cap = (size_t)ntask;
        }
        if ((size_t)nk > W.nhod_cap) {  // HOD vectors and their factor tables
            if (W.hods) cudaFree(W.hods);
            if (W.cache) cudaFree(W.cache);
            W.hods = nullptr;
            W.cache = nullptr;
            W.nhod_cap = 0;
            PC_CK(cudaMalloc((void **)&W.hods, sizeof(double) * 6 * nk));
            PC_CK(cudaMalloc(&W.cache, (size_t)nk * (NBAR_NODES * kNbarNodeBytes +
                                                     (size_t)(B.Nm - 1) * NBAR_NDEEP * 2 *
                                                         kNbarDeepBytes) +
                                   8));  // + alignment of the deep keys
            W.nhod_cap = (size_t)nk;
        }
        const size_t E = (size_t)W.nhod_cap * NBAR_NODES * 15;
        NbarArgs A{};
        A.hmf = d_hmf;
        A.hods = W.hods;
        A.Nm = B.Nm;
        A.mmin = B.mmin;
        A.ln_mratio = std::log(B.mmax / B.mmin);
        A.lo = lo;
        A.hi = hi;
        A.inv_hw0 = 1.0 / (0.5 * (hi - lo));
        A.fm = (double *)W.cache;
        A.fS = A.fm + E;
        A.fmix = (int *)(A.fS + E);
        // deep nodes along the mass-bin edges
        A.xm0 = std::log10(B.mmin);
        A.dx = std::log(B.mmax / B.mmin) / (std::log(10.0) * B.Nm);
        A.inv_dx = 1 / A.dx;
        A.ne = B.Nm - 1;
        const size_t E2 = (size_t)W.nhod_cap * A.ne * NBAR_NDEEP * 2;
        A.dkey = (long long *)(A.fmix + E + (E & 1));  // 8-byte aligned
        A.dm = (double *)(A.dkey + E2);
        A.dS = A.dm + E2 * 15;
        A.dmix = (int *)(A.dS + E2 * 15);
        PC_CK(cudaMemcpyAsync(W.tasks, tasks.data(), sizeof(NbarTask) * ntask,
                              cudaMemcpyHostToDevice, s));
        PC_CK(cudaMemcpyAsync(W.hods, hods + (size_t)6 * h0, sizeof(double) * 6 * nk,
                              cudaMemcpyHostToDevice, s));
        {
            const long long nthr = (long long)nk * NBAR_NODES * 15;
            const int grid = (int)std::min<long long>((nthr + 255) / 256, (long long)nsm * 16);
            k_nbar_factors<<<grid, 256, 0, s>>>(A, nk);
            PC_CK(cudaGetLastError());
            const long long nthr2 = (long long)nk * A.ne * NBAR_NDEEP * 2 * 15;
            const int grid2 = (int)std::min<long long>((nthr2 + 255) / 256, (long long)nsm * 16);
            if (nthr2 > 0) k_nbar_deep<<<grid2, 256, 0, s>>>(A, nk);
            PC_CK(cudaGetLastError());
        }
        k_nbar<kNbarCapSmall><<<std::min(ntask, nsm * 2), NBAR_THREADS, nbar_smem(kNbarCapSmall), s>>>(
            A, (const NbarTask *)W.tasks, nullptr, ntask, (PcOut *)W.out);
        PC_CK(cudaGetLastError());
        res.resize(ntask);
        PC_CK(cudaMemcpyAsync(res.data(), W.out, sizeof(PcOut) * ntask, cudaMemcpyDeviceToHost, s));
        PC_CK(cudaStreamSynchronize(s));
        big.clear();
        for (int i = 0; i < ntask; ++i)
            if (res[i].status == G3L_ERR_POOL) big.push_back(i);
        if (!big.empty()) {  // the rest with the larger heap, from their root regions
            const int nb = (int)big.size();
            PC_CK(cudaMemcpyAsync(W.idx, big.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
            k_nbar<PC_CAP_LARGE><<<std::min(nb, nsm), NBAR_THREADS, nbar_smem(PC_CAP_LARGE), s>>>(
                A, (const NbarTask *)W.tasks, (const int *)W.idx, nb, (PcOut *)W.out);
            PC_CK(cudaGetLastError());
            PC_CK(cudaMemcpyAsync(res.data(), W.out, sizeof(PcOut) * ntask, cudaMemcpyDeviceToHost,
                                  s));
            PC_CK(cudaStreamSynchronize(s));
        }
        for (int i = 0; i < ntask; ++i) {
            if (res[i].status) {
                set_error(res[i].status == G3L_ERR_POOL
                              ? "n_bar: an integral needed more than 2048 regions"
                              : "n_bar: an integral exceeded 4096 rounds");
                return res[i].status;
            }
            out[(size_t)h0 * Nz + i] = ln10 * res[i].val;
        }
    }
    return G3L_OK;
}

}  // namespace host
}  // namespace g3l

using namespace g3l;

namespace {
int precompute_impl(const g3l_precompute_in *in, int device, g3l_precompute_out *out);
}

extern "C" int g3l_precompute_tables(const g3l_precompute_in *in, int device,
                                     g3l_precompute_out *out)
{
    try {
        return precompute_impl(in, device, out);
    } catch (const std::bad_alloc &) {
        host::set_error("g3l_precompute_tables: host allocation failed");
        return G3L_ERR_NOMEM;
    } catch (...) {
        host::set_error("g3l_precompute_tables: unexpected host error");
        return G3L_ERR_INVALID;
    }
}

namespace {
int precompute_impl(const g3l_precompute_in *in, int device, g3l_precompute_out *out)
{
    if (!in || !out || in->nbins < 1 || in->nbins > 4096 || in->n_nz < 1 ||
        in->n_nz > (1 << 22) || !in->nz_z || !in->nz_v ||
        !(in->mmin > 0 && in->mmax > in->mmin && in->kmin > 0 && in->kmax > in->kmin &&
          in->zmax > in->zmin && in->zmin >= 0) ||
        !out->g || !out->w || !out->dwdz || !out->P_lin || !out->conc || !out->hmf || !out->b_h) {
        host::set_error("g3l_precompute_tables: invalid arguments");
        return G3L_ERR_INVALID;
    }
    for (int k = 0; k < 6; ++k)
        if (!std::isfinite(in->cosmo[k])) {
            host::set_error("g3l_precompute_tables: non-finite cosmology");
            return G3L_ERR_INVALID;
        }
    PC_CK(cudaSetDevice(device));
    int nsm = 0;
    PC_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    PC_CK(cudaFuncSetAttribute(k_pc_integrate<PC_CAP_SMALL>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pc_smem(PC_CAP_SMALL)));
    PC_CK(cudaFuncSetAttribute(k_pc_integrate<PC_CAP_LARGE>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pc_smem(PC_CAP_LARGE)));
    cudaStream_t s;
    PC_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    cudaEvent_t e0, e1;
    PC_CK(cudaEventCreate(&e0));
    PC_CK(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard()
        {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } eg{e0, e1};
    PC_CK(cudaEventRecord(e0, s));

    const int N = in->nbins, Ns = in->n_nz, Nstar = 256;
    PkDev P{};
    P.Om = in->cosmo[0];
    P.OL = in->cosmo[1];
    P.H0 = in->cosmo[4];
    P.ns = in->cosmo[5];
    P.rho_crit = 3 * P.H0 * P.H0 * 3.086e19 / 8 / kPiTrunc / 1.327e11;  // src/Cosmology.h:41-47
    transfer_parameters(P, in->cosmo[2]);
    // grids (src/doPrecomputations.cpp:43-54) and M*'s mass grid (src/Powerspectrum.cpp:122-131)
    const double z_bin = (in->zmax - in->zmin) / N, m_bin = std::log(in->mmax / in->mmin) / N,
                 k_bin = std::log(in->kmax / in->kmin) / N;
    std::vector<double> zs(N), ms(N), ks(N), gzs(N), mst(Nstar);
    for (int i = 0; i < N; ++i) {
        zs[i] = in->zmin + i * z_bin;
        ms[i] = std::exp(std::log(in->mmin) + m_bin * i);
        ks[i] = std::exp(std::log(in->kmin) + k_bin * i);
        gzs[i] = h_growth(P, zs[i]) / h_growth(P, 0.0);
    }
    const double ms_bin = std::log(1e18 / 1e10) / Nstar;
    for (int j = 0; j < Nstar; ++j) mst[j] = std::exp(std::log(1e10) + ms_bin * j);

    // pass 1: the amplitude (src/Powerspectrum.cpp:67-77) and the comoving distances
    std::vector<PcTask> t1;
    t1.push_back(PcTask{PC_AMP, 0, 0, 0, 0, 0.0, 1e12});
    for (int i = 0; i < N; ++i) t1.push_back(PcTask{PC_CHI, 0, 0, 0, 0, 0.0, zs[i]});
    for (int j = 0; j < Ns; ++j) t1.push_back(PcTask{PC_CHI, 0, 0, 0, 0, 0.0, in->nz_z[j]});
    DevBuf<PkDev> dP;
    PC_CK(dP.alloc(1));
    PC_CK(cudaMemcpyAsync(dP.p, &P, sizeof P, cudaMemcpyHostToDevice, s));
    std::vector<PcOut> r1;
    DevBuf<PcOut> dr1;
    int st = run_tasks(dP.p, t1, r1, dr1, s, nsm);
    if (st) return st;
    const double factor = kPi * in->cosmo[3];
    P.amplitude = 2 * factor * factor / r1[0].val;
    PC_CK(cudaMemcpyAsync(dP.p, &P, sizeof P, cudaMemcpyHostToDevice, s));

    // pass 2: sigma^2 and dsigma^2/dm at every (z, m), sigma^2 on M*'s grid
    // (radii: src/Powerspectrum.cpp:201-202, 249-251)
    std::vector<PcTask> t2;
    t2.reserve((size_t)N * (2 * N + Nstar));
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            const double om = h_Om(P, zs[i]);
            t2.push_back(PcTask{PC_SIGMA2, 0, std::pow(0.75 / kPi * ms[j] / P.rho_crit / om, 1. / 3.),
                                0, gzs[i], 0.0, 1e12});
        }
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            const double rho_m = P.rho_crit * h_Om(P, zs[i]);
            t2.push_back(PcTask{PC_DSIGMA2, 0, 0.6204 * std::pow(ms[j] / rho_m, 1. / 3.),
                                0.2068 * std::pow(rho_m * ms[j] * ms[j], -1. / 3.), gzs[i], 0.0,
                                1e12});
        }
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < Nstar; ++j) {
            const double om = h_Om(P, zs[i]);
            t2.push_back(PcTask{PC_SIGMA2, 0, std::pow(0.75 / kPi * mst[j] / P.rho_crit / om, 1. / 3.),
                                0, gzs[i], 0.0, 1e12});
        }
    std::vector<PcOut> r2;
    DevBuf<PcOut> dr2;
    st = run_tasks(dP.p, t2, r2, dr2, s, nsm);
    if (st) return st;

    // the tables
    DevBuf<double> dzs, dms, dks, dgz, dzsrc, dnz, dmst, dg, dw, ddw, dpl, dcn, dhm, dbh;
    DevBuf<int> dmix;
    PC_CK(upload(dzs, zs, s));
    PC_CK(upload(dms, ms, s));
    PC_CK(upload(dks, ks, s));
    PC_CK(upload(dgz, gzs, s));
    PC_CK(upload(dzsrc, std::vector<double>(in->nz_z, in->nz_z + Ns), s));
    PC_CK(upload(dnz, std::vector<double>(in->nz_v, in->nz_v + Ns), s));
    PC_CK(upload(dmst, mst, s));
    const size_t NN = (size_t)N * N;
    PC_CK(dg.alloc(N));
    PC_CK(dw.alloc(N));
    PC_CK(ddw.alloc(N));
    PC_CK(dpl.alloc(NN));
    PC_CK(dcn.alloc(NN));
    PC_CK(dhm.alloc(NN));
    PC_CK(dbh.alloc(NN));
    PC_CK(dmix.alloc(N));
    TableArgs A{};
    A.N = N;
    A.Ns = Ns;
    A.Nstar = Nstar;
    A.zs = dzs.p;
    A.ms = dms.p;
    A.ks = dks.p;
    A.gz = dgz.p;
    A.zsrc = dzsrc.p;
    A.nzsrc = dnz.p;
    A.chi_z = dr1.p + 1;
    A.chi_src = dr1.p + 1 + N;
    A.sig = dr2.p;
    A.dsig = dr2.p + NN;
    A.sig_star = dr2.p + 2 * NN;
    A.mstar_grid = dmst.p;
    A.deltaZ = (in->nz_z[Ns - 1] - in->nz_z[0]) / Ns;  // src/Cosmology.cpp:137
    A.g = dg.p;
    A.w = dw.p;
    A.dwdz = ddw.p;
    A.P_lin = dpl.p;
    A.conc = dcn.p;
    A.hmf = dhm.p;
    A.b_h = dbh.p;
    A.mstar_ix = dmix.p;
    k_pc_zrow<<<(N + 127) / 128, 128, 0, s>>>(dP.p, A);
    PC_CK(cudaGetLastError());
    k_pc_table<<<(int)((NN + 127) / 128), 128, 0, s>>>(dP.p, A);
    PC_CK(cudaGetLastError());
    PC_CK(cudaEventRecord(e1, s));
    PC_CK(cudaMemcpyAsync(out->g, dg.p, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->w, dw.p, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->dwdz, ddw.p, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->P_lin, dpl.p, NN * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->conc, dcn.p, NN * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->hmf, dhm.p, NN * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaMemcpyAsync(out->b_h, dbh.p, NN * sizeof(double), cudaMemcpyDeviceToHost, s));
    PC_CK(cudaStreamSynchronize(s));
    float ms_ = 0;
    PC_CK(cudaEventElapsedTime(&ms_, e0, e1));
    out->device_ms = ms_;
    out->amplitude = P.amplitude;
    out->integrals = (long long)(t1.size() + t2.size());
    unsigned long long ne = 0;
    for (const PcOut &o : r1) ne += o.neval;
    for (const PcOut &o : r2) ne += o.neval;
    out->points = (long long)ne;
    return G3L_OK;
}
}  // namespace
