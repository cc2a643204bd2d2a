#pragma once
// evalmx_impl.cuh -- mixed-precision rule evaluation: FP32 integrand, wide accumulation
// (instantiated in evalmx_k0.cu and evalmx_k1.cu).
//
// Same work decomposition as eval_fp64.cu (one warp cuts one parent region and
// applies the Genz-Malik 7/5 rule to both children), with the arithmetic
// rearranged for a GPU whose FP64 rate is ~1/60 of its FP32 rate:
//  * Region centres stay FP64 in HBM; each is split into a double-float with
//    integer operations, and the 7 coordinate variants c, c-+lambda h of every
//    dimension are formed as double-floats (~48-bit mantissas).
//  * Every quantity that depends on one coordinate is computed once per child:
//    10^x, aperture filters of l1 and l2, HOD occupations, the z-dependent
//    factors, and the nearest-bin / truncated indices of z and m.  Indices come
//    from the double-float argument; within 1e-7 of a rounding boundary the
//    exact index is taken from the host table of tie-prone centre values, or
//    computed with the reference's FP64 expression.
//  * The integrand is FP32 in scaled units (l / 1e3, m / 1e12, tables scaled to
//    O(1)); the constant scale is folded into the region volume on the host, so
//    region values and errors are stored unscaled in FP64.
//  * The NFW profile uses a cancellation-free form of the Si/Ci differences:
//    ln(a2/a1) = ln(1+c) replaces the two logarithms of the small-argument Ci,
//    and for a1 >= 4 the numerator collapses to
//    g(a1) - g(a2) cos(a1 c) + (f(a2) - 1/a2) sin(a1 c) with f(x) - 1/x
//    evaluated from the difference polynomial.  An FP64 branch remains for
//    a1 below a threshold (option; counted).
//  * The u_NFW calls that depend on one l, one mass and z only are evaluated once
//    per distinct (l, m, z) variant combination of the work item (at most 33 per
//    child, against 93-241 points) and read by the points.
//  * Rule sums, fourth differences and the 7th/5th-degree combination are
//    double-float; the final value and error are formed in FP64 by four lanes
//    at once.
#include "dfloat.cuh"
#include "g3l_device.cuh"
#include "phys64.cuh"

namespace g3l {

constexpr float HALF_PI_F = 1.57079632679489662f;
constexpr float GAMMA_F = 0.5772156649f;

struct SlotF {
    float f[6];
    int i0, i1;
};

// ---------------------------------------------------------------- Si / Ci (FP32)
// Rowe et al. (2015) rational approximations (the reference's SiCi,
// src/generalFunctions.cu:44-87) in Horner form.  Small x (< 4): Si = x P(x^2)/Q(x^2),
// Ci = gamma + ln x + x^2 R(x^2)/S(x^2).  Large x: Si = pi/2 - f cos x - g sin x,
// Ci = f sin x - g cos x with f = (1/x) A(t)/B(t), g = t C(t)/D(t), t = 1/x^2.
__device__ __forceinline__ float si_small(float x)
{
    float t = x * x;
    float p = -6.05338212010422477e-16f;
    p = fmaf(p, t, 7.08240282274875911e-13f);
    p = fmaf(p, t, -3.53201978997168357e-10f);
    p = fmaf(p, t, 9.43280809438713025e-8f);
    p = fmaf(p, t, -1.41018536821330254e-5f);
    p = fmaf(p, t, 1.15457225751016682e-3f);
    p = fmaf(p, t, -4.54393409816329991e-2f);
    p = fmaf(p, t, 1.0f);
    float q = 3.21107051193712168e-16f;
    q = fmaf(q, t, 4.5049097575386581e-13f);
    q = fmaf(q, t, 3.28067571055789734e-10f);
    q = fmaf(q, t, 1.55654986308745614e-7f);
    q = fmaf(q, t, 4.99175116169755106e-5f);
    q = fmaf(q, t, 1.01162145739225565e-2f);
    q = fmaf(q, t, 1.0f);
    return x * __fdividef(p, q);
}

// x^2 R(x^2)/S(x^2): the non-logarithmic part of the small-argument Ci
__device__ __forceinline__ float ci_small_poly(float x)
{
    float t = x * x;
    float p = -9.93728488857585407e-15f;
    p = fmaf(p, t, 1.06480802891189243e-11f);
    p = fmaf(p, t, -4.68889508144848019e-9f);
    p = fmaf(p, t, 1.05297363846239184e-6f);
    p = fmaf(p, t, -1.27528342240267686e-4f);
    p = fmaf(p, t, 7.51851524438898291e-3f);
    p = fmaf(p, t, -0.25f);
    float q = 1.39759616731376855e-18f;
    q = fmaf(q, t, 1.89106054713059759e-15f);
    q = fmaf(q, t, 1.38536352772778619e-12f);
    q = fmaf(q, t, 6.97071295760958946e-10f);
    q = fmaf(q, t, 2.55533277086129636e-7f);
    q = fmaf(q, t, 6.72126800814254432e-5f);
    q = fmaf(q, t, 1.1592605689110735e-2f);
    q = fmaf(q, t, 1.0f);
    return t * __fdividef(p, q);
}

// f(x), g(x) and f(x) - 1/x for x >= 4
__device__ __forceinline__ void fg_large(float x, float &f, float &g, float &fm)
{
    float ix = __frcp_rn(x);
    float t = ix * ix;
    // A(t) and B(t) of f
    float a = -4.94701168645415959931e11f;
    a = fmaf(a, t, 4.94816688199951963482e12f);
    a = fmaf(a, t, 1.00795182980368574617e13f);
    a = fmaf(a, t, 4.20968180571076940208e12f);
    a = fmaf(a, t, 6.40533830574022022911e11f);
    a = fmaf(a, t, 4.33736238870432522765e10f);
    a = fmaf(a, t, 1.43073403821274636888e9f);
    a = fmaf(a, t, 2.37750310125431834034e7f);
    a = fmaf(a, t, 1.96396372895146869801e5f);
    a = fmaf(a, t, 7.44437068161936700618e2f);
    a = fmaf(a, t, 1.0f);
    float b = 1.11535493509914254097e13f;
    b = fmaf(b, t, 1.43468549171581016479e13f);
    b = fmaf(b, t, 5.06084464593475076774e12f);
    b = fmaf(b, t, 7.08501308149515401563e11f);
    b = fmaf(b, t, 4.58595115847765779830e10f);
    b = fmaf(b, t, 1.47478952192985464958e9f);
    b = fmaf(b, t, 2.41535670165126845144e7f);
    b = fmaf(b, t, 1.97865247031583951450e5f);
    b = fmaf(b, t, 7.46437068161927678031e2f);
    b = fmaf(b, t, 1.0f);
    // A - B, coefficient-wise (exact differences of the published values, rounded)
    float dab = -4.94701168645415954590e11f;
    dab = fmaf(dab, t, -6.20538246899190625000e12f);
    dab = fmaf(dab, t, -4.26733661912124414062e12f);
    dab = fmaf(dab, t, -8.51162840223981323242e11f);
    dab = fmaf(dab, t, -6.79674775754933776855e10f);
    dab = fmaf(dab, t, -2.48588769773332548141e9f);
    dab = fmaf(dab, t, -4.40554837171082794666e7f);
    dab = fmaf(dab, t, -3.78536003969501121901e5f);
    dab = fmaf(dab, t, -1.46887413643708168820e3f);
    dab = fmaf(dab, t, -1.99999999999097743952f);
    dab = dab * t;
    float ib = __frcp_rn(b);
    f = a * ib * ix;
    fm = dab * ib * ix;
    float c = -1.36517137670871689e12f;
    c = fmaf(c, t, 6.43291613143049485e12f);
    c = fmaf(c, t, 1.81004487464664575e13f);
    c = fmaf(c, t, 7.57664583257834349e12f);
    c = fmaf(c, t, 1.09049528450362786e12f);
    c = fmaf(c, t, 6.83052205423625007e10f);
    c = fmaf(c, t, 2.06297595146763354e9f);
    c = fmaf(c, t, 3.12557570795778731e7f);
    c = fmaf(c, t, 2.35239181626478200e5f);
    c = fmaf(c, t, 8.1359520115168615e2f);
    c = fmaf(c, t, 1.0f);
    float d = 3.99653257887490811e13f;
    d = fmaf(d, t, 4.01839087307656620e13f);
    d = fmaf(d, t, 1.17164723371736605e13f);
    d = fmaf(d, t, 1.39866710696414565e12f);
    d = fmaf(d, t, 7.87465017341829930e10f);
    d = fmaf(d, t, 2.23355543278099360e9f);
    d = fmaf(d, t, 3.26026661647090822e7f);
    d = fmaf(d, t, 2.40036752835578777e5f);
    d = fmaf(d, t, 8.19595201151451564e2f);
    d = fmaf(d, t, 1.0f);
    g = t * __fdividef(c, d);
}

// The FP64 form of u_nfw32 for a1 = kr / c below the small-argument threshold, where the
// Si/Ci differences cancel.  Kept out of line: it is rare, and inlined in every call
// site it would crowd the instruction cache of the rule kernels.
static __device__ __noinline__ float u_nfw_small64(float kr, float c)
{
    const double cd = (double)c;
    const double a1d = (double)kr / cd;
    const double a2d = a1d * (1 + cd);
    double si1, ci1, si2, ci2, s1, c1;
    sici64_sc(a1d, si1, ci1, s1, c1);
    sici64(a2d, si2, ci2);
    double num = s1 * (si2 - si1) + c1 * (ci2 - ci1) - sin(a1d * cd) / a2d;
    return (float)(num / (log(1. + cd) - cd / (1. + cd)));
}

// NFW profile u(k, m) from kr = k r_200 and c = f conc; a1 = kr / c, a2 = a1 (1 + c),
// a1 c = kr.  Returns the FP32 value; lanes with a1 < small_arg take the FP64 form.
// The Si/Ci parts of a1 and a2 (a1 < a2) come from one loop body, small-argument form
// below 4 and auxiliary functions f, g above, so the code holds each form once; and the
// function is one out-of-line copy for all its call sites.  The rule kernels are bound by
// instruction fetch, not by the call: measured 5-15% faster than inlined.
static __device__ __noinline__ float u_nfw32(float kr, float c, float small_arg, int &small_hits)
{
    if (!(kr > 0.f)) return 1.f;  // k -> 0 limit of the profile
    const float opc = 1.f + c;
    const float a1 = __fdividef(kr, c);
    const float a2 = a1 * opc;
    const float lnopc = log1pf(c);
    const float F = lnopc - __fdividef(c, opc);
    if (a1 < small_arg) {
        ++small_hits;
        return u_nfw_small64(kr, c);
    }
    float s1, c1, sk, ck;
    sincosf(a1, &s1, &c1);
    sincosf(kr, &sk, &ck);
    // (a, b, e) of a1 and of a2: small form (Si, Ci polynomial, 0) below 4, else
    // (f, g, f - 1/x)
    float a1a = 0.f, a1b = 0.f, a2a = 0.f, a2b = 0.f, a2e = 0.f;
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        const float x = q ? a2 : a1;
        float a, b, e;
        if (x < 4.f) {
            a = si_small(x);
            b = ci_small_poly(x);
            e = 0.f;
        } else {
            fg_large(x, a, b, e);
        }
        if (q == 0) {
            a1a = a;
            a1b = b;
        } else {
            a2a = a;
            a2b = b;
            a2e = e;
        }
    }
    float N;
    if (a2 < 4.f) {
        const float dS = a2a - a1a;
        const float dC = lnopc + (a2b - a1b);
        N = s1 * dS + c1 * dC - __fdividef(sk, a2);
    } else if (a1 >= 4.f) {
        N = a1b - a2b * ck + a2e * sk;  // g(a1) - g(a2) cos(kr) + (f(a2) - 1/a2) sin(kr)
    } else {
        const float f2 = a2a, g2 = a2b;
        const float s2 = s1 * ck + c1 * sk;  // sin(a1 + a1 c)
        const float c2 = c1 * ck - s1 * sk;
        const float Si2 = HALF_PI_F - f2 * c2 - g2 * s2;
        const float Ci2 = f2 * s2 - g2 * c2;
        const float Si1 = a1a;
        const float Ci1 = GAMMA_F + __logf(a1) + a1b;
        N = s1 * (Si2 - Si1) + c1 * (Ci2 - Ci1) - __fdividef(sk, a2);
    }
    return __fdividef(N, F);
}

__device__ __forceinline__ float aperture32(float eta)
{
    const float e2 = eta * eta;
    return 0.5f * e2 * __expf(-0.5f * e2);
}

// nearest-bin / truncated index from a double-float argument
__device__ __forceinline__ bool idx_df(df a, int N, float tol, int &ir, int &it)
{
    float fl = floorf(a.hi);
    float fr = (a.hi - fl) + a.lo;
    if (fr < 0.f) {
        fl -= 1.f;
        fr += 1.f;
    } else if (fr >= 1.f) {
        fl += 1.f;
        fr -= 1.f;
    }
    const bool near = fabsf(fr - 0.5f) < tol || fr < tol || fr > 1.f - tol;
    int b = (int)fl;
    ir = min(max(b + (fr > 0.5f ? 1 : 0), 0), N - 1);
    it = min(max(b, 0), N - 1);
    return near;
}

__device__ __forceinline__ bool tie_lookup(const unsigned long long *bits, const int *ro,
                                           const int *tr, int n, double x, int &ir, int &it)
{
    const unsigned long long key = (unsigned long long)__double_as_longlong(x);
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        unsigned long long b = bits[mid];
        if (b == key) {
            ir = ro[mid];
            it = tr[mid];
            return true;
        }
        if (b < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return false;
}

constexpr float IDX_TOL = 1e-7f;   // double-float index arguments
constexpr float K3_TOL = 3e-5f;    // FP32 argument of the l3-based k index

// P_lin (scaled) at k = ls * kw with the small-k extrapolation (src/NNMap_Model.cu:819-839)
__device__ __forceinline__ float plin32(const DevTables &T, int zr, int kix, float k)
{
    if (kix >= 0) {
        if (T.clamp_k && kix > T.Nk - 1) kix = T.Nk - 1;
        long long flat = (long long)zr * T.Nk + kix;
        const long long last = (long long)T.Nz * T.Nk - 1;
        return __ldg(T.f_plin + (flat > last ? last : flat));
    }
    return __ldg(T.f_plin + zr * T.Nk) * (k / (float)T.kmin);
}

// exact (reference-expression) k index, used when the estimate sits on a boundary
__device__ __forceinline__ int kix_exact64(const DevTables &T, double k)
{
    return (int)round(log(k / T.kmin) * T.Nk / T.ln_kratio);
}

// signed nearest index of a double-float argument; near = within tol of a .5 boundary
__device__ __forceinline__ int round_df(df a, float tol, bool &near)
{
    float fl = floorf(a.hi);
    float fr = (a.hi - fl) + a.lo;
    if (fr < 0.f) {
        fl -= 1.f;
        fr += 1.f;
    } else if (fr >= 1.f) {
        fl += 1.f;
        fr -= 1.f;
    }
    near = fabsf(fr - 0.5f) < tol;
    return (int)fl + (fr > 0.5f ? 1 : 0);
}

// double-float natural log of a positive float: exponent part exact, mantissa by logf
__device__ __forceinline__ df ln_df(float v)
{
    int e;
    const float m = frexpf(v, &e);  // v = m 2^e, m in [0.5, 1)
    const df el = df_mul_f({0.693147182464599609375f, -1.904654323148236017e-09f}, (float)e);
    return df_add_f(el, logf(m));
}

// Exact nearest-bin / truncated indices for arguments within IDX_TOL of a rounding
// boundary: the tie table for the dyadic centre values (v == 0), else the reference's FP64
// expression (src/NNMap_Model.cu:555-556, 796-799).  Out of line, like the k indices
// below: they are rare, and their FP64 code would otherwise crowd the rule kernels'
// instruction cache.  Return 1 when the FP64 expression was evaluated (counted).
static __device__ __noinline__ int m_index_exact(const DevTables &T, double x64, int v, int &ir, int &it)
{
    if (v == 0 && tie_lookup(T.tie_m_bits, T.tie_m_round, T.tie_m_trunc, T.n_tie_m, x64, ir, it))
        return 0;
    double m = pow(10.0, x64);
    double ar = log(m / T.mmin) * T.Nm / T.ln_mratio;
    ir = min(max((int)round(ar), 0), T.Nm - 1);
    it = min(max((int)ar, 0), T.Nm - 1);
    return 1;
}

static __device__ __noinline__ int z_index_exact(const DevTables &T, double x64, int v, int &ir, int &it)
{
    if (v == 0 && tie_lookup(T.tie_z_bits, T.tie_z_round, T.tie_z_trunc, T.n_tie_z, x64, ir, it))
        return 0;
    double zr = (x64 - T.zmin) * T.Nz / (T.zmax - T.zmin);
    ir = min(max((int)round(zr), 0), T.Nz - 1);
    it = min(max((int)zr, 0), T.Nz - 1);
    return 1;
}

// the k index of k = 10^x / w(z), by the reference's expression
static __device__ __noinline__ int kidx_l_exact(const DevTables &T, double x, int zr)
{
    const double l = pow(10.0, x);
    return kix_exact64(T, l / T.w[zr]);
}

// the k index of k3 from the FP64 coordinates of l1, l2 and phi: |l1 + l2| / w
// (src/NNMap_Model.cu:814-817), or the bispectrum's k3 from k1 = l1 / w, k2 = l2 / w
// (src/generalFunctions.cu:99)
static __device__ __noinline__ int kidx_k3_exact(const DevTables &T, double x1, double x2, double xphi,
                                          int zr, bool from_k)
{
    const double cph = cos(xphi);
    double p1 = pow(10.0, x1), p2 = pow(10.0, x2);
    const double wz = T.w[zr];
    if (from_k) {
        p1 = p1 / wz;
        p2 = p2 / wz;
    }
    double q = __dadd_rn(__dadd_rn(__dmul_rn(p1, p1), __dmul_rn(p2, p2)),
                         __dmul_rn(__dmul_rn(__dmul_rn(2.0, p1), p2), cph));
    q = sqrt(q);
    if (!from_k) q = q / wz;
    return kix_exact64(T, q);
}

// ------------------------------------------------------------------ per-term models
struct Child {
    double c64[MAX_DIM + 1];  // FP64 centres: dims of child 0, then child 1's split dim
    int lev[MAX_DIM + 1];
};

template <int KIND, int TERM>
struct ModelF {
    static constexpr int DIM = TERM + 4;

    // exact FP64 coordinate of a variant (the reference's c -+ (h lambda))
    __device__ static double coord64(const IntDesc &d, const Child &C, int slotdim, int dim, int v)
    {
        double c = C.c64[slotdim];
        if (v == 0) return c;
        double hw = ldexp(d.hw0[dim], -C.lev[slotdim]);
        double lam = (v <= 2) ? G3L_LAMBDA2 : (v <= 4 ? G3L_LAMBDA4 : G3L_LAMBDA5);
        double r = __dmul_rn(hw, lam);
        return (v & 1) ? __dsub_rn(c, r) : __dadd_rn(c, r);
    }

    __device__ static void fill(const DevTables &T, const IntDesc &d, const Child &C, int slotdim,
                                int dim, int v, df x, SlotF &S, unsigned &ties)
    {
        if (dim < 2) {  // l1, l2: ls = 10^x / L0, A = ls^2 * U(theta l)
            float ls = exp10f(x.hi) * fmaf(2.302585093f, x.lo, 1.f) * 1e-3f;
            float U = aperture32(d.th_s[dim] * ls);
            S.f[0] = ls;
            S.f[1] = ls * ls * U;
            S.f[2] = x.hi;
            S.f[3] = x.lo;
        } else if (dim == 2) {  // phi: cos and 1 + cos = 2 cos^2(phi/2)
            float s, c;
            sincosf(x.hi, &s, &c);
            S.f[0] = c - s * x.lo;
            float sh, ch;
            sincosf(0.5f * x.hi, &sh, &ch);
            ch = ch - sh * 0.5f * x.lo;
            S.f[1] = 2.f * ch * ch;
        } else if (dim < 3 + TERM) {  // halo mass (log10 m)
            int ir, it;
            df a = df_mul(df_add(x, df_neg({T.m_x02.x, T.m_x02.y})), {T.m_s2.x, T.m_s2.y});
            if (idx_df(a, T.Nm, IDX_TOL, ir, it))
                ties += m_index_exact(T, coord64(d, C, slotdim, dim, v), v, ir, it);
            S.i0 = ir;
            S.i1 = it;
            S.f[0] = exp10f(x.hi - 12.f) * fmaf(2.302585093f, x.lo, 1.f);  // m / 1e12
            // occupations (src/HOD.cu:35-76) from log10 m; hodp = {f, alpha, log10 Mth (df),
            // ln10 / (sigma 1.414213562), log10 M' (df), beta}.  erfc keeps 1 + erf accurate
            // far below the threshold mass.
            // one loop body for the populations (NNMap: hod1 and hod2; the same values
            // when they are one slot), so the erfc and exp10 code is held once
            const float xm = x.hi + x.lo;
            const int npop = (KIND == 0 && !d.same) ? 2 : 1;
#pragma unroll 1
            for (int q = 0; q < npop; ++q) {
                const float *h = T.f_hodp + 8 * (q ? d.hod2 : d.hod1);
                const float e = erfcf(-((x.hi - h[2]) + (x.lo - h[3])) * h[4]);
                const float nc = 0.5f * h[1] * e;
                const float ns = 0.5f * e * exp10f(h[7] * ((x.hi - h[5]) + (x.lo - h[6])));
                if (q == 0) {
                    S.f[1] = nc;
                    S.f[2] = ns;
                } else {
                    S.f[3] = nc;
                    S.f[4] = ns;
                }
            }
            if (KIND == 0) {
                if (d.same) {
                    S.f[3] = S.f[1];
                    S.f[4] = S.f[2];  // (N_s + s^2 - 1) N_s, s^2 - 1 per slot and mass bin
                    S.f[5] = (S.f[2] + __ldg(T.f_scale + d.hod1 * T.Nm + ir)) * S.f[2];
                } else {
                    float n12 = S.f[2] * S.f[4];
                    float r = n12 + T.fA * exp10f(T.feps * xm) * sqrtf(n12);
                    S.f[5] = r < 0.f ? 0.f : r;
                }
            }
        } else {  // z
            int ir, it;
            df a = df_mul(df_add(x, df_neg({T.z_02.x, T.z_02.y})), {T.z_s2.x, T.z_s2.y});
            if (idx_df(a, T.Nz, IDX_TOL, ir, it))
                ties += z_index_exact(T, coord64(d, C, slotdim, dim, v), v, ir, it);
            S.i0 = ir;
            S.i1 = it;
            const float opz = 1.f + (x.hi + x.lo);
            if (KIND == 0) {
                const float nb1 = __ldg(T.f_nbar + d.hod1 * T.Nz + ir);
                const float nb2 = __ldg(T.f_nbar + d.hod2 * T.Nz + ir);
                S.f[0] = __ldg(T.f_zA + ir) * opz / (nb1 * nb2);
            } else {
                const float nb = __ldg(T.f_nbar + d.hod1 * T.Nz + ir);
                S.f[0] = __ldg(T.f_zB + ir) * opz * opz / (nb * nb);
            }
            S.f[1] = __ldg(T.f_kw + ir);    // L0 / w
            S.f[2] = __ldg(T.f_k200 + it);  // r_200^3 / (m / 1e12)
        }
    }

    // FP64 coordinate of point (for the rare exact k-index fallback)
    __device__ static double px64(const IntDesc &d, const Child &C, int ch, int sdim, int dim,
                                  uint32_t vv)
    {
        int v = (vv >> (3 * dim)) & 7;
        int sd = (ch && dim == sdim) ? DIM : dim;
        return coord64(d, C, sd, dim, v);
    }

    // k index of k = l/w for the l coordinate of dimension dl, exact on a boundary
    __device__ static int kidx_l(const DevTables &T, const IntDesc &d, const Child &C, int ch,
                                 int sdim, uint32_t vv, int dl, const SlotF &L, int zr,
                                 unsigned &ties)
    {
        df a = df_add(df_mul({L.f[2], L.f[3]}, {T.k_a.x, T.k_a.y}),
                      df_neg({T.f_kb[zr].x, T.f_kb[zr].y}));
        bool near;
        int ix = round_df(a, IDX_TOL, near);
        if (!near) return ix;
        ++ties;
        return kidx_l_exact(T, px64(d, C, ch, sdim, dl, vv), zr);
    }

    // k index of k3 (|l1 + l2| / w, or from k1, k2 in the bispectrum), exact on a boundary
    __device__ static int kidx_k3(const DevTables &T, const IntDesc &d, const Child &C, int ch,
                                  int sdim, uint32_t vv, int zr, float k3, bool from_k,
                                  unsigned &ties)
    {
        df a = df_mul(df_add(ln_df(k3), df_neg({T.lnkmin2.x, T.lnkmin2.y})),
                      {T.kscale2.x, T.kscale2.y});
        bool near;
        int ix = round_df(a, K3_TOL, near);
        if (!near) return ix;
        ++ties;
        return kidx_k3_exact(T, px64(d, C, ch, sdim, 0, vv), px64(d, C, ch, sdim, 1, vv),
                             px64(d, C, ch, sdim, 2, vv), zr, from_k);
    }

    // u_NFW calls that depend on one l, one mass and z only: evaluated once per distinct
    // (l, m, z) variant combination of a work item (ucached) and passed to point() in uc[].
    // {l dim, m dim, concentration factor: 0 = 1, 1 = f of hod1, 2 = f of hod2}
    static constexpr int NF = ucache_nf(TERM);
    // cache the (l, m, z) u_NFW for every term (measured faster for all six)
    static constexpr bool UC = true;
    __host__ __device__ static constexpr int ufun(int f, int k)
    {
        return ucache_fun(KIND, TERM, f, k);
    }

    // the cached u_NFW f at slots L (l), M (mass), Z (z), with the expressions of point()
    __device__ static float ucached(const DevTables &T, const IntDesc &d, int f, const SlotF &L,
                                    const SlotF &M, const SlotF &Z, int &small)
    {
        const float kx = L.f[0] * Z.f[1];
        const float r = cbrtf(M.f[0] * Z.f[2]);
        const float cc = __ldg(T.f_conc + Z.i1 * T.Nm + M.i1);
        const int fs = ufun(f, 2);
        const float fac = fs == 0 ? cc : (fs == 1 ? T.f_hodp[8 * d.hod1] : T.f_hodp[8 * d.hod2]) * cc;
        return u_nfw32(kx * r, fac, T.small_arg, small);
    }

    __device__ static float point(const DevTables &T, const IntDesc &d, const SlotF *const *s,
                                  const Child &C, int ch, int sdim, uint32_t vv, unsigned &ties,
                                  int &small, const float *uc)
    {
        const SlotF &L1 = *s[0], &L2 = *s[1], &PH = *s[2], &Z = *s[DIM - 1];
        const float l1 = L1.f[0], l2 = L2.f[0], cphi = PH.f[0];
        const float dl = l1 - l2;
        const float l3 = sqrtf(fmaf(dl, dl, 2.f * l1 * l2 * PH.f[1]));
        const float U3 = aperture32(d.th_s[2] * l3);
        const float kw = Z.f[1], k200 = Z.f[2];
        const int zr = Z.i0, zt = Z.i1, Nm = T.Nm;
        const float k1 = l1 * kw, k2 = l2 * kw, k3 = l3 * kw;
        const float A12 = L1.f[1] * L2.f[1];
        const float sa = T.small_arg;
        if (KIND == 0) {
            const float f1 = T.f_hodp[8 * d.hod1], f2 = T.f_hodp[8 * d.hod2];
            if (TERM == 1) {
                const SlotF &M = *s[3];
                const float r2 = cbrtf(M.f[0] * k200);
                const float cc = __ldg(T.f_conc + zt * Nm + M.i1);
                const float u3 = u_nfw32(k3 * r2, cc, sa, small);
                const float u1 = uc[0];
                const float u2 = uc[1];
                const float H = __ldg(T.f_hmf + zr * Nm + M.i0);
                const float Ggg = M.f[1] * M.f[4] * u2 + M.f[3] * M.f[2] * u1 + M.f[5] * u1 * u2;
                return A12 * U3 * Z.f[0] * (H * M.f[0] * M.f[0]) * u3 * Ggg;
            } else if (TERM == 2) {
                const SlotF &M1 = *s[3], &M2 = *s[4];
                const int kx3 = kidx_k3(T, d, C, ch, sdim, vv, zr, k3, false, ties);
                float P1, P2;
                plin_l12(T, d, C, ch, sdim, vv, L1, L2, zr, k1, k2, ties, P1, P2);
                const float P3 = plin32(T, zr, kx3, k3);
                float u3_1, u3_2;
                u3_pair(T, M1, M2, k3, k200, zt, small, u3_1, u3_2);
                const float u1_1 = uc[0];
                const float u2_1 = uc[1];
                const float u1_2 = uc[2];
                const float u2_2 = uc[3];
                const float Ggg = M2.f[1] * M2.f[4] * u2_2 + M2.f[3] * M2.f[2] * u1_2 +
                                  M2.f[5] * u1_2 * u2_2;
                const float G11 = M1.f[1] + M1.f[2] * u1_1, G22 = M2.f[3] + M2.f[4] * u2_2;
                const float G21 = M1.f[3] + M1.f[4] * u2_1, G12 = M2.f[1] + M2.f[2] * u1_2;
                const float m1 = M1.f[0], m2 = M2.f[0];
                const float HB = (__ldg(T.f_hmf + zr * Nm + M1.i0) * m1) *
                                 (__ldg(T.f_hmf + zr * Nm + M2.i0) * m2) *
                                 __ldg(T.f_bh + zr * Nm + M1.i0) * __ldg(T.f_bh + zr * Nm + M2.i0);
                const float br = m1 * u3_1 * Ggg * P3 + m2 * u3_2 * (G11 * G22 * P1 + G21 * G12 * P2);
                return A12 * U3 * Z.f[0] * HB * br;
            } else {
                const SlotF &M1 = *s[3], &M2 = *s[4], &M3 = *s[5];
                const float m1 = M1.f[0], m2 = M2.f[0], m3 = M3.f[0];
                const float u3 = u_nfw32(k3 * cbrtf(m3 * k200), __ldg(T.f_conc + zt * Nm + M3.i1), sa, small);
                const float u1 = UC ? uc[0] : u_nfw32(k1 * cbrtf(m1 * k200), f1 * __ldg(T.f_conc + zt * Nm + M1.i1), sa, small);
                const float u2 = UC ? uc[1] : u_nfw32(k2 * cbrtf(m2 * k200), f2 * __ldg(T.f_conc + zt * Nm + M2.i1), sa, small);
                const float G1 = M1.f[1] + M1.f[2] * u1, G2 = M2.f[3] + M2.f[4] * u2;
                const float Bi = bi32(T, d, C, ch, sdim, vv, zr, k1, k2, k3, cphi, L1, L2, ties);
                const float HB = (__ldg(T.f_hmf + zr * Nm + M1.i0) * m1) *
                                 (__ldg(T.f_hmf + zr * Nm + M2.i0) * m2) *
                                 (__ldg(T.f_hmf + zr * Nm + M3.i0) * m3 * m3) *
                                 __ldg(T.f_bh + zr * Nm + M1.i0) * __ldg(T.f_bh + zr * Nm + M2.i0) *
                                 __ldg(T.f_bh + zr * Nm + M3.i0);
                return A12 * U3 * Z.f[0] * HB * u3 * G1 * G2 * Bi;
            }
        } else {
            const float f = T.f_hodp[8 * d.hod1];
            if (TERM == 1) {
                const SlotF &M = *s[3];
                const float r2 = cbrtf(M.f[0] * k200);
                const float cc = __ldg(T.f_conc + zt * Nm + M.i1);
                const float m = M.f[0];
                const float G = M.f[1] + M.f[2] * uc[0];
                const float u2 = uc[1];
                const float u3 = u_nfw32(k3 * r2, cc, sa, small);
                return A12 * U3 * Z.f[0] * (__ldg(T.f_hmf + zr * Nm + M.i0) * m * m * m) * G * u2 * u3;
            } else if (TERM == 2) {
                const SlotF &M1 = *s[3], &M2 = *s[4];
                const int kx3 = kidx_k3(T, d, C, ch, sdim, vv, zr, k3, false, ties);
                float P1, P2;
                plin_l12(T, d, C, ch, sdim, vv, L1, L2, zr, k1, k2, ties, P1, P2);
                const float P3 = plin32(T, zr, kx3, k3);
                float u3_1, u3_2;
                u3_pair(T, M1, M2, k3, k200, zt, small, u3_1, u3_2);
                const float u2_1 = uc[0];
                const float u1_2f = uc[1];
                const float u2_2 = uc[2];
                const float u1_1f = uc[3];
                const float G2 = M2.f[1] + M2.f[2] * u1_2f, G1 = M1.f[1] + M1.f[2] * u1_1f;
                const float m1 = M1.f[0], m2 = M2.f[0];
                const float HB = (__ldg(T.f_hmf + zr * Nm + M1.i0) * m1) *
                                 (__ldg(T.f_hmf + zr * Nm + M2.i0) * m2) *
                                 __ldg(T.f_bh + zr * Nm + M1.i0) * __ldg(T.f_bh + zr * Nm + M2.i0);
                const float br = m1 * m2 * G2 * (u2_1 * u3_2 * P2 + u3_1 * u2_2 * P3) +
                                 m2 * m2 * u2_1 * u3_2 * G1 * P1;
                return A12 * U3 * Z.f[0] * HB * br;
            } else {
                const SlotF &M1 = *s[3], &M2 = *s[4], &M3 = *s[5];
                const float m1 = M1.f[0], m2 = M2.f[0], m3 = M3.f[0];
                const float ra = cbrtf(m1 * k200), rb = cbrtf(m2 * k200);
                const float ca = __ldg(T.f_conc + zt * Nm + M1.i1);
                const float cb = __ldg(T.f_conc + zt * Nm + M2.i1);
                const float u2_1 = UC ? uc[0] : u_nfw32(k2 * ra, ca, sa, small);
                const float u3_2 = u_nfw32(k3 * rb, cb, sa, small);
                const float G = M3.f[1] + M3.f[2] * (UC ? uc[1] : u_nfw32(k1 * rb, f * cb, sa, small));
                const float Bi = bi32(T, d, C, ch, sdim, vv, zr, k1, k2, k3, cphi, L1, L2, ties);
                const float HB = (__ldg(T.f_hmf + zr * Nm + M1.i0) * m1 * m1) *
                                 (__ldg(T.f_hmf + zr * Nm + M2.i0) * m2 * m2) *
                                 (__ldg(T.f_hmf + zr * Nm + M3.i0) * m3) *
                                 __ldg(T.f_bh + zr * Nm + M1.i0) * __ldg(T.f_bh + zr * Nm + M2.i0) *
                                 __ldg(T.f_bh + zr * Nm + M3.i0);
                return A12 * U3 * Z.f[0] * HB * u2_1 * u3_2 * G * Bi;
            }
        }
    }

    // P_lin at k1 = l1 / w and k2 = l2 / w with their exact-on-a-boundary indices, through
    // one copy of the index code
    __device__ static void plin_l12(const DevTables &T, const IntDesc &d, const Child &C, int ch,
                                    int sdim, uint32_t vv, const SlotF &L1, const SlotF &L2,
                                    int zr, float k1, float k2, unsigned &ties, float &P1,
                                    float &P2)
    {
        float P[2];
#pragma unroll 1
        for (int q = 0; q < 2; ++q) {
            const int kx = kidx_l(T, d, C, ch, sdim, vv, q, q ? L2 : L1, zr, ties);
            const float v = plin32(T, zr, kx, q ? k2 : k1);
            if (q == 0) P[0] = v;
            else P[1] = v;
        }
        P1 = P[0];
        P2 = P[1];
    }

    // u_NFW(k3 r_200(m_a), c(m_a)) for the two masses of a 2-halo point, through one call
    // site (a single copy of u_nfw32 in the kernel's hot loop)
    __device__ static void u3_pair(const DevTables &T, const SlotF &M1, const SlotF &M2,
                                   float k3, float k200, int zt, int &small, float &u1, float &u2)
    {
        float u[2];
#pragma unroll 1
        for (int q = 0; q < 2; ++q) {
            const SlotF &M = q ? M2 : M1;
            const float r = cbrtf(M.f[0] * k200);
            const float c = __ldg(T.f_conc + zt * T.Nm + M.i1);
            const float v = u_nfw32(k3 * r, c, T.small_arg, small);
            if (q == 0) u[0] = v;
            else u[1] = v;
        }
        u1 = u[0];
        u2 = u[1];
    }

    // tree-level bispectrum (src/generalFunctions.cu:94-147), scaled by the P_lin scale^2;
    // cos(k1,k3) and cos(k2,k3) in the cancellation-free forms -(k1 + k2 c)/k3, -(k2 + k1 c)/k3
    // k3 = |k1 + k2| is passed in from the cancellation-free l3 (k3 = l3 L0 / w).
    __device__ static float bi32(const DevTables &T, const IntDesc &d, const Child &C, int ch,
                                 int sdim, uint32_t vv, int zr, float k1, float k2, float k3,
                                 float cphi, const SlotF &L1, const SlotF &L2, unsigned &ties)
    {
        const float c13 = -(k1 + k2 * cphi) / k3;
        const float c23 = -(k2 + k1 * cphi) / k3;
        const int kx3 = kidx_k3(T, d, C, ch, sdim, vv, zr, k3, true, ties);
        float P1, P2;
        plin_l12(T, d, C, ch, sdim, vv, L1, L2, zr, k1, k2, ties, P1, P2);
        const float P3 = plin32(T, zr, kx3, k3);
        const float F12 = 0.7143f + 0.2857f * cphi * cphi + 0.5f * cphi * (k1 / k2 + 1.f);
        const float F13 = 0.7143f + 0.2857f * c13 * c13 + 0.5f * c13 * (k1 / k3 + 1.f);
        const float F23 = 0.7143f + 0.2857f * c23 * c23 + 0.5f * c23 * (k2 / k3 + 1.f);
        return 2.f * (F12 * P1 * P2 + F13 * P1 * P3 + F23 * P2 * P3);
    }
};

// ------------------------------------------------------------------ rule sums
__host__ __device__ constexpr float df_hi_of(double x) { return (float)x; }
__host__ __device__ constexpr float df_lo_of(double x) { return (float)(x - (double)(float)x); }

template <int DIM>
struct RuleW {
    static constexpr double w1 = (double)(12824 - 9120 * DIM + 400 * DIM * DIM) / (double)19683;
    static constexpr double w3 = (double)(1820 - 400 * DIM) / (double)19683;
    static constexpr double w5 = (double)6859 / (double)19683 / (double)(1u << DIM);
    static constexpr double wE1 = (double)(729 - 950 * DIM + 50 * DIM * DIM) / (double)729;
    static constexpr double wE3 = (double)(265 - 100 * DIM) / (double)1458;
    static constexpr double w2 = 980. / 6561., w4 = 200. / 19683.;
    static constexpr double wE2 = 245. / 486., wE4 = 25. / 729.;
};

__device__ __forceinline__ df shfl_xor_df(df a, int m, unsigned mask = 0xffffffffu)
{
    return {__shfl_xor_sync(mask, a.hi, m), __shfl_xor_sync(mask, a.lo, m)};
}

// half-warp (16-lane) reductions; lanes 0-15 serve child 0, 16-31 child 1
__device__ __forceinline__ df hw_sum(df a)
{
    for (int m = 8; m > 0; m >>= 1) a = df_add(a, shfl_xor_df(a, m));
    return a;
}

// The bound on the FP32 error of one point value has a relative part (the FP32
// chain) and an absolute part (values so small that intermediate products may
// have lost range): T.unc_eps |v| + T.unc_abs.  A split the bounds do not settle is
// flagged (bit 7 of split) when the region's error exceeds T.tau_impact of the
// integral (default 0: always); the selection kernel has it re-taken in FP64 if the
// region is cut.  The error estimate's bound (unc) decides selection boundaries.

template <int KIND, int TERM>
__device__ void warp_itemF(const DevTables &T, const IntDesc &d, int iint, double Vcur,
                           const Pool &P, BatchHdr *H, long long pslot, long long qslot, bool cut,
                           SlotF *slots, float *vals, Child &C, const uint32_t *sdesc,
                           unsigned &ties, int &small, const uint8_t *ucidx,
                           const uint16_t *ucl, const int *ucn, float *ucache)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    constexpr int NRR = 2 * DIM * (DIM - 1);
    using W = RuleW<DIM>;
    const int lane = threadIdx.x & 31;
    const long long stride = P.stride;
    const int sdim = cut ? (P.split[pslot] & 0x7F) : 0;
    const int nchild = cut ? 2 : 1;
    // parent geometry -> child centres (FP64: one add per child)
    double c_l = 0;
    int lev = 0;
    if (lane < DIM) {
        c_l = P.center[lane * stride + pslot];
        lev = P.level[lane * stride + pslot];
    }
    const int levs = __shfl_sync(0xffffffffu, lev, sdim) + (cut ? 1 : 0);
    const double cs = __shfl_sync(0xffffffffu, c_l, sdim);
    double cchild = cs;
    if (cut && lane < 2) {
        const double hws = ldexp(d.hw0[sdim], -levs);
        cchild = lane == 0 ? __dsub_rn(cs, hws) : __dadd_rn(cs, hws);
    }
    const double cL = __shfl_sync(0xffffffffu, cchild, 0);
    const double cR = __shfl_sync(0xffffffffu, cchild, 1);
    const int levsum = __reduce_add_sync(0xffffffffu, lane < DIM ? lev : 0) + (cut ? 1 : 0);
    if (lane < DIM) {
        C.c64[lane] = (cut && lane == sdim) ? cL : c_l;
        C.lev[lane] = (cut && lane == sdim) ? levs : lev;
    }
    if (lane == DIM) {
        C.c64[DIM] = cR;
        C.lev[DIM] = levs;
    }
    __syncwarp();
    // coordinate-variant slots
    const int nslot = (DIM + nchild - 1) * NVAR;
    for (int t = lane; t < nslot; t += 32) {
        const int sd = t / NVAR, v = t - sd * NVAR;
        const int dim = sd < DIM ? sd : sdim;
        df x = df_from_double(C.c64[sd]);
        if (v > 0) {
            const int li = (v <= 2) ? 0 : (v <= 4 ? 1 : 2);
            df r = df_ldexp({d.hwl[dim][li].x, d.hwl[dim][li].y}, -C.lev[sd]);
            x = (v & 1) ? df_add(x, df_neg(r)) : df_add(x, r);
        }
        ModelF<KIND, TERM>::fill(T, d, C, sd, dim, v, x, slots[t], ties);
    }
    __syncwarp();
    // u_NFW of the (l, m, z) variant combinations the points share, per child
    constexpr int NF = ModelF<KIND, TERM>::NF;
    for (int t = lane; ModelF<KIND, TERM>::UC && t < nchild * NF * UC_MAX; t += 32) {
        const int ch = t / (NF * UC_MAX), r = t - ch * NF * UC_MAX;
        const int f = r / UC_MAX, j = r - f * UC_MAX;
        if (j >= ucn[f]) continue;
        const uint32_t key = ucl[f * UC_MAX + j];
        const int dl = ModelF<KIND, TERM>::ufun(f, 0), dm = ModelF<KIND, TERM>::ufun(f, 1);
        const int vl = key & 7, vm = (key >> 3) & 7, vz = (key >> 6) & 7;
        auto sl = [&](int dim, int v) -> const SlotF & {
            return (ch && dim == sdim) ? slots[DIM * NVAR + v] : slots[dim * NVAR + v];
        };
        ucache[(ch * NF + f) * UC_MAX + j] =
            ModelF<KIND, TERM>::ucached(T, d, f, sl(dl, vl), sl(dm, vm), sl(DIM - 1, vz), small);
    }
    __syncwarp();
    // points
    for (int p = lane; p < nchild * NP; p += 32) {
        const int ch = p >= NP ? 1 : 0;
        const int pp = p - ch * NP;
        const uint32_t vv = sdesc[pp];
        const SlotF *sp[DIM];
#pragma unroll
        for (int dd = 0; dd < DIM; ++dd) {
            const int v = (vv >> (3 * dd)) & 7;
            sp[dd] = (ch && dd == sdim) ? &slots[DIM * NVAR + v] : &slots[dd * NVAR + v];
        }
        float uc[NF] = {};
        if (ModelF<KIND, TERM>::UC) {
#pragma unroll
            for (int f = 0; f < NF; ++f) uc[f] = ucache[(ch * NF + f) * UC_MAX + ucidx[f * NP + pp]];
        }
        vals[p] = ModelF<KIND, TERM>::point(T, d, sp, C, ch, sdim, vv, ties, small, uc);
        if (H->dbg) H->dbg[p] = (double)vals[p];
    }
    __syncwarp();
    // rule sums in double-float, uncertainty sums in FP32: half-warp hh serves child hh
    const int hh = lane >> 4, hl = lane & 15;
    const bool active = hh < nchild;
    const float *v = vals + hh * NP;
    df s2 = {0.f, 0.f}, s3 = {0.f, 0.f}, s45 = {0.f, 0.f}, s4 = {0.f, 0.f};
    float u2 = 0.f, u3 = 0.f, u4 = 0.f, u5 = 0.f;
    df diff = {-1.f, 0.f};
    float udiff = 0.f;
    const float val0 = active ? v[0] : 0.f;
    const float EPS_REL = T.unc_eps, TAU_ABS = T.unc_abs;
    const float u0 = fmaf(EPS_REL, fabsf(val0), TAU_ABS);
    constexpr float RATIO = (float)((G3L_LAMBDA2 * G3L_LAMBDA2) / (G3L_LAMBDA4 * G3L_LAMBDA4));
    if (active && hl < DIM) {
        const float a0 = v[1 + 4 * hl], a1 = v[2 + 4 * hl], b0 = v[3 + 4 * hl], b1 = v[4 + 4 * hl];
        const df a = df_two_sum(a0, a1);
        const df b = df_two_sum(b0, b1);
        s2 = a;
        s3 = b;
        const float ua = fmaf(EPS_REL, fabsf(a0), TAU_ABS) + fmaf(EPS_REL, fabsf(a1), TAU_ABS);
        const float ub = fmaf(EPS_REL, fabsf(b0), TAU_ABS) + fmaf(EPS_REL, fabsf(b1), TAU_ABS);
        u2 = ua;
        u3 = ub;
        const df tv = {-2.f * val0, 0.f};
        const df da = df_add(a, tv), db = df_add(b, tv);
        df dd = df_add(da, df_neg(df_mul(db, {df_hi_of((G3L_LAMBDA2 * G3L_LAMBDA2) /
                                                       (G3L_LAMBDA4 * G3L_LAMBDA4)),
                                              df_lo_of((G3L_LAMBDA2 * G3L_LAMBDA2) /
                                                       (G3L_LAMBDA4 * G3L_LAMBDA4))})));
        diff = dd.hi < 0.f ? df_neg(dd) : dd;
        udiff = ua + RATIO * ub + (2.f - 2.f * RATIO) * u0;
    }
    if (active) {
        for (int k = hl; k < NRR; k += 16) {
            const float x = v[1 + 4 * DIM + k];
            s4 = df_add_f(s4, x);
            u4 += fmaf(EPS_REL, fabsf(x), TAU_ABS);
        }
        for (int k = hl; k < (1 << DIM); k += 16) {
            const float x = v[1 + 4 * DIM + NRR + k];
            s45 = df_add_f(s45, x);
            u5 += fmaf(EPS_REL, fabsf(x), TAU_ABS);
        }
    }
    s2 = hw_sum(s2);
    s3 = hw_sum(s3);
    s4 = hw_sum(s4);
    s45 = hw_sum(s45);
    for (int m = 8; m > 0; m >>= 1) {
        u2 += __shfl_xor_sync(0xffffffffu, u2, m);
        u3 += __shfl_xor_sync(0xffffffffu, u3, m);
        u4 += __shfl_xor_sync(0xffffffffu, u4, m);
        u5 += __shfl_xor_sync(0xffffffffu, u5, m);
    }
    // split dimension: first maximum of the fourth differences, and the runner-up
    int sidx = hl;
    df best = diff;
    float ubest = udiff;
    for (int m = 8; m > 0; m >>= 1) {
        df od = shfl_xor_df(best, m);
        int oi = __shfl_xor_sync(0xffffffffu, sidx, m);
        float ou = __shfl_xor_sync(0xffffffffu, ubest, m);
        if (df_gt(od, best) || (od.hi == best.hi && od.lo == best.lo && oi < sidx)) {
            best = od;
            sidx = oi;
            ubest = ou;
        }
    }
    df second = (hl == sidx) ? df{-1.f, 0.f} : diff;
    float usecond = (hl == sidx) ? 0.f : udiff;
    for (int m = 8; m > 0; m >>= 1) {
        df od = shfl_xor_df(second, m);
        float ou = __shfl_xor_sync(0xffffffffu, usecond, m);
        if (df_gt(od, second)) {
            second = od;
            usecond = ou;
        }
    }
    // decisive when the gap between the two largest differences exceeds both bounds
    const bool split_sure = (best.hi - fmaxf(second.hi, 0.f)) > (ubest + usecond) &&
                            best.hi > ubest;
    // the contenders: dimensions whose difference may reach the leader's under the bounds
    // (an FP64 re-take of an unsettled split evaluates only their axis points)
    const unsigned cbits = __ballot_sync(
        0xffffffffu, active && hl < DIM &&
                         diff.hi + udiff >= (best.hi - ubest) - 1e-6f * fabsf(best.hi));
    const unsigned cmask = (cbits >> (16 * hh)) & ((1u << DIM) - 1u);
    // 7th- and 5th-degree brackets (double-float), then FP64 on four lanes
    df b7 = df_mul_f({df_hi_of(W::w1), df_lo_of(W::w1)}, val0);
    b7 = df_add(b7, df_mul(s2, {df_hi_of(W::w2), df_lo_of(W::w2)}));
    b7 = df_add(b7, df_mul(s3, {df_hi_of(W::w3), df_lo_of(W::w3)}));
    b7 = df_add(b7, df_mul(s4, {df_hi_of(W::w4), df_lo_of(W::w4)}));
    df b5 = df_mul_f({df_hi_of(W::wE1), df_lo_of(W::wE1)}, val0);
    b5 = df_add(b5, df_mul(s2, {df_hi_of(W::wE2), df_lo_of(W::wE2)}));
    b5 = df_add(b5, df_mul(s3, {df_hi_of(W::wE3), df_lo_of(W::wE3)}));
    b5 = df_add(b5, df_mul(s4, {df_hi_of(W::wE4), df_lo_of(W::wE4)}));
    df e = df_add(b5, df_neg(df_add(b7, df_mul(s45, {df_hi_of(W::w5), df_lo_of(W::w5)}))));
    b7 = df_add(b7, df_mul(s45, {df_hi_of(W::w5), df_lo_of(W::w5)}));
    if (e.hi < 0.f) e = df_neg(e);
    // bound on the error of e from the point-value bounds (weights of res7 - res5)
    const float ue = fabsf((float)(W::w1 - W::wE1)) * u0 + fabsf((float)(W::w2 - W::wE2)) * u2 +
                     fabsf((float)(W::w3 - W::wE3)) * u3 + fabsf((float)(W::w4 - W::wE4)) * u4 +
                     fabsf((float)W::w5) * u5;
    const float urel =
        e.hi > 0.f ? fminf(T.unc_sel_ratio * ue / e.hi, 1e30f) : (ue > 0.f ? 1e30f : 0.f);
    // and of the value (weights of res7)
    const float uv = fabsf((float)W::w1) * u0 + fabsf((float)W::w2) * u2 +
                     fabsf((float)W::w3) * u3 + fabsf((float)W::w4) * u4 +
                     fabsf((float)W::w5) * u5;
    const float ab7 = fabsf(b7.hi);
    const float uvrel =
        ab7 > 0.f ? fminf(T.unc_val_ratio * uv / ab7, 1e30f) : (uv > 0.f ? 1e30f : 0.f);
    // lane 16h+0 -> value, 16h+1 -> error of child h
    const df q = hl == 1 ? e : b7;
    if (active && hl < 2) {
        const double vol = ldexp(d.rootvol_mx, -levsum);
        const double out = ((double)q.hi + (double)q.lo) * vol;
        const long long slot = hh == 0 ? pslot : qslot;
        if (hl == 0) {
            P.val[slot] = out;
            P.uval[slot] = uvrel;
        } else {
            P.err[slot] = out;
            P.unc[slot] = urel;
            // An unsettled split is flagged (bit 7); the selection kernel has it re-taken
            // in FP64 only if the region is selected for cutting, so leaves never pay.
            const bool flag = !split_sure && out > T.tau_impact * fabs(Vcur);
            P.split[slot] = (unsigned char)(sidx | (flag ? 0x80 : 0));
            P.cmask[slot] = (unsigned char)cmask;
        }
    }
    // child geometry
    if (cut && lane < DIM) {
        P.center[lane * stride + pslot] = C.c64[lane];
        P.level[lane * stride + pslot] = (unsigned char)C.lev[lane];
        P.center[lane * stride + qslot] = lane == sdim ? cR : c_l;
        P.level[lane * stride + qslot] = (unsigned char)C.lev[lane];
    }
    __syncwarp();
}

// MINB: the blocks per SM the register budget is cut for (6: 80 registers per thread,
// 7: 72, 8: 64); the autotuner picks it per kind x term.
template <int KIND, int TERM, int MINB>
__global__ void __launch_bounds__(128, MINB) k_evalmx(DevTables T, const IntDesc *__restrict__ D,
                                                IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                const long long *__restrict__ woff)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    constexpr int NSLOT = (DIM + 1) * NVAR;
    constexpr int WPB = 4;
    __shared__ uint32_t sdesc[NP];
    __shared__ SlotF sslot[WPB][NSLOT];
    __shared__ float svals[WPB][2 * NP];
    __shared__ Child schild[WPB];
    constexpr int NF = ModelF<KIND, TERM>::NF;
    __shared__ uint8_t ucidx[NF * NP];           // combination of each point, per function
    __shared__ uint16_t ucl[NF * UC_MAX];        // variants (l | m << 3 | z << 6) of each
    __shared__ int ucn[NF];
    __shared__ float ucache[WPB][2 * NF * UC_MAX];
    __shared__ uint8_t ucmap[NF * 343];
    if (ModelF<KIND, TERM>::UC) ucache_tables<KIND, TERM>(ucidx, ucl, ucn, ucmap);
    const int g = KIND * 3 + TERM - 1;
    for (int p = threadIdx.x; p < NP; p += blockDim.x) sdesc[p] = point_variants(DIM, p);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gb = H->gbeg[g], ge = H->gbeg[g + 1];
    if (gb >= ge) return;
    const long long wbeg = woff[gb], wend = woff[ge];
    unsigned ties = 0;
    int small = 0;
    const long long nwarps = (long long)gridDim.x * WPB;
    for (long long w = wbeg + (long long)blockIdx.x * WPB + wib; w < wend; w += nwarps) {
        int lo = gb, hi = ge - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (woff[mid] <= w) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo;
        const long long j = w - woff[i];
        const IntDesc &d = D[i];
        const int cj = P.cand[d.base + j];
        const bool cut = cj >= 0;
        const long long pslot = d.base + (cut ? cj : 0);
        const long long qslot = cut ? d.base + (S[i].nR - S[i].K) + j : -1;
        warp_itemF<KIND, TERM>(T, d, i, S[i].val, P, H, pslot, qslot, cut, sslot[wib],
                               svals[wib], schild[wib], sdesc, ties, small, ucidx, ucl, ucn,
                               ucache[wib]);
    }
    // warp-aggregated diagnostics
    unsigned tw = __reduce_add_sync(0xffffffffu, ties);
    unsigned sw = __reduce_add_sync(0xffffffffu, (unsigned)small);
    if (lane == 0) {
        if (tw) atomicAdd(&H->ties, (unsigned long long)tw);
        if (sw) atomicAdd(&H->small_arg, (unsigned long long)sw);
    }
}

}  // namespace g3l
