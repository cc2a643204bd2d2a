// phys64.cuh -- FP64 halo-model primitives on the device.
//
// Each function keeps the reference's IEEE operation order (compile with
// -fmad=false) so that, apart from the last-ulp differences between this
// device's libm and glibc, the values equal the reference's CPU path:
//   SiCi           src/generalFunctions.cu:44-87
//   u_NFW, r_200   src/generalFunctions.cu:6-37
//   apertureFilter src/generalFunctions.cu:39-42
//   Ncen, Nsat     src/HOD.cu:35-76;  NsatNsat src/HOD.cu:78-94
//   F, Bi_lin      src/generalFunctions.cu:89-147
// The Si/Ci coefficients are the published Pade approximants of Rowe et al.
// (2015, GalSim).  The small-argument branch evaluates them with explicit powers left
// to right as the reference does; the large-argument branch in Horner form on 1/x^2
// (one FP64 division instead of forty; ~1e-16 relative from the reference's order).
#pragma once
#include "g3l_device.cuh"

namespace g3l {

// Si(x), Ci(x); sx, cx receive sin(x), cos(x) (the large-argument branch needs them; the
// small one computes them for the caller, so that u_NFW evaluates them once)
__device__ __forceinline__ void sici64_sc(double x, double &si, double &ci, double &sx, double &cx)
{
    double x2 = x * x;
    double x4 = x2 * x2;
    double x6 = x2 * x4;
    double x8 = x4 * x4;
    double x10 = x8 * x2;
    double x12 = x6 * x6;
    double x14 = x12 * x2;
    if (x < 4) {
        double a = 1 - 4.54393409816329991e-2 * x2 + 1.15457225751016682e-3 * x4 -
                   1.41018536821330254e-5 * x6 + 9.43280809438713025e-8 * x8 -
                   3.53201978997168357e-10 * x10 + 7.08240282274875911e-13 * x12 -
                   6.05338212010422477e-16 * x14;
        double b = 1 + 1.01162145739225565e-2 * x2 + 4.99175116169755106e-5 * x4 +
                   1.55654986308745614e-7 * x6 + 3.28067571055789734e-10 * x8 +
                   4.5049097575386581e-13 * x10 + 3.21107051193712168e-16 * x12;
        si = x * a / b;
        a = -0.25 + 7.51851524438898291e-3 * x2 - 1.27528342240267686e-4 * x4 +
            1.05297363846239184e-6 * x6 - 4.68889508144848019e-9 * x8 +
            1.06480802891189243e-11 * x10 - 9.93728488857585407e-15 * x12;
        b = 1 + 1.1592605689110735e-2 * x2 + 6.72126800814254432e-5 * x4 +
            2.55533277086129636e-7 * x6 + 6.97071295760958946e-10 * x8 +
            1.38536352772778619e-12 * x10 + 1.89106054713059759e-15 * x12 +
            1.39759616731376855e-18 * x14;
        ci = 0.5772156649 + log(x) + x2 * a / b;
        sincos(x, &sx, &cx);
    } else {
        // f = (1/x) A(t)/B(t), g = t C(t)/D(t) with t = 1/x^2: the reference's explicit
        // powers of 1/x (src/generalFunctions.cu:65-81) in Horner form, one division for t
        // instead of one per term (each FP64 division is a multi-instruction sequence)
        const double t = 1 / x2;
        double sin_x, cos_x;
        sincos(x, &sin_x, &cos_x);
        double A = -4.94701168645415959931e11;
        A = A * t + 4.94816688199951963482e12;
        A = A * t + 1.00795182980368574617e13;
        A = A * t + 4.20968180571076940208e12;
        A = A * t + 6.40533830574022022911e11;
        A = A * t + 4.33736238870432522765e10;
        A = A * t + 1.43073403821274636888e9;
        A = A * t + 2.37750310125431834034e7;
        A = A * t + 1.96396372895146869801e5;
        A = A * t + 7.44437068161936700618e2;
        A = A * t + 1;
        double B = 1.11535493509914254097e13;
        B = B * t + 1.43468549171581016479e13;
        B = B * t + 5.06084464593475076774e12;
        B = B * t + 7.08501308149515401563e11;
        B = B * t + 4.58595115847765779830e10;
        B = B * t + 1.47478952192985464958e9;
        B = B * t + 2.41535670165126845144e7;
        B = B * t + 1.97865247031583951450e5;
        B = B * t + 7.46437068161927678031e2;
        B = B * t + 1;
        double C = -1.36517137670871689e12;
        C = C * t + 6.43291613143049485e12;
        C = C * t + 1.81004487464664575e13;
        C = C * t + 7.57664583257834349e12;
        C = C * t + 1.09049528450362786e12;
        C = C * t + 6.83052205423625007e10;
        C = C * t + 2.06297595146763354e9;
        C = C * t + 3.12557570795778731e7;
        C = C * t + 2.35239181626478200e5;
        C = C * t + 8.1359520115168615e2;
        C = C * t + 1;
        double Dd = 3.99653257887490811e13;
        Dd = Dd * t + 4.01839087307656620e13;
        Dd = Dd * t + 1.17164723371736605e13;
        Dd = Dd * t + 1.39866710696414565e12;
        Dd = Dd * t + 7.87465017341829930e10;
        Dd = Dd * t + 2.23355543278099360e9;
        Dd = Dd * t + 3.26026661647090822e7;
        Dd = Dd * t + 2.40036752835578777e5;
        Dd = Dd * t + 8.19595201151451564e2;
        Dd = Dd * t + 1;
        const double f = A / B / x;
        const double g = C / Dd * t;
        si = 0.5 * 3.14159265358979323846 - f * cos_x - g * sin_x;
        ci = f * sin_x - g * cos_x;
        sx = sin_x;
        cx = cos_x;
    }
}

__device__ __forceinline__ void sici64(double x, double &si, double &ci)
{
    double sx, cx;
    sici64_sc(x, si, ci, sx, cx);
}

// NFW Fourier profile from k, r_200, c = f x concentration and the normalisation
// F = ln(1 + c) - c / (1 + c) (callers that share one (mass, z) pair pass F once computed)
__device__ __forceinline__ double u_nfw64_F(double k, double r200, double c, double F)
{
    double arg1 = k * r200 / c;
    double arg2 = arg1 * (1 + c);
    double si1, ci1, si2, ci2, s1, c1;
    sici64_sc(arg1, si1, ci1, s1, c1);  // s1, c1 = sin(arg1), cos(arg1)
    sici64(arg2, si2, ci2);
    double term1 = s1 * (si2 - si1);
    double term2 = c1 * (ci2 - ci1);
    double term3 = -sin(arg1 * c) / arg2;
    return (term1 + term2 + term3) / F;
}

__device__ __forceinline__ double nfw_norm64(double c) { return log(1. + c) - c / (1. + c); }

// NFW Fourier profile given k, r_200 and the tabulated concentration (truncated indices
// are resolved by the caller, as in src/generalFunctions.cu:11-15).
__device__ __forceinline__ double u_nfw64(double k, double r200, double conc, double f)
{
    const double c = f * conc;
    return u_nfw64_F(k, r200, c, nfw_norm64(c));
}

__device__ __forceinline__ double r200_64(double m, double rho)
{
    return pow(0.239 * m / rho / 200, 1. / 3.);
}

__device__ __forceinline__ double aperture64(double eta)
{
    return 0.5 * eta * eta * exp(-0.5 * eta * eta);
}

// hod = {f, alpha, Mth, sigma, M', beta}
// N_c and N_s of one HOD at mass m from one evaluation of their common factor
// 1 + erf(ln(m/Mth) / (sigma sqrt 2)) (the reference evaluates it in each, src/HOD.cu:35-76;
// the same expression, so the same values)
__device__ __forceinline__ void occupations64(const double *h, double m, double &nc, double &ns)
{
    const double e1 = 1 + erf(log(m / h[2]) / h[3] / 1.414213562);
    nc = 0.5 * h[1] * e1;
    ns = 0.5 * e1 * pow(m / h[4], h[5]);
}
// NsatNsat from the two satellite occupations Ns1 (hod1) and Ns2 (hod2) at m, the
// reference's expression (src/HOD.cu:78-94) with its nsat calls' values passed in;
// scale1: satellite-variance rescaling (1 = none); the reference reads scale1 only
__device__ __forceinline__ double nsatnsat64(double Ns1, double Ns2, int same, double A,
                                             double eps, double m, double scale1)
{
    if (same) return (Ns1 + scale1 * scale1 - 1) * Ns1;
    double result = Ns1 * Ns2 + A * pow(m, eps) * sqrt(Ns1 * Ns2);
    if (result < 0) return 0;
    return result;
}

__device__ __forceinline__ double F2_64(double k1, double k2, double cosphi)
{
    return 0.7143 + 0.2857 * cosphi * cosphi + 0.5 * cosphi * (k1 / k2 + k2 / k2);
}

// P_lin lookup with the small-k linear extrapolation (src/NNMap_Model.cu:819-839)
__device__ __forceinline__ double plin64(const DevTables &T, int z_ix, double k)
{
    int k_ix = (int)round(log(k / T.kmin) * T.Nk / T.ln_kratio);
    if (k_ix >= 0) {
        // clamp_k: stay in the z row; otherwise the reference's flat read, bounded by
        // the end of the table (the reference reads past it)
        if (T.clamp_k && k_ix > T.Nk - 1) k_ix = T.Nk - 1;
        long long flat = (long long)z_ix * T.Nk + k_ix;
        const long long last = (long long)T.Nz * T.Nk - 1;
        return __ldg(T.P_lin + (flat > last ? last : flat));
    }
    return __ldg(T.P_lin + z_ix * T.Nk) / T.kmin * k;
}

__device__ __forceinline__ double bi_lin64(const DevTables &T, double k1, double k2,
                                           double cosphi, int z_ix)
{
    double k3 = sqrt(k1 * k1 + k2 * k2 + 2 * k1 * k2 * cosphi);
    double c_phi12 = cosphi;
    double c_phi13 = (k2 * k2 - k3 * k3 - k1 * k1) / (2 * k1 * k3);
    double c_phi23 = (k1 * k1 - k2 * k2 - k3 * k3) / (2 * k3 * k2);
    double Pk1 = plin64(T, z_ix, k1);
    double Pk2 = plin64(T, z_ix, k2);
    double Pk3 = plin64(T, z_ix, k3);
    return 2 * (F2_64(k1, k2, c_phi12) * Pk1 * Pk2 + F2_64(k1, k3, c_phi13) * Pk1 * Pk3 +
                F2_64(k2, k3, c_phi23) * Pk2 * Pk3);
}

// Nearest-bin and truncated mass indices of log10 m = x (src/NNMap_Model.cu:556,
// src/generalFunctions.cu:12).  The fast form (x - log10 mmin) * Nm / log10(mmax/mmin)
// agrees with the reference expression to ~1e-12; within 1e-9 of a rounding boundary
// the exact index comes from the host-resolved table of tie-prone centre values, or
// else from the reference expression evaluated here.
__device__ __forceinline__ void m_index(const DevTables &T, double x, double m, int &ir, int &it,
                                        unsigned long long *ties)
{
    double a = (x - T.m_x0) * T.m_scale;
    double fl = floor(a);
    double fr = a - fl;
    const double tol = 1e-9;
    if (fabs(fr - 0.5) > tol && fr > tol && fr < 1 - tol) {
        ir = min(max((int)fl + (fr > 0.5 ? 1 : 0), 0), T.Nm - 1);
        it = min(max((int)fl, 0), T.Nm - 1);
        return;
    }
    unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    int lo = 0, hi = T.n_tie_m - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        unsigned long long b = T.tie_m_bits[mid];
        if (b == bits) {
            ir = T.tie_m_round[mid];
            it = T.tie_m_trunc[mid];
            return;
        }
        if (b < bits) lo = mid + 1;
        else hi = mid - 1;
    }
    double ar = log(m / T.mmin) * T.Nm / T.ln_mratio;
    ir = min(max((int)round(ar), 0), T.Nm - 1);
    it = min(max((int)ar, 0), T.Nm - 1);
    if (ties) atomicAdd(ties, 1ull);
}

}  // namespace g3l
