// eval_fp64.cu -- all-FP64 rule evaluation: the plain FP64 form of the engine.
//
// One warp evaluates one work item: it cuts a selected parent region along its
// split dimension (cut_region, src/hcubature.cpp:206-218) and applies the
// Genz-Malik 7/5 rule to both children (rule75genzmalik_evalError,
// src/hcubature.cpp:456-577), or evaluates a root region.  The per-dimension
// coordinate variants (c, c-+lambda*h) are computed once per child together
// with everything that depends on one coordinate only (10^x, aperture filter,
// HOD occupations, bin indices); each lane then evaluates whole points.  The
// rule sums are formed by one lane per child in the reference's summation
// order.  Compiled with -fmad=false so every product and sum rounds as in the
// reference's CPU build.
#include "phys64.cuh"

namespace g3l {

struct Slot64 {
    double a[6];
    int i0, i1;
};

// coordinate variant v (0 c, 1/2 c -+ r2, 3/4 c -+ r4, 5/6 c -+ r5) of centre c, half-width hw
__device__ __forceinline__ double variant_x(double c, double hw, int v)
{
    double x = c;
    if (v > 0) {
        double lam = (v <= 2) ? G3L_LAMBDA2 : (v <= 4 ? G3L_LAMBDA4 : G3L_LAMBDA5);
        double rr = hw * lam;
        x = (v & 1) ? c - rr : c + rr;
    }
    return x;
}

// truncated z bin of z = x (the z slot's i1, Model64::fill)
__device__ __forceinline__ int z_trunc64(const DevTables &T, double x)
{
    double zr = (x - T.zmin) * T.Nz / (T.zmax - T.zmin);
    return min(max((int)zr, 0), T.Nz - 1);
}

// An FP64 re-take of an unsettled split (a split-only entry) needs the centre and the axis
// points of the contending dimensions only: cm, the dimensions whose fourth-difference
// bounds reach the leader's (P.cmask, written by the FP32 rule kernel with the flag).  The
// others' differences are below the leader's under those bounds, so the FP64 choice among
// the contenders is the FP64 choice among all dimensions.
__device__ __forceinline__ unsigned split_cmask(const Pool &P, const IntDesc &d, int2 ent)
{
    return (unsigned)P.cmask[d.base + (ent.y & 0x3FFFFFFF)];
}

template <int KIND, int TERM>
struct Model64 {
    static constexpr int DIM = TERM + 4;

    // Fill one coordinate-variant slot (everything that depends on one coordinate).
    __device__ static void fill(const DevTables &T, const IntDesc &d, int dimidx, double x,
                                Slot64 &S, unsigned long long *ties)
    {
        if (dimidx < 2) {  // l1, l2 (log10 l)
            double l = pow(10, x);
            S.a[0] = l;
            S.a[1] = aperture64(d.theta[dimidx] * l);
        } else if (dimidx == 2) {  // phi
            S.a[0] = cos(x);
        } else if (dimidx < 3 + TERM) {  // halo masses (log10 m)
            double m = pow(10, x);
            S.a[0] = m;
            m_index(T, x, m, S.i0, S.i1, ties);
            const double *h1 = T.hod + 6 * d.hod1;
            const double *h2 = T.hod + 6 * d.hod2;
            occupations64(h1, m, S.a[1], S.a[2]);
            if (KIND == 0) {
                // the second population's occupations: the same values as the first's when
                // the slots are the same
                if (d.same) {
                    S.a[3] = S.a[1];
                    S.a[4] = S.a[2];
                } else {
                    occupations64(h2, m, S.a[3], S.a[4]);
                }
                // rescaling s of the hod1 slot at this mass's rounded bin
                // (src/NNMap_Model.cu:563,808)
                S.a[5] = nsatnsat64(S.a[2], S.a[4], d.same, T.A, T.eps, m,
                                    __ldg(T.scale + (size_t)d.hod1 * T.Nm + S.i0));
            }
        } else {  // z
            S.a[0] = x;
            double zr = (x - T.zmin) * T.Nz / (T.zmax - T.zmin);
            S.i0 = min(max((int)round(zr), 0), T.Nz - 1);
            S.i1 = min(max((int)zr, 0), T.Nz - 1);
        }
    }

    // Integrand at one point from its variant slots (kernel_function_* of the reference).
    // cached u_NFW f (ucache_fun) at slots L (l), M (mass), Z (z): the expressions of point()
    // mz: r_200 and F of the (M, Z) pair (MZ_VALS values, k_re_fill), or null
    __device__ static double ucached(const DevTables &T, const IntDesc &d, int f, const Slot64 &L,
                                     const Slot64 &M, const Slot64 &Z, const double *mz)
    {
        const double w_ = __ldg(T.w + Z.i0);
        const double k = L.a[0] / w_;
        const double conc = __ldg(T.conc + Z.i1 * T.Nm + M.i1);
        const int fs = ucache_fun(KIND, TERM, f, 2);
        const double c = (fs == 0 ? 1.0 : (fs == 1 ? T.hod[6 * d.hod1] : T.hod[6 * d.hod2])) * conc;
        if (!mz) return u_nfw64_F(k, r200_64(M.a[0], __ldg(T.rho_bar + Z.i1)), c, nfw_norm64(c));
        return u_nfw64_F(k, mz[0], c, mz[1 + fs]);
    }

    // r_200 and F at factors 1, f of hod1, f of hod2 (nf of them) of halo mass slot M at
    // z bin zt, with the expressions of point(): o[0..nf]
    __device__ static void mz_values(const DevTables &T, const IntDesc &d, const Slot64 &M, int zt,
                                     int nf, double *o)
    {
        const double conc = __ldg(T.conc + zt * T.Nm + M.i1);
        o[0] = r200_64(M.a[0], __ldg(T.rho_bar + zt));
        for (int q = 0; q < nf; ++q)
            o[1 + q] = nfw_norm64((q == 0 ? 1.0 : (q == 1 ? T.hod[6 * d.hod1] : T.hod[6 * d.hod2])) * conc);
    }

    // u_NFW(k3, mass u3_mass(f)) of the 2- and 3-halo terms, with the expressions of
    // point(): shared by the points with the same projection (u3_drop)
    // mz: r_200 and F of the (mass, z) pair (k_re_fill), or null
    __device__ static double u3(const DevTables &T, int f, const Slot64 *const *s, const double *mz)
    {
        const Slot64 &L1 = *s[0], &L2 = *s[1], &PH = *s[2], &Z = *s[DIM - 1];
        const Slot64 &M = *s[u3_mass(KIND, TERM, f)];
        const double l1 = L1.a[0], l2 = L2.a[0], cphi = PH.a[0];
        const double w_ = __ldg(T.w + Z.i0);
        const double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cphi);
        const double k3 = l3 / w_;
        const double c = 1.0 * __ldg(T.conc + Z.i1 * T.Nm + M.i1);
        if (!mz) return u_nfw64_F(k3, r200_64(M.a[0], __ldg(T.rho_bar + Z.i1)), c, nfw_norm64(c));
        return u_nfw64_F(k3, mz[0], c, mz[1]);
    }

    // auxiliary function a (aux_dims) with the expressions of point(): the aperture filter
    // of l3; P_lin at k1, k2, k3 (2-halo); the tree-level bispectrum (3-halo)
    __device__ static double aux(const DevTables &T, const IntDesc &d, int a, const Slot64 *const *s)
    {
        const Slot64 &L1 = *s[0], &L2 = *s[1], &PH = *s[2];
        const double l1 = L1.a[0], l2 = L2.a[0], cphi = PH.a[0];
        const double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cphi);
        if (a == 0) return aperture64(d.theta[2] * l3);
        const int z_ix = s[DIM - 1]->i0;
        const double w_ = __ldg(T.w + z_ix);
        if (TERM == 3) return bi_lin64(T, l1 / w_, l2 / w_, cphi, z_ix);
        return plin64(T, z_ix, (a == 1 ? l1 : (a == 2 ? l2 : l3)) / w_);
    }

    // uc: the cached u_NFW values of this point (ucache_fun order), or null; u3c: its
    // cached u_NFW at k3 (u3()), or null; ax: its cached auxiliary values (aux()), or null;
    // mz: r_200 and F of its (mass, z) pair (1-halo terms), or null
    __device__ static double point(const DevTables &T, const IntDesc &d, const Slot64 *const *s,
                                   const double *uc = nullptr, const double *u3c = nullptr,
                                   const double *ax = nullptr, const double *mz = nullptr)
    {
        const Slot64 &L1 = *s[0], &L2 = *s[1], &PH = *s[2], &Z = *s[DIM - 1];
        const double l1 = L1.a[0], l2 = L2.a[0], cphi = PH.a[0], z = Z.a[0];
        const int z_ix = Z.i0, z_it = Z.i1, Nm = T.Nm;
        const double w_ = __ldg(T.w + z_ix);
        const double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cphi);
        const double k1 = l1 / w_;
        const double k2 = l2 / w_;
        const double k3 = l3 / w_;
        const double rho = __ldg(T.rho_bar + z_ix);
        const double rhot = __ldg(T.rho_bar + z_it);
        const double f1 = T.hod[6 * d.hod1];
        const double U3 = ax ? ax[0] : aperture64(d.theta[2] * l3);
        if (KIND == 0) {
            const double nbar1 = __ldg(T.nbar + d.hod1 * T.Nz + z_ix);
            const double nbar2 = __ldg(T.nbar + d.hod2 * T.Nz + z_ix);
            const double f2 = T.hod[6 * d.hod2];
            if (TERM == 1) {
                // src/NNMap_Model.cu:544-593
                const Slot64 &M = *s[3];
                const double m = M.a[0];
                const double r2 = mz ? mz[0] : r200_64(m, rhot);  // mz[0] is this value
                const double cc = __ldg(T.conc + z_it * Nm + M.i1);
                const double u3 = mz ? u_nfw64_F(k3, mz[0], 1.0 * cc, mz[1]) : u_nfw64(k3, r2, cc, 1);
                const double u2 = uc ? uc[1] : u_nfw64(k2, r2, cc, f2);
                const double u1 = uc ? uc[0] : u_nfw64(k1, r2, cc, f1);
                double Bggd = 1. / nbar1 / nbar2 / rho * __ldg(T.hmf + z_ix * Nm + M.i0) * m * u3;
                Bggd *= M.a[1] * M.a[4] * u2 + M.a[3] * M.a[2] * u1 + M.a[5] * u1 * u2;
                double bggk = Bggd / __ldg(T.dwdz + z_ix) * __ldg(T.g + z_ix) *
                              __ldg(T.p1 + z_ix) * __ldg(T.p2 + z_ix) / w_ / w_ / w_ * (1. + z);
                return l1 * l2 * m * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bggk;
            } else if (TERM == 2) {
                // src/NNMap_Model.cu:787-856
                const Slot64 &M1 = *s[3], &M2 = *s[4];
                const double m1 = M1.a[0], m2 = M2.a[0];
                const double Pk1 = ax ? ax[1] : plin64(T, z_ix, k1);
                const double Pk2 = ax ? ax[2] : plin64(T, z_ix, k2);
                const double Pk3 = ax ? ax[3] : plin64(T, z_ix, k3);
                const double ra = r200_64(m1, rhot), rb = r200_64(m2, rhot);
                const double ca = __ldg(T.conc + z_it * Nm + M1.i1);
                const double cb = __ldg(T.conc + z_it * Nm + M2.i1);
                const double u3_1 = u3c ? u3c[0] : u_nfw64(k3, ra, ca, 1);
                const double u3_2 = u3c ? u3c[1] : u_nfw64(k3, rb, cb, 1);
                const double u1_1 = uc ? uc[0] : u_nfw64(k1, ra, ca, f1);
                const double u2_1 = uc ? uc[1] : u_nfw64(k2, ra, ca, f2);
                const double u1_2 = uc ? uc[2] : u_nfw64(k1, rb, cb, f1);
                const double u2_2 = uc ? uc[3] : u_nfw64(k2, rb, cb, f2);
                // G_gg(k1, k2, m2)
                const double Ggg = M2.a[1] * M2.a[4] * u2_2 + M2.a[3] * M2.a[2] * u1_2 +
                                   M2.a[5] * u1_2 * u2_2;
                const double Gg_k1m1 = M1.a[1] + M1.a[2] * u1_1;  // hod1 at m1
                const double Gg_k2m2 = M2.a[3] + M2.a[4] * u2_2;  // hod2 at m2
                const double Gg_k2m1 = M1.a[3] + M1.a[4] * u2_1;  // hod2 at m1
                const double Gg_k1m2 = M2.a[1] + M2.a[2] * u1_2;  // hod1 at m2
                double Bggd = 1. / nbar1 / nbar2 / rho * __ldg(T.hmf + z_ix * Nm + M1.i0) *
                              __ldg(T.hmf + z_ix * Nm + M2.i0) * __ldg(T.b_h + z_ix * Nm + M1.i0) *
                              __ldg(T.b_h + z_ix * Nm + M2.i0) *
                              (m1 * u3_1 * Ggg * Pk3 + m2 * u3_2 * Gg_k1m1 * Gg_k2m2 * Pk1 +
                               m2 * u3_2 * Gg_k2m1 * Gg_k1m2 * Pk2);
                double bggk = 1. / __ldg(T.dwdz + z_ix) * __ldg(T.g + z_ix) * __ldg(T.p1 + z_ix) *
                              __ldg(T.p2 + z_ix) / w_ / w_ / w_ * (1. + z) * Bggd;
                return l1 * l2 * m1 * m2 * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bggk;
            } else {
                // src/NNMap_Model.cu:1003-1037
                const Slot64 &M1 = *s[3], &M2 = *s[4], &M3 = *s[5];
                const double m1 = M1.a[0], m2 = M2.a[0], m3 = M3.a[0];
                const double u3 = u3c ? u3c[0]
                                      : u_nfw64(k3, r200_64(m3, rhot), __ldg(T.conc + z_it * Nm + M3.i1), 1);
                const double u1 = uc ? uc[0] : u_nfw64(k1, r200_64(m1, rhot), __ldg(T.conc + z_it * Nm + M1.i1), f1);
                const double u2 = uc ? uc[1] : u_nfw64(k2, r200_64(m2, rhot), __ldg(T.conc + z_it * Nm + M2.i1), f2);
                const double Gg1 = M1.a[1] + M1.a[2] * u1;  // hod1 at m1
                const double Gg2 = M2.a[3] + M2.a[4] * u2;  // hod2 at m2
                double Bggd = 1. / nbar1 / nbar2 / rho * __ldg(T.hmf + z_ix * Nm + M1.i0) *
                              __ldg(T.hmf + z_ix * Nm + M2.i0) * __ldg(T.hmf + z_ix * Nm + M3.i0) *
                              m3 * u3 * Gg1 * Gg2 * (ax ? ax[1] : bi_lin64(T, k1, k2, cphi, z_ix)) *
                              __ldg(T.b_h + z_ix * Nm + M1.i0) * __ldg(T.b_h + z_ix * Nm + M2.i0) *
                              __ldg(T.b_h + z_ix * Nm + M3.i0);
                double bggk = Bggd / __ldg(T.dwdz + z_ix) * __ldg(T.g + z_ix) * __ldg(T.p1 + z_ix) *
                              __ldg(T.p2 + z_ix) / w_ / w_ / w_ * (1. + z);
                return l1 * l2 * m1 * m2 * m3 * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bggk;
            }
        } else {
            const double nbar = __ldg(T.nbar + d.hod1 * T.Nz + z_ix);
            const double f = f1;
            const double gz = __ldg(T.g + z_ix);
            if (TERM == 1) {
                // src/NMapMap_Model.cu:263-301
                const Slot64 &M = *s[3];
                const double m = M.a[0];
                const double r2 = mz ? mz[0] : r200_64(m, rhot);  // mz[0] is this value
                const double cc = __ldg(T.conc + z_it * Nm + M.i1);
                double Bgdd = 1. / nbar / rho / rho * __ldg(T.hmf + z_ix * Nm + M.i0) * m * m *
                              (M.a[1] + M.a[2] * (uc ? uc[0] : u_nfw64(k1, r2, cc, f))) *
                              (uc ? uc[1] : u_nfw64(k2, r2, cc, 1)) *
                              (mz ? u_nfw64_F(k3, mz[0], 1.0 * cc, mz[1]) : u_nfw64(k3, r2, cc, 1));
                double bgkk = Bgdd / __ldg(T.dwdz + z_ix) * gz * gz * __ldg(T.p1 + z_ix) / w_ / w_ *
                              (1. + z) * (1. + z);
                return l1 * l2 * m * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bgkk / nbar;
            } else if (TERM == 2) {
                // src/NMapMap_Model.cu:402-468
                const Slot64 &M1 = *s[3], &M2 = *s[4];
                const double m1 = M1.a[0], m2 = M2.a[0];
                const double Pk1 = ax ? ax[1] : plin64(T, z_ix, k1);
                const double Pk2 = ax ? ax[2] : plin64(T, z_ix, k2);
                const double Pk3 = ax ? ax[3] : plin64(T, z_ix, k3);
                const double ra = r200_64(m1, rhot), rb = r200_64(m2, rhot);
                const double ca = __ldg(T.conc + z_it * Nm + M1.i1);
                const double cb = __ldg(T.conc + z_it * Nm + M2.i1);
                const double u2_1 = uc ? uc[0] : u_nfw64(k2, ra, ca, 1);
                const double u3_2 = u3c ? u3c[1] : u_nfw64(k3, rb, cb, 1);
                const double u1_2f = uc ? uc[1] : u_nfw64(k1, rb, cb, f);
                const double u3_1 = u3c ? u3c[0] : u_nfw64(k3, ra, ca, 1);
                const double u2_2 = uc ? uc[2] : u_nfw64(k2, rb, cb, 1);
                const double u1_1f = uc ? uc[3] : u_nfw64(k1, ra, ca, f);
                double Bgdd = 1. / nbar / rho / rho * __ldg(T.hmf + z_ix * Nm + M1.i0) *
                              __ldg(T.hmf + z_ix * Nm + M2.i0) * __ldg(T.b_h + z_ix * Nm + M1.i0) *
                              __ldg(T.b_h + z_ix * Nm + M2.i0) *
                              (m1 * m2 * u2_1 * u3_2 * (M2.a[1] + M2.a[2] * u1_2f) * Pk2 +
                               m1 * m2 * u3_1 * u2_2 * (M2.a[1] + M2.a[2] * u1_2f) * Pk3 +
                               m2 * m2 * u2_1 * u3_2 * (M1.a[1] + M1.a[2] * u1_1f) * Pk1);
                double bgkk = Bgdd / __ldg(T.dwdz + z_ix) * gz * gz * __ldg(T.p1 + z_ix) / w_ / w_ *
                              (1. + z) * (1. + z);
                return l1 * l2 * m1 * m2 * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bgkk / nbar;
            } else {
                // src/NMapMap_Model.cu:592-632 (Nc, Ns at m3; u_NFW(k1, m2, f))
                const Slot64 &M1 = *s[3], &M2 = *s[4], &M3 = *s[5];
                const double m1 = M1.a[0], m2 = M2.a[0], m3 = M3.a[0];
                const double ra = r200_64(m1, rhot), rb = r200_64(m2, rhot);
                const double ca = __ldg(T.conc + z_it * Nm + M1.i1);
                const double cb = __ldg(T.conc + z_it * Nm + M2.i1);
                double Bgdd = 1. / nbar / rho / rho * __ldg(T.hmf + z_ix * Nm + M1.i0) *
                              __ldg(T.hmf + z_ix * Nm + M2.i0) * __ldg(T.hmf + z_ix * Nm + M3.i0) *
                              __ldg(T.b_h + z_ix * Nm + M1.i0) * __ldg(T.b_h + z_ix * Nm + M2.i0) *
                              __ldg(T.b_h + z_ix * Nm + M3.i0) * m1 * m2 *
                              (uc ? uc[0] : u_nfw64(k2, ra, ca, 1)) *
                              (u3c ? u3c[0] : u_nfw64(k3, rb, cb, 1)) *
                              (M3.a[1] + M3.a[2] * (uc ? uc[1] : u_nfw64(k1, rb, cb, f))) *
                              (ax ? ax[1] : bi_lin64(T, k1, k2, cphi, z_ix));
                double bgkk = Bgdd / __ldg(T.dwdz + z_ix) * gz * gz * __ldg(T.p1 + z_ix) / w_ / w_ *
                              (1. + z) * (1. + z);
                return l1 * l2 * m1 * m2 * m3 * l1 * l2 * L1.a[1] * L2.a[1] * U3 * bgkk / nbar;
            }
        }
    }
};

// Rule sums of one region in the reference's order (src/hcubature.cpp:512-576).
template <int DIM>
__device__ void combine64(const double *v, double vol, double &val, double &err, int &split)
{
    const double ratio = (G3L_LAMBDA2 * G3L_LAMBDA2) / (G3L_LAMBDA4 * G3L_LAMBDA4);
    const double weight1 = (double)(12824 - 9120 * DIM + 400 * DIM * DIM) / (double)19683;
    const double weight3 = (double)(1820 - 400 * DIM) / (double)19683;
    const double weight5 = (double)6859 / (double)19683 / (double)(1u << DIM);
    const double weightE1 = (double)(729 - 950 * DIM + 50 * DIM * DIM) / (double)729;
    const double weightE3 = (double)(265 - 100 * DIM) / (double)1458;
    const double weight2 = 980. / 6561., weight4 = 200. / 19683.;
    const double weightE2 = 245. / 486., weightE4 = 25. / 729.;
    double val0 = v[0], sum2 = 0, sum3 = 0, sum4 = 0, sum5 = 0;
    double maxdiff = 0;
    int dimDiffMax = 0;
    int k0 = 1;
    for (int k = 0; k < DIM; ++k) {
        double v0 = v[k0 + 4 * k], v1 = v[k0 + 4 * k + 1];
        double v2 = v[k0 + 4 * k + 2], v3 = v[k0 + 4 * k + 3];
        sum2 += v0 + v1;
        sum3 += v2 + v3;
        double diff = 0;
        diff += fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
        if (diff > maxdiff) {
            maxdiff = diff;
            dimDiffMax = k;
        }
    }
    k0 += 4 * DIM;
    for (int k = 0; k < 2 * DIM * (DIM - 1); ++k) sum4 += v[k0 + k];
    k0 += 2 * DIM * (DIM - 1);
    for (int k = 0; k < (1 << DIM); ++k) sum5 += v[k0 + k];
    double result = vol * (weight1 * val0 + weight2 * sum2 + weight3 * sum3 + weight4 * sum4 +
                           weight5 * sum5);
    double res5th = vol * (weightE1 * val0 + weightE2 * sum2 + weightE3 * sum3 + weightE4 * sum4);
    val = result;
    err = fabs(res5th - result);
    split = dimDiffMax;
}

// One work item on one warp: `cut` = bisect the region at pslot along its split
// dimension into pslot (lower half) and qslot (upper half) and evaluate both;
// otherwise evaluate the region at pslot in place (roots, FP64 re-evaluation).
template <int KIND, int TERM>
__device__ void warp_item64(const DevTables &T, const IntDesc &d, const Pool &P, long long pslot,
                            long long qslot, bool cut, Slot64 *slots, double *vals,
                            const uint32_t *sdesc, unsigned long long *ties, double *dbg)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    const int lane = threadIdx.x & 31;
    const long long stride = P.stride;
    const int sdim = cut ? P.split[pslot] : 0;
    const int nchild = cut ? 2 : 1;
    double c_l = 0;
    int lev = 0;
    if (lane < DIM) {
        c_l = P.center[lane * stride + pslot];
        lev = P.level[lane * stride + pslot];
    }
    double cL = 0, cR = 0;
    const int levs = __shfl_sync(0xffffffffu, lev, sdim) + (cut ? 1 : 0);
    const double cs = __shfl_sync(0xffffffffu, c_l, sdim);
    const double hws = ldexp(d.hw0[sdim], -levs);
    if (cut) {
        cL = cs - hws;
        cR = cs + hws;
    }
    const int levsum = __reduce_add_sync(0xffffffffu, lane < DIM ? lev : 0) + (cut ? 1 : 0);
    // coordinate variant slots: dims 0..DIM-1 of child 0, then dim sdim of child 1
    const int nslot = (DIM + nchild - 1) * NVAR;
    for (int t = lane; t < nslot; t += 32) {
        int dd = t / NVAR, v = t - dd * NVAR;
        int dim = dd < DIM ? dd : sdim;
        double c = P.center[dim * stride + pslot];
        int L = P.level[dim * stride + pslot];
        if (cut && dim == sdim) {
            L += 1;
            c = (dd < DIM) ? cL : cR;
        }
        double hw = ldexp(d.hw0[dim], -L);
        double x = c;
        if (v > 0) {
            double lam = (v <= 2) ? G3L_LAMBDA2 : (v <= 4 ? G3L_LAMBDA4 : G3L_LAMBDA5);
            double r = hw * lam;
            x = (v & 1) ? c - r : c + r;
        }
        Model64<KIND, TERM>::fill(T, d, dim, x, slots[t], ties);
    }
    __syncwarp();
    for (int p = lane; p < nchild * NP; p += 32) {
        int ch = p >= NP ? 1 : 0;
        int pp = p - ch * NP;
        uint32_t vv = sdesc[pp];
        const Slot64 *sp[DIM];
#pragma unroll
        for (int dd = 0; dd < DIM; ++dd) {
            int v = (vv >> (3 * dd)) & 7;
            sp[dd] = (ch && dd == sdim) ? &slots[DIM * NVAR + v] : &slots[dd * NVAR + v];
        }
        vals[p] = Model64<KIND, TERM>::point(T, d, sp);
        if (dbg) dbg[p] = vals[p];
    }
    __syncwarp();
    // rule sums: lane 0 -> child 0, lane 1 -> child 1
    if (lane < nchild) {
        double vol = ldexp(d.rootvol, -levsum);
        double val, err;
        int split;
        combine64<DIM>(vals + lane * NP, vol, val, err, split);
        long long slot = lane == 0 ? pslot : qslot;
        P.val[slot] = val;
        P.err[slot] = err;
        P.split[slot] = (unsigned char)split;
        if (P.unc) P.unc[slot] = 0.f;
        if (P.uval) P.uval[slot] = 0.f;
    }
    if (cut && lane < DIM) {
        double cnew = c_l;
        int lnew = lev;
        if (lane == sdim) {
            lnew = levs;
            cnew = cL;
        }
        P.center[lane * stride + pslot] = cnew;
        P.level[lane * stride + pslot] = (unsigned char)lnew;
        P.center[lane * stride + qslot] = lane == sdim ? cR : c_l;
        P.level[lane * stride + qslot] = (unsigned char)lnew;
    }
    __syncwarp();
}

template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_eval64(DevTables T, const IntDesc *__restrict__ D,
                                                IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                const long long *__restrict__ woff)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    constexpr int NSLOT = (DIM + 1) * NVAR;
    constexpr int WPB = 4;
    __shared__ uint32_t sdesc[NP];
    __shared__ Slot64 sslot[WPB][NSLOT];
    __shared__ double svals[WPB][2 * NP];
    const int g = KIND * 3 + TERM - 1;
    for (int p = threadIdx.x; p < NP; p += blockDim.x) sdesc[p] = point_variants(DIM, p);
    __syncthreads();
    const int wib = threadIdx.x >> 5;
    const int gb = H->gbeg[g], ge = H->gbeg[g + 1];
    if (gb >= ge) return;
    const long long wbeg = woff[gb], wend = woff[ge];
    const long long nwarps = (long long)gridDim.x * WPB;
    for (long long w = wbeg + (long long)blockIdx.x * WPB + wib; w < wend; w += nwarps) {
        int lo = gb, hi = ge - 1;  // last integral i with woff[i] <= w
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (woff[mid] <= w) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo;
        const long long j = w - woff[i];
        const IntDesc &d = D[i];
        const int cj = P.cand[d.base + j];
        const bool cut = cj >= 0;  // cj < 0: a fresh integral's root region
        const long long pslot = d.base + (cut ? cj : 0);
        const long long qslot = cut ? d.base + (S[i].nR - S[i].K) + j : -1;
        warp_item64<KIND, TERM>(T, d, P, pslot, qslot, cut, sslot[wib], svals[wib], sdesc,
                                &H->ties, H->dbg);
    }
}

static_assert(sizeof(Slot64) == reeval_slot_bytes, "re-evaluation scratch layout");

// FP64 re-evaluation of the regions the mixed-precision pass queued for one group; each
// entry is (integral, local slot | kind << 30): kind 0 = split decision only (the centre
// and the 4 dim axis points enter the fourth differences, src/hcubature.cpp:527-575),
// kind 1 = whole rule (value, error and split: ambiguous selection boundaries and the
// final polish).  The FP64 pipe issues one warp instruction per 64 cycles per SM
// sub-partition, so a round's re-evaluation time is set by the busiest sub-partition:
// the work is spread evenly over the whole device in three passes over the first
// P.rcap entries -- coordinate slots (one per thread), rule points (one per thread, each
// entry's points padded to whole warps) and the sums (one thread per entry, in the
// reference's order).  Entries beyond P.rcap take the batched kernel k_reeval64.
template <int KIND, int TERM>
struct Reeval {
    static constexpr int DIM = TERM + 4;
    static constexpr int NP = rule_points(DIM);
    static constexpr int NAX = 1 + 4 * DIM;
    static constexpr int NS = DIM * NVAR;
    static constexpr int NPAD = (NP + 31) / 32 * 32;
    static constexpr int G = KIND * 3 + TERM - 1;
    // the pass of cached values (measured faster for every term): the points then
    // evaluate no FP64 u_NFW of their own except the 1-halo terms' k3 one
    static constexpr bool UCACHE = true;
    // r_200 and F once per (mass, z) pair (k_re_fill) instead of per u_NFW call
    static constexpr bool MZ = UCACHE;
    __device__ static Slot64 *slots(const Pool &P)
    {
        return (Slot64 *)(P.rscr + (long long)G * P.rscr_group);
    }
    __device__ static double *vals(const Pool &P)
    {
        return (double *)(P.rscr + (long long)G * P.rscr_group +
                          ((long long)P.rcap * MAX_DIM * NVAR * reeval_slot_bytes + 255) / 256 * 256);
    }
    __device__ static double *ucv(const Pool &P)  // [rcap][UC_NF_MAX][UC_MAX]
    {
        return vals(P) + (long long)P.rcap * 256;
    }
    __device__ static double *u3v(const Pool &P)  // [rcap][U3_NF_MAX][U3_MAX]
    {
        return ucv(P) + (long long)P.rcap * UC_NF_MAX * UC_MAX;
    }
    __device__ static double *auxv(const Pool &P)  // [rcap][AUX_MAX]
    {
        return u3v(P) + (long long)P.rcap * U3_NF_MAX * U3_MAX;
    }
    __device__ static double *mzv(const Pool &P)  // [rcap][3][MZ_PAIRS][MZ_VALS]
    {
        return auxv(P) + (long long)P.rcap * AUX_MAX;
    }
    __device__ static double *mz(const Pool &P, int k, int mdim, uint32_t vv)
    {
        const int vm = (vv >> (3 * mdim)) & 7, vz = (vv >> (3 * (DIM - 1))) & 7;
        return mzv(P) + (((long long)k * 3 + (mdim - 3)) * MZ_PAIRS + mz_index(vm, vz)) * MZ_VALS;
    }
    // auxiliary values per entry (124 for the 2-halo terms)
    static constexpr int NAUX = aux_off(TERM, aux_nfun(TERM) - 1) + aux_count(TERM, aux_nfun(TERM) - 1);
    static_assert(NAUX <= AUX_MAX, "auxiliary projections exceed AUX_MAX");
    __device__ static int count(const Pool &P, const BatchHdr *H)
    {
        const int cap = H->esc_cap[G];
        const int n = H->n_esc[G] < cap ? H->n_esc[G] : cap;
        return n < P.rcap ? n : P.rcap;
    }
};

// Point tables of a group's re-evaluation passes: the point codes, the (l, m, z)
// combinations of the cached u_NFW (ucache_tables) and the projections of the k3 u_NFW
// (u3_tables) and of the auxiliary functions (aux_tables).  The same for every launch, so
// k_re_tables builds them once per context into P.retab and each block copies them to
// shared memory (building them per block cost more than the cached work saves).
template <int KIND, int TERM>
struct ReTab {
    static constexpr int DIM = TERM + 4, NP = rule_points(DIM), NF = ucache_nf(TERM);
    static constexpr int NU3 = u3_nfun(TERM) > 0 ? u3_nfun(TERM) : 1, NA = aux_nfun(TERM);
    uint32_t sdesc[NP];
    int ucn[NF];
    uint16_t ucl[NF * UC_MAX];
    uint8_t ucidx[NF * NP];
    uint8_t u3rep[NU3 * NP];
    uint8_t u3list[NU3 * U3_MAX];
    uint8_t auxrep[NA * NP];
    uint8_t auxlist[AUX_MAX];
};

template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_re_tables(unsigned char *out)
{
    using RT = ReTab<KIND, TERM>;
    static_assert(sizeof(RT) <= RETAB_BYTES && sizeof(RT) % 4 == 0, "re-evaluation table size");
    __shared__ __align__(16) unsigned char buf[sizeof(RT)];
    __shared__ uint8_t map[RT::NF * 343];
    RT &t = *reinterpret_cast<RT *>(buf);
    ucache_tables<KIND, TERM>(t.ucidx, t.ucl, t.ucn, map);
    for (int p = threadIdx.x; p < RT::NP; p += blockDim.x) t.sdesc[p] = point_variants(RT::DIM, p);
    __syncthreads();
    u3_tables<KIND, TERM>(t.sdesc, t.u3rep, t.u3list, map);  // map is free again
    aux_tables<TERM>(t.sdesc, t.auxrep, t.auxlist, map);
    uint32_t *dst = reinterpret_cast<uint32_t *>(out + (KIND * 3 + TERM - 1) * RETAB_BYTES);
    for (int i = threadIdx.x; i < (int)(sizeof(RT) / 4); i += blockDim.x)
        dst[i] = reinterpret_cast<const uint32_t *>(buf)[i];
}

// copy group (KIND, TERM)'s tables to shared memory buf (every thread calls it)
template <int KIND, int TERM>
__device__ inline const ReTab<KIND, TERM> &load_retab(const Pool &P, unsigned char *buf)
{
    using RT = ReTab<KIND, TERM>;
    const uint32_t *src =
        reinterpret_cast<const uint32_t *>(P.retab + (KIND * 3 + TERM - 1) * RETAB_BYTES);
    for (int i = threadIdx.x; i < (int)(sizeof(RT) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t *>(buf)[i] = __ldg(src + i);
    __syncthreads();
    return *reinterpret_cast<const RT *>(buf);
}

template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_re_fill(DevTables T, const IntDesc *__restrict__ D,
                                                 IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                 const long long *__restrict__ woff)
{
    using R = Reeval<KIND, TERM>;
    const int m = R::count(P, H);
    if (m == 0) return;
    const int2 *Q = P.esc + H->esc_beg[R::G];
    Slot64 *SL = R::slots(P);
    const long long stride = P.stride;
    const long long tot1 = (long long)m * R::NS;
    // then the (mass, z) pairs' r_200 and F, one thread each (their mass and bin from the
    // same expressions as the mass slot's)
    constexpr int NMZ = R::MZ ? TERM * MZ_PAIRS : 0;
    const long long tot = tot1 + (long long)m * NMZ;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        if (NMZ > 0 && t >= tot1) {
            constexpr int NMZ1 = NMZ > 0 ? NMZ : 1;
            const long long t2 = t - tot1;
            const int k = (int)(t2 / NMZ1), r = (int)(t2 - (long long)k * NMZ1);
            const int md = 3 + r / MZ_PAIRS, j = r - (md - 3) * MZ_PAIRS;
            const int vm = mz_vm_of(j), vz = mz_vz_of(j);
            const int2 ent = Q[k];
            const IntDesc &d = D[ent.x];
            constexpr int zd = R::DIM - 1;
            if (!(ent.y >> 30)) {  // split only: the centre and the contenders' axis variants
                const unsigned cm = split_cmask(P, d, ent);
                if ((vm && vz) || !split_variant(cm, md, vm) || !split_variant(cm, zd, vz)) continue;
            }
            const long long slot = d.base + (ent.y & 0x3FFFFFFF);
            Slot64 M;
            const double xm = variant_x(P.center[md * stride + slot],
                                        ldexp(d.hw0[md], -(int)P.level[md * stride + slot]), vm);
            M.a[0] = pow(10, xm);
            m_index(T, xm, M.a[0], M.i0, M.i1, nullptr);
            const int zt = z_trunc64(T, variant_x(P.center[zd * stride + slot],
                                                  ldexp(d.hw0[zd], -(int)P.level[zd * stride + slot]), vz));
            Model64<KIND, TERM>::mz_values(T, d, M, zt, KIND == 0 ? 3 : 2,
                                           R::mzv(P) + (((long long)k * 3 + (md - 3)) * MZ_PAIRS + j) * MZ_VALS);
            continue;
        }
        const int k = (int)(t / R::NS), r = (int)(t - (long long)k * R::NS);
        const int dim = r / NVAR, v = r - dim * NVAR;
        const int2 ent = Q[k];
        const IntDesc &d = D[ent.x];
        // split only: the centre of every dimension, the contenders' axis variants
        if (!(ent.y >> 30) && !split_variant(split_cmask(P, d, ent), dim, v)) continue;
        const long long slot = d.base + (ent.y & 0x3FFFFFFF);
        const double c = P.center[dim * stride + slot];
        const double hw = ldexp(d.hw0[dim], -(int)P.level[dim * stride + slot]);
        Model64<KIND, TERM>::fill(T, d, dim, variant_x(c, hw, v), SL[(long long)k * R::NS + r], &H->ties);
    }
}

// cached u_NFW of each entry's (l, m, z) combinations (whole rules: all of them; split
// only: those without corner variants, whose slots are not filled)
template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_re_ucache(DevTables T, const IntDesc *__restrict__ D,
                                                   IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                   const long long *__restrict__ woff)
{
    using R = Reeval<KIND, TERM>;
    constexpr int NF = ucache_nf(TERM);
    __shared__ __align__(16) unsigned char tbuf[sizeof(ReTab<KIND, TERM>)];
    const int m = R::count(P, H);
    if (m == 0 || !R::UCACHE) return;
    const long long tot1 = (long long)m * NF * UC_MAX;
    // the k3 u_NFW of each projection (2- and 3-halo terms): after the (l, m, z) ones
    const long long tot2 = tot1 + (long long)m * u3_nfun(TERM) * U3_MAX;
    // the auxiliary functions of each projection: last
    const long long tot = tot2 + (long long)m * R::NAUX;
    if ((long long)blockIdx.x * blockDim.x >= tot) return;  // no work here: skip the tables
    const ReTab<KIND, TERM> &tb = load_retab<KIND, TERM>(P, tbuf);
    const uint32_t *sdesc = tb.sdesc;
    const uint16_t *ucl = tb.ucl;
    const int *ucn = tb.ucn;
    const uint8_t *u3list = tb.u3list, *auxlist = tb.auxlist;
    const int2 *Q = P.esc + H->esc_beg[R::G];
    const Slot64 *SL = R::slots(P);
    double *UC = R::ucv(P);
    double *U3C = R::u3v(P);
    double *AX = R::auxv(P);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        if (t >= tot2) {
            const long long t3 = t - tot2;
            const int k = (int)(t3 / R::NAUX), r = (int)(t3 - (long long)k * R::NAUX);
            int a = 0;
            while (a + 1 < aux_nfun(TERM) && r >= aux_off(TERM, a + 1)) ++a;
            const int pr = auxlist[r];
            const int2 ent = Q[k];
            // split only: the projections of the centre and the contenders' axis points
            if (!(ent.y >> 30) && !split_point(split_cmask(P, D[ent.x], ent), pr, R::NAX)) continue;
            const uint32_t vv = sdesc[pr];
            const Slot64 *base = SL + (long long)k * R::NS;
            const Slot64 *sp[R::DIM];
#pragma unroll
            for (int dd = 0; dd < R::DIM; ++dd) sp[dd] = base + dd * NVAR + ((vv >> (3 * dd)) & 7);
            AX[(long long)k * AUX_MAX + r] = Model64<KIND, TERM>::aux(T, D[ent.x], a, sp);
            continue;
        }
        if (t >= tot1) {
            const long long t2 = t - tot1;
            const int k = (int)(t2 / (u3_nfun(TERM) * U3_MAX));
            const int r = (int)(t2 - (long long)k * u3_nfun(TERM) * U3_MAX);
            const int f = r / U3_MAX, j = r - f * U3_MAX;
            const int pr = u3list[f * U3_MAX + j];  // every projection index is used (93)
            const int2 ent = Q[k];
            if (!(ent.y >> 30) && !split_point(split_cmask(P, D[ent.x], ent), pr, R::NAX)) continue;
            const uint32_t vv = sdesc[pr];
            const Slot64 *base = SL + (long long)k * R::NS;
            const Slot64 *sp[R::DIM];
#pragma unroll
            for (int dd = 0; dd < R::DIM; ++dd) sp[dd] = base + dd * NVAR + ((vv >> (3 * dd)) & 7);
            U3C[((long long)k * U3_NF_MAX + f) * U3_MAX + j] =
                Model64<KIND, TERM>::u3(T, f, sp, R::MZ ? R::mz(P, k, u3_mass(KIND, TERM, f), vv) : nullptr);
            continue;
        }
        const int k = (int)(t / (NF * UC_MAX)), r = (int)(t - (long long)k * NF * UC_MAX);
        const int f = r / UC_MAX, j = r - f * UC_MAX;
        if (j >= ucn[f]) continue;
        const int2 ent = Q[k];
        const uint32_t key = ucl[f * UC_MAX + j];
        const int vl = key & 7, vm = (key >> 3) & 7, vz = (key >> 6) & 7;
        const int dl = ucache_fun(KIND, TERM, f, 0), dm = ucache_fun(KIND, TERM, f, 1);
        if (!(ent.y >> 30)) {  // split only: combinations of the centre and one contender axis
            const unsigned cm = split_cmask(P, D[ent.x], ent);
            if ((vl != 0) + (vm != 0) + (vz != 0) > 1 || !split_variant(cm, dl, vl) ||
                !split_variant(cm, dm, vm) || !split_variant(cm, R::DIM - 1, vz))
                continue;
        }
        const Slot64 *base = SL + (long long)k * R::NS;
        UC[((long long)k * UC_NF_MAX + f) * UC_MAX + j] = Model64<KIND, TERM>::ucached(
            T, D[ent.x], f, base[dl * NVAR + vl], base[dm * NVAR + vm], base[(R::DIM - 1) * NVAR + vz],
            R::MZ ? R::mz(P, k, dm, ((uint32_t)vm << (3 * dm)) | ((uint32_t)vz << (3 * (R::DIM - 1))))
                  : nullptr);
    }
}

template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_re_points(DevTables T, const IntDesc *__restrict__ D,
                                                   IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                   const long long *__restrict__ woff)
{
    using R = Reeval<KIND, TERM>;
    constexpr int DIM = R::DIM;
    constexpr int NF = ucache_nf(TERM);
    constexpr int NU3 = u3_nfun(TERM);
    constexpr int NA = aux_nfun(TERM);
    __shared__ __align__(16) unsigned char tbuf[sizeof(ReTab<KIND, TERM>)];
    const int m = R::count(P, H);
    if (m == 0) return;
    const long long tot = (long long)m * R::NPAD;
    if ((long long)blockIdx.x * blockDim.x >= tot) return;  // no work here: skip the tables
    const ReTab<KIND, TERM> &tb = load_retab<KIND, TERM>(P, tbuf);
    const uint32_t *sdesc = tb.sdesc;
    const uint8_t *ucidx = tb.ucidx, *u3rep = tb.u3rep, *auxrep = tb.auxrep;
    const double *U3C = R::u3v(P);
    const double *AX = R::auxv(P);
    const int2 *Q = P.esc + H->esc_beg[R::G];
    const Slot64 *SL = R::slots(P);
    double *VL = R::vals(P);
    const double *UC = R::ucv(P);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t / R::NPAD), p = (int)(t - (long long)k * R::NPAD);
        const int2 ent = Q[k];
        if (p >= R::NP) continue;
        const IntDesc &d = D[ent.x];
        if (!(ent.y >> 30) && !split_point(split_cmask(P, d, ent), p, R::NAX)) continue;
        const uint32_t vv = sdesc[p];
        const Slot64 *base = SL + (long long)k * R::NS;
        const Slot64 *sp[DIM];
#pragma unroll
        for (int dd = 0; dd < DIM; ++dd) sp[dd] = base + dd * NVAR + ((vv >> (3 * dd)) & 7);
        double uc[NF];
        if (R::UCACHE) {
#pragma unroll
            for (int f = 0; f < NF; ++f)
                uc[f] = UC[((long long)k * UC_NF_MAX + f) * UC_MAX + ucidx[f * R::NP + p]];
        }
        double u3c[NU3 > 0 ? NU3 : 1];
        if (R::UCACHE) {
#pragma unroll
            for (int f = 0; f < NU3; ++f)
                u3c[f] = U3C[((long long)k * U3_NF_MAX + f) * U3_MAX + u3rep[f * R::NP + p]];
        }
        double ax[NA];
        if (R::UCACHE) {
#pragma unroll
            for (int a = 0; a < NA; ++a)
                ax[a] = AX[(long long)k * AUX_MAX + aux_off(TERM, a) + auxrep[a * R::NP + p]];
        }
        VL[(long long)k * R::NPAD + p] = Model64<KIND, TERM>::point(
            T, d, sp, R::UCACHE ? uc : nullptr, (R::UCACHE && NU3 > 0) ? u3c : nullptr,
            R::UCACHE ? ax : nullptr, (R::MZ && TERM == 1) ? R::mz(P, k, 3, vv) : nullptr);
    }
}

// the sums of one re-evaluated region (vl: its rule-point values)
template <int DIM>
__device__ void reeval_finish(const IntDesc &d, const Pool &P, long long slot, bool full,
                              const double *vl, unsigned cm)
{
    const long long stride = P.stride;
    if (full) {
        int lsum = 0;
        for (int q = 0; q < DIM; ++q) lsum += P.level[q * stride + slot];
        double val, err;
        int split;
        combine64<DIM>(vl, ldexp(d.rootvol, -lsum), val, err, split);
        P.val[slot] = val;
        P.err[slot] = err;
        P.split[slot] = (unsigned char)split;
        P.unc[slot] = 0.f;
        P.uval[slot] = 0.f;
    } else {
        const double ratio = (G3L_LAMBDA2 * G3L_LAMBDA2) / (G3L_LAMBDA4 * G3L_LAMBDA4);
        const double val0 = vl[0];
        double maxdiff = 0;
        int dimDiffMax = 0;
        for (int q = 0; q < DIM; ++q) {
            if (!((cm >> q) & 1u)) continue;  // not a contender (its points were not taken)
            double v0 = vl[1 + 4 * q], v1 = vl[2 + 4 * q];
            double v2 = vl[3 + 4 * q], v3 = vl[4 + 4 * q];
            double diff = 0;
            diff += fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
            if (diff > maxdiff) {
                maxdiff = diff;
                dimDiffMax = q;
            }
        }
        P.split[slot] = (unsigned char)dimDiffMax;
    }
}

template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_re_combine(DevTables T, const IntDesc *__restrict__ D,
                                                    IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                    const long long *__restrict__ woff)
{
    using R = Reeval<KIND, TERM>;
    const int m = R::count(P, H);
    const int2 *Q = P.esc + H->esc_beg[R::G];
    const double *VL = R::vals(P);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const int2 ent = Q[k];
        const IntDesc &d = D[ent.x];
        reeval_finish<R::DIM>(d, P, d.base + (ent.y & 0x3FFFFFFF), (ent.y >> 30) != 0,
                              VL + (long long)k * R::NPAD, (ent.y >> 30) ? 0u : split_cmask(P, d, ent));
    }
}

// Entries beyond P.rcap: a block takes a batch of RB entries and spreads their slots and
// points over its threads (shared-memory staging, no scratch).
template <int KIND, int TERM>
__global__ void __launch_bounds__(128) k_reeval64(DevTables T, const IntDesc *__restrict__ D,
                                                  IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                  const long long *__restrict__ woff)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    constexpr int NAX = 1 + 4 * DIM;
    constexpr int RB = 4;  // entries per batch
    constexpr int NS = DIM * NVAR;
    __shared__ uint32_t sdesc[NP];
    __shared__ Slot64 slots[RB][NS];
    __shared__ double vals[RB][NP];
    __shared__ int2 sent[RB];
    const int g = KIND * 3 + TERM - 1;
    const int cap = H->esc_cap[g];
    const int n = H->n_esc[g] < cap ? H->n_esc[g] : cap;
    const int first = P.rcap;
    if (n <= first) return;
    for (int p = threadIdx.x; p < NP; p += blockDim.x) sdesc[p] = point_variants(DIM, p);
    const int2 *Q = P.esc + H->esc_beg[g];
    const long long stride = P.stride;
    const int nb = (n - first + RB - 1) / RB;
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const int e0 = first + b * RB;
        const int ne = n - e0 < RB ? n - e0 : RB;
        __syncthreads();
        if (threadIdx.x < ne) sent[threadIdx.x] = Q[e0 + threadIdx.x];
        __syncthreads();
        for (int t = threadIdx.x; t < ne * NS; t += blockDim.x) {
            const int k = t / NS, r = t - k * NS;
            const int dim = r / NVAR, v = r - dim * NVAR;
            const int2 ent = sent[k];
            const IntDesc &d = D[ent.x];
            if (!(ent.y >> 30) && !split_variant(split_cmask(P, d, ent), dim, v)) continue;
            const long long slot = d.base + (ent.y & 0x3FFFFFFF);
            const double c = P.center[dim * stride + slot];
            const double hw = ldexp(d.hw0[dim], -(int)P.level[dim * stride + slot]);
            double x = c;
            if (v > 0) {
                double lam = (v <= 2) ? G3L_LAMBDA2 : (v <= 4 ? G3L_LAMBDA4 : G3L_LAMBDA5);
                double rr = hw * lam;
                x = (v & 1) ? c - rr : c + rr;
            }
            Model64<KIND, TERM>::fill(T, d, dim, x, slots[k][r], &H->ties);
        }
        __syncthreads();
        int pb[RB + 1];
        pb[0] = 0;
#pragma unroll
        for (int k = 0; k < RB; ++k)
            pb[k + 1] = pb[k] + (k < ne ? ((sent[k].y >> 30) ? NP : NAX) : 0);
        for (int t = threadIdx.x; t < pb[RB]; t += blockDim.x) {
            int k = 0;
#pragma unroll
            for (int q = 1; q < RB; ++q) k += t >= pb[q] ? 1 : 0;
            const int p = t - pb[k];
            const IntDesc &d = D[sent[k].x];
            if (!(sent[k].y >> 30) && !split_point(split_cmask(P, d, sent[k]), p, NAX)) continue;
            const uint32_t vv = sdesc[p];
            const Slot64 *sp[DIM];
#pragma unroll
            for (int dd = 0; dd < DIM; ++dd) sp[dd] = &slots[k][dd * NVAR + ((vv >> (3 * dd)) & 7)];
            vals[k][p] = Model64<KIND, TERM>::point(T, d, sp);
        }
        __syncthreads();
        if (threadIdx.x < ne) {
            const int2 ent = sent[threadIdx.x];
            const IntDesc &d = D[ent.x];
            reeval_finish<DIM>(d, P, d.base + (ent.y & 0x3FFFFFFF), (ent.y >> 30) != 0,
                               vals[threadIdx.x], (ent.y >> 30) ? 0u : split_cmask(P, d, ent));
        }
    }
}

#define G3L_INST64(K, Tm)                                                                        \
    template __global__ void k_eval64<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,      \
                                             BatchHdr *, const long long *);                     \
    template __global__ void k_reeval64<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,    \
                                               BatchHdr *, const long long *);                   \
    template __global__ void k_re_fill<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,     \
                                              BatchHdr *, const long long *);                    \
    template __global__ void k_re_ucache<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,   \
                                                BatchHdr *, const long long *);                  \
    template __global__ void k_re_points<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,   \
                                                BatchHdr *, const long long *);                  \
    template __global__ void k_re_combine<K, Tm>(DevTables, const IntDesc *, IntState *, Pool,  \
                                                 BatchHdr *, const long long *);                 \
    template __global__ void k_re_tables<K, Tm>(unsigned char *);
G3L_INST64(0, 1)
G3L_INST64(0, 2)
G3L_INST64(0, 3)
G3L_INST64(1, 1)
G3L_INST64(1, 2)
G3L_INST64(1, 3)

// Build the re-evaluation point tables of every group into out (NGROUPS * RETAB_BYTES
// bytes of device memory), on stream s.
cudaError_t build_reeval_tables(unsigned char *out, cudaStream_t s)
{
    k_re_tables<0, 1><<<1, 128, 0, s>>>(out);
    k_re_tables<0, 2><<<1, 128, 0, s>>>(out);
    k_re_tables<0, 3><<<1, 128, 0, s>>>(out);
    k_re_tables<1, 1><<<1, 128, 0, s>>>(out);
    k_re_tables<1, 2><<<1, 128, 0, s>>>(out);
    k_re_tables<1, 3><<<1, 128, 0, s>>>(out);
    return cudaGetLastError();
}

// re-evaluation kernels of a group: 0 = fill, 1 = cached u_NFW, 2 = points, 3 = combine,
// 4 = batched tail
void *reeval_phase_kernel(int kind, int term, int phase)
{
#define G3L_RE_ROW(K, Tm)                                                                       \
    {(void *)k_re_fill<K, Tm>, (void *)k_re_ucache<K, Tm>, (void *)k_re_points<K, Tm>,           \
     (void *)k_re_combine<K, Tm>, (void *)k_reeval64<K, Tm>}
    static void *tab[2][3][5] = {{G3L_RE_ROW(0, 1), G3L_RE_ROW(0, 2), G3L_RE_ROW(0, 3)},
                                 {G3L_RE_ROW(1, 1), G3L_RE_ROW(1, 2), G3L_RE_ROW(1, 3)}};
#undef G3L_RE_ROW
    return tab[kind][term - 1][phase];
}

void *reeval64_kernel(int kind, int term)
{
    static void *tab[2][3] = {
        {(void *)k_reeval64<0, 1>, (void *)k_reeval64<0, 2>, (void *)k_reeval64<0, 3>},
        {(void *)k_reeval64<1, 1>, (void *)k_reeval64<1, 2>, (void *)k_reeval64<1, 3>}};
    return tab[kind][term - 1];
}

void *eval64_kernel(int kind, int term)
{
    static void *tab[2][3] = {
        {(void *)k_eval64<0, 1>, (void *)k_eval64<0, 2>, (void *)k_eval64<0, 3>},
        {(void *)k_eval64<1, 1>, (void *)k_eval64<1, 2>, (void *)k_eval64<1, 3>}};
    return tab[kind][term - 1];
}

}  // namespace g3l
