// g3l_device.cuh -- data layout shared by the engine kernels.
//
// Region pool (per call, in HBM, structure of arrays):
//   center[d * stride + slot]  FP64 region centre per dimension
//   level [d * stride + slot]  bisection depth per dimension; the half-width is
//                              hw0[d] * 2^-level exactly, and the reference's cached
//                              volume is rootvol * 2^-(sum of levels) exactly
//                              (compute_vol / cut_region, src/hcubature.cpp:134-141,
//                              206-218: halving and products scale exactly by 2)
//   val, err                   FP64 rule value and error of the region
//   split                      dimension to bisect next (src/hcubature.cpp:565-575); in the
//                              mixed pass bit 7 flags a split the FP32 values did not settle
// Integral i owns slots [base_i, base_i + cap_i); its live regions are the first nR_i.
#pragma once
#include <cstdint>

namespace g3l {

constexpr int MAX_DIM = 7;
constexpr int NVAR = 7;  // coordinate variants per dimension: c, c-+r2, c-+r4, c-+r5
constexpr int MAX_HOD_SLOTS = 1024;
constexpr int NGROUPS = 6;  // kind * 3 + (term - 1)
constexpr int UC_MAX = 1 + 12 + 12 + 8;  // (l, m, z) variant combinations of one rule
constexpr int UC_NF_MAX = 4;             // cached u_NFW functions per integrand at most

// status codes (mirror g3l_status)
enum : int {
    ST_OK = 0, ST_INVALID = 1, ST_CUDA = 2, ST_NOMEM = 3, ST_POOL = 4, ST_NONFINITE = 5,
    ST_CANCELLED = 6, ST_ROUNDS = 7, ST_DEADLINE = 10
};

// Genz-Malik degree 7/5 rule (Genz & Malik 1983; src/hcubature.cpp:458-466).
// lambda2 = sqrt(9/70), lambda4 = sqrt(9/10), lambda5 = sqrt(9/19).
#define G3L_LAMBDA2 0.3585685828003180919906451539079374954541
#define G3L_LAMBDA4 0.9486832980505137995996680633298155601160
#define G3L_LAMBDA5 0.6882472016116852977216287342936235251269

__host__ __device__ constexpr int rule_points(int dim)
{
    return 1 + 4 * dim + 2 * dim * (dim - 1) + (1 << dim);
}

// Tables and model scalars, passed by value to every kernel.
struct DevTables {
    int Nz, Nm, Nk, clamp_k;
    double zmin, zmax, mmin, mmax, kmin, kmax;
    double ln_mratio, ln_kratio;  // log(mmax/mmin), log(kmax/kmin)
    double m_x0, m_scale;         // m index ~ (log10 m - m_x0) * m_scale
    double A, eps;                // satellite-pair correlation
    const double *g, *p1, *p2, *w, *dwdz, *rho_bar;  // [Nz]
    const double *hmf, *b_h, *conc;                  // [Nz*Nm]
    const double *P_lin;                             // [Nz*Nk]
    const double *nbar;                              // [slot][Nz]
    const double *hod;                               // [slot][6] f, alpha, Mth, sigma, M', beta
    const double *scale;   // [slot][Nm] satellite-variance rescaling s (1 = none)
    const float *f_scale;  // [slot][Nm] s^2 - 1 in FP32 (mixed path)
    // exact nearest-bin indices of the tie-prone m-centre values, resolved on the
    // host with the reference's own expression (sorted by bit pattern)
    const unsigned long long *tie_m_bits;
    const int *tie_m_round, *tie_m_trunc;
    int n_tie_m;
    // mixed-precision path: FP32 tables in scaled units (see evalmx_impl.cuh)
    const float *f_hmf, *f_bh, *f_conc, *f_plin;  // [Nz*Nm] x3, [Nz*Nk]
    const float *f_zA, *f_zB, *f_kw, *f_k200;      // [Nz]
    const float *f_nbar;                           // [slot][Nz]
    const float *f_hodp;                           // [slot][8]
    const float2 *f_kb;                            // [Nz] (ln w + ln kmin) Nk / ln(kmax/kmin)
    float2 k_a, m_s2, m_x02, z_s2, z_02, lnkmin2, kscale2;  // double-float constants
    float fA, feps, small_arg;
    float unc_eps, unc_abs;        // FP32 point-value error bound (decisions)
    float unc_val_ratio;           // value-noise bound / decision bound
    float unc_sel_ratio;           // error-estimate bound (selection) / decision bound
    double tau_impact, tau_sel;    // escalation thresholds (fraction of the integral)
    double tau_val;                // bound on the FP32 noise left in a finished integral
    const unsigned long long *tie_z_bits;
    const int *tie_z_round, *tie_z_trunc;
    int n_tie_z;
};

struct IntDesc {
    double theta[3];
    double c0[MAX_DIM];   // root centre
    double hw0[MAX_DIM];  // root half-widths
    double rootvol;       // product of the root widths (FP64 rule)
    double rootvol_mx;    // mixed path: rootvol * FP32 integrand scale
    double rtol;
    double scale;         // mixed path: true value = scaled value * scale
    unsigned long long max_eval;
    long long base;       // first pool slot
    int cap;              // pool capacity in regions
    int hod1, hod2, same; // HOD slots; same = same-population branch
    int kind, term, dim, npts;
    int pad;
    float2 hwl[MAX_DIM][3];  // mixed path: hw0 * {lambda2, lambda4, lambda5} as double-floats
    float th_s[3];           // mixed path: theta * 1e3 (l in units of 1e3)
};

struct IntState {
    double val, err;
    unsigned long long neval;
    int nR, K, done, status, rounds, pad;  // pad: FP64 polish passes so far
    int defer, pad2;                       // defer: selection deferred in this round's first pass
};

struct Pool {
    double *center;
    unsigned char *level;
    double *val, *err;
    unsigned char *split;
    // mixed path: the dimensions whose fourth-difference bounds reach the leader's (bit
    // per dimension), written with an unsettled split; its FP64 re-take evaluates only
    // their axis points
    unsigned char *cmask;
    unsigned long long *q;  // fixed-point errors (selection scratch)
    int *cand;              // selected parents, per-integral segment at base
    float *unc;             // mixed path: bound on the FP32 error of err, relative (0 = FP64)
    float *uval;            // mixed path: bound on the FP32 error of val, relative (0 = FP64)
    double *key;            // selection scratch (polish keys |val| * uval)
    int2 *esc;              // regions queued for FP64 re-evaluation: (integral, local slot)
    long long stride;
    // FP64 re-evaluation scratch: per group, coordinate slots and rule-point values of the
    // first rcap queued entries of a round (later entries take the batched kernel)
    unsigned char *rscr;
    long long rscr_group;   // bytes per group
    int rcap;
    // the point tables of the re-evaluation passes, RETAB_BYTES per group (built once per
    // context by k_re_tables)
    const unsigned char *retab;
};
constexpr int RETAB_BYTES = 4096;

// u_NFW at k3 = |l1 + l2| / w with one halo mass (2- and 3-halo terms) does not depend
// on the other mass dimensions, so the rule points that differ only there share it:
// function f (u3_nfun(term) of them) uses mass dimension u3_mass(kind, term, f) and
// ignores the variant fields u3_drop(kind, term, f) of the point code.  Dropping one of 6
// or two of 7 dimensions leaves U3_MAX = rule_points(5) = 93 distinct projections.
constexpr int U3_MAX = 93;
constexpr int U3_NF_MAX = 2;
__host__ __device__ constexpr int u3_nfun(int term) { return term == 1 ? 0 : (term == 2 ? 2 : 1); }
__host__ __device__ constexpr int u3_mass(int kind, int term, int f)
{
    return term == 2 ? 3 + f : (kind == 0 ? 5 : 4);
}
__host__ __device__ constexpr uint32_t u3_drop(int kind, int term, int f)
{
    return term == 2 ? (7u << (3 * (4 - f)))
                     : (kind == 0 ? ((7u << 9) | (7u << 12)) : ((7u << 9) | (7u << 15)));
}

// Other quantities of a point that depend on a few of its dimensions only, cached per
// projection in the FP64 re-evaluation (function a of a term keeps the dimensions
// aux_dims(term, a), a bit per dimension): the aperture filter of l3 (l1, l2, phi) for
// every term; P_lin at k1 (l1, z), k2 (l2, z) and k3 (l1, l2, phi, z) for the 2-halo
// terms; the tree-level bispectrum (l1, l2, phi, z) for the 3-halo terms.  A projection
// onto k dimensions has rule_points(k) members (33, 17 or 57); function a's values are
// at [aux_off(term, a), + rule_points(k)) of the entry's AUX_MAX.
constexpr int AUX_MAX = 128;
__host__ __device__ constexpr int aux_nfun(int term) { return term == 1 ? 1 : (term == 2 ? 4 : 2); }
__host__ __device__ constexpr uint32_t aux_dims(int term, int a)
{
    return a == 0 ? 7u
                  : (term == 2 ? (a == 1 ? (1u | (1u << 5)) : a == 2 ? (2u | (1u << 5)) : (7u | (1u << 5)))
                               : (7u | (1u << 6)));
}
__host__ __device__ constexpr int aux_nkept(int term, int a)
{
    return a == 0 ? 3 : (term == 2 ? (a == 3 ? 4 : 2) : 4);
}
__host__ __device__ constexpr int aux_count(int term, int a) { return rule_points(aux_nkept(term, a)); }
__host__ __device__ constexpr int aux_off(int term, int a)
{
    return a == 0 ? 0 : aux_off(term, a - 1) + aux_count(term, a - 1);
}
__host__ __device__ constexpr uint32_t aux_keep(int term, int a)
{
    uint32_t k = 0;
    for (int d = 0; d < MAX_DIM; ++d)
        if ((aux_dims(term, a) >> d) & 1u) k |= 7u << (3 * d);
    return k;
}

// (mass, z) quantities of the FP64 re-evaluation: r_200 and the NFW normalisation
// F(c) = ln(1 + c) - c / (1 + c) at c = factor x concentration (factors 1, f of hod1, f of
// hod2) depend on one halo mass and z only.  Per mass dimension a rule's points take 17
// (mass variant, z variant) pairs -- the centre, the axis variants of either dimension
// with the other at the centre, the (+-r4, +-r4) pairs and the (+-r5, +-r5) corners --
// numbered by mz_index; mz_nz(vm) z variants go with mass variant vm, the i-th being
// mz_vz(vm, i).  Per entry: [mass dimension][MZ_PAIRS][MZ_VALS] doubles.
constexpr int MZ_PAIRS = 17;
constexpr int MZ_VALS = 4;  // r_200, F at factor 1, f of hod1, f of hod2
__host__ __device__ constexpr int mz_nz(int vm)
{
    return vm == 0 ? 5 : (vm <= 2 ? 1 : (vm <= 4 ? 3 : 2));
}
__host__ __device__ constexpr int mz_vz(int vm, int i)
{
    return vm == 0 ? i : (vm <= 2 ? 0 : (vm <= 4 ? (i == 0 ? 0 : 2 + i) : 5 + i));
}
__host__ __device__ constexpr int mz_vm_of(int j)
{
    return j < 5 ? 0 : (j < 7 ? j - 4 : (j < 13 ? 3 + (j - 7) / 3 : 5 + (j - 13) / 2));
}
__host__ __device__ constexpr int mz_vz_of(int j)
{
    return j < 5 ? j : (j < 7 ? 0 : (j < 13 ? ((j - 7) % 3 == 0 ? 0 : 2 + (j - 7) % 3) : 5 + (j - 13) % 2));
}
__host__ __device__ constexpr int mz_index(int vm, int vz)
{
    return vm == 0 ? vz
                   : (vm <= 2 ? 4 + vm
                              : (vm <= 4 ? 7 + 3 * (vm - 3) + (vz == 0 ? 0 : vz - 2)
                                         : 13 + 2 * (vm - 5) + (vz - 5)));
}

// An FP64 re-take of an unsettled split reads the centre and the axis points of the
// contending dimensions cm (bit per dimension) only.  Whether it needs coordinate
// variant v of dimension dim (the centre, or an axis variant of a contender):
__host__ __device__ inline bool split_variant(unsigned cm, int dim, int v)
{
    return v == 0 || (v < 5 && ((cm >> dim) & 1u));
}
// and rule point p (the centre, or an axis point of a contender; nax = 1 + 4 dim)
__host__ __device__ inline bool split_point(unsigned cm, int p, int nax)
{
    return p == 0 || (p < nax && ((cm >> ((p - 1) >> 2)) & 1u));
}

// Bytes of re-evaluation scratch per group for rcap entries (any term).
constexpr long long reeval_slot_bytes = 56;  // sizeof(Slot64)
__host__ __device__ constexpr long long reeval_scratch_group_bytes(int rcap)
{
    return ((long long)rcap * MAX_DIM * NVAR * reeval_slot_bytes + 255) / 256 * 256 +
           (long long)rcap * 256 * 8 + (long long)rcap * UC_NF_MAX * UC_MAX * 8 +
           (long long)rcap * U3_NF_MAX * U3_MAX * 8 + (long long)rcap * AUX_MAX * 8 +
           (long long)rcap * 3 * MZ_PAIRS * MZ_VALS * 8;
}

// Per-call header kept in device memory so one instantiated graph serves any batch.
struct BatchHdr {
    int n;                       // integrals (sorted by group)
    int gbeg[NGROUPS + 1];       // group g = integrals [gbeg[g], gbeg[g+1])
    int max_rounds;
    int cancel;                  // nonzero stops the loop at the next selection: 1 =
                                 //   cancelled, 2 = deadline passed (set by k_scan)
    int any_active;              // written by the scan kernel
    long long total_work;
    unsigned long long points;   // statistics
    unsigned long long ties;
    unsigned long long small_arg;
    unsigned long long regions;
    int rounds_done;
    int chunk_rounds;            // > 0: stop the device loop after this many rounds (serving)
    int chunk_count;             //   rounds run in the current launch
    int mixed;                   // 1: mixed-precision pass (uncertainty bookkeeping on)
    int n_esc[NGROUPS];          // FP64 re-evaluation queue of each group: fill,
    int esc_cap[NGROUPS];        //   capacity (the group's pool slots)
    long long esc_beg[NGROUPS];  //   and first entry in Pool::esc
    unsigned long long escalated;// statistics: regions re-evaluated in FP64
    unsigned long long deferred; // statistics: selections deferred for re-evaluation
    unsigned long long polished; // statistics: finished integrals polished in FP64
    unsigned long long esc_full; // statistics: whole-rule FP64 re-evaluations queued
    double *dbg;                 // debug: per-point integrand values of one work item
    // In-flight stop of a call: a host-mapped word the host sets from any thread
    // (nullptr: none), and a deadline on the device's global timer, measured from the
    // start of the loop (k_init); both are read once per round by k_scan.
    const volatile int *cancel_word;
    unsigned long long t0_ns;
    unsigned long long deadline_ns;  // 0 = none
    // Mixed precision, threshold decisions (convergence, the Gladwell count): multiplier
    // of the regions' FP32 bounds (0 = unguarded) and the value bounds' conversion to the
    // selection bounds' basis (eps_sel / eps_val)
    float thr_ratio, val_ratio;
    double tau_thr;                  //   checked only if the region moved carries > tau_thr |V|
    unsigned long long thr_checks;   // statistics: threshold decisions re-taken in FP64
};

__device__ __forceinline__ unsigned long long global_timer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// u_NFW calls of the integrands that depend on one l, one mass and z only.  The points
// of one Genz-Malik rule take at most UC_MAX distinct (l, m, z) variant combinations
// (the centre, 4 axis variants of each of the 3 dimensions, 4 (+-l4, +-l4) pairs of each
// of the 3 dimension pairs, the 8 corners), so these are evaluated once per
// combination.  ucache_fun(kind, term, f, k): function f's l dimension (k = 0), mass
// dimension (k = 1) and concentration factor (k = 2: 0 = 1, 1 = f of hod1, 2 = f of hod2).
__host__ __device__ constexpr int ucache_nf(int term) { return term == 2 ? 4 : 2; }
__host__ __device__ constexpr int ucache_fun(int kind, int term, int f, int k)
{
    // rows {l, m, factor}
    return kind == 0
               ? (term == 1 ? (f == 0 ? (k == 0 ? 0 : k == 1 ? 3 : 1) : (k == 0 ? 1 : k == 1 ? 3 : 2))
                  : term == 2 ? (f == 0 ? (k == 0 ? 0 : k == 1 ? 3 : 1)
                                 : f == 1 ? (k == 0 ? 1 : k == 1 ? 3 : 2)
                                 : f == 2 ? (k == 0 ? 0 : k == 1 ? 4 : 1)
                                          : (k == 0 ? 1 : k == 1 ? 4 : 2))
                              : (f == 0 ? (k == 0 ? 0 : k == 1 ? 3 : 1) : (k == 0 ? 1 : k == 1 ? 4 : 2)))
               : (term == 1 ? (f == 0 ? (k == 0 ? 0 : k == 1 ? 3 : 1) : (k == 0 ? 1 : k == 1 ? 3 : 0))
                  : term == 2 ? (f == 0 ? (k == 0 ? 1 : k == 1 ? 3 : 0)
                                 : f == 1 ? (k == 0 ? 0 : k == 1 ? 4 : 1)
                                 : f == 2 ? (k == 0 ? 1 : k == 1 ? 4 : 0)
                                          : (k == 0 ? 0 : k == 1 ? 3 : 1))
                              : (f == 0 ? (k == 0 ? 1 : k == 1 ? 3 : 0) : (k == 0 ? 0 : k == 1 ? 4 : 1)));
}

// Queue region `code` (local slot | whole-rule flag << 30) of integral i, group g, for
// FP64 re-evaluation in this round.
__device__ inline void push_esc(BatchHdr *H, const Pool &P, int g, int i, int code)
{
    const int k = atomicAdd(&H->n_esc[g], 1);
    if (k < H->esc_cap[g]) P.esc[H->esc_beg[g] + k] = make_int2(i, code);
    if (code >> 30) atomicAdd(&H->esc_full, 1ull);
}

// Point p of a dim-dimensional Genz-Malik rule -> coordinate variant of dim d,
// in the reference's generation order (src/hcubature.cpp:343-414, 476-503):
//   p = 0                   centre
//   p = 1 + 4k + s          axis k: s = 0..3 -> c-r2, c+r2, c-r4, c+r4
//   then the 2 dim (dim-1)  (+-r4, +-r4) pairs (i<j), order (-,-) (+,-) (+,+) (-,+)
//   then 2^dim corners      +-r5 in reflected Gray-code order, first all '+'
// variant codes: 0 c, 1 c-r2, 2 c+r2, 3 c-r4, 4 c+r4, 5 c-r5, 6 c+r5.
// Packed 3 bits per dimension.
__host__ __device__ inline uint32_t point_variants(int dim, int p)
{
    if (p == 0) return 0u;
    int q = p - 1;
    if (q < 4 * dim) {
        int k = q >> 2, s = q & 3;
        return (uint32_t)(s + 1) << (3 * k);
    }
    q -= 4 * dim;
    int nrr = 2 * dim * (dim - 1);
    if (q < nrr) {
        int pair = q >> 2, t = q & 3;
        int i = 0, rem = pair;
        while (rem >= dim - 1 - i) { rem -= dim - 1 - i; ++i; }
        int j = i + 1 + rem;
        uint32_t vi = (t == 1 || t == 2) ? 4u : 3u;
        uint32_t vj = (t >= 2) ? 4u : 3u;
        return (vi << (3 * i)) | (vj << (3 * j));
    }
    q -= nrr;
    uint32_t gray = (uint32_t)q ^ ((uint32_t)q >> 1);
    uint32_t out = 0;
    for (int d = 0; d < dim; ++d) out |= (((gray >> d) & 1u) ? 5u : 6u) << (3 * d);
    return out;
}

// Combination tables of one rule: ucl[f][j] = variants (l | m << 3 | z << 6) of
// combination j of function f (in key order), ucn[f] their count, ucidx[f][p] the
// combination of point p.  Block-cooperative (every thread of the block calls it; it
// synchronises); map is NF * 343 bytes of shared scratch.
template <int KIND, int TERM>
__device__ inline void ucache_tables(uint8_t *ucidx, uint16_t *ucl, int *ucn, uint8_t *map)
{
    constexpr int DIM = TERM + 4;
    constexpr int NP = rule_points(DIM);
    constexpr int NF = ucache_nf(TERM);
    auto key_of = [](int f, int p) -> uint32_t {
        const int dl = ucache_fun(KIND, TERM, f, 0), dm = ucache_fun(KIND, TERM, f, 1);
        const uint32_t vv = point_variants(DIM, p);
        return ((vv >> (3 * dl)) & 7) | (((vv >> (3 * dm)) & 7) << 3) |
               (((vv >> (3 * (DIM - 1))) & 7) << 6);
    };
    for (int i = threadIdx.x; i < NF * 343; i += blockDim.x) map[i] = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < NF * NP; t += blockDim.x) {
        const int f = t / NP, p = t - f * NP;
        const uint32_t k = key_of(f, p);
        map[f * 343 + (k & 7) + 7 * (((k >> 3) & 7) + 7 * (k >> 6))] = 1;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // number the present keys in key order
        const int lane = threadIdx.x;
        for (int f = 0; f < NF; ++f) {
            int base = 0;
            for (int c = 0; c < 343; c += 32) {
                const int q = c + lane;
                const bool on = q < 343 && map[f * 343 + q];
                const unsigned b = __ballot_sync(0xffffffffu, on);
                const int idx = base + __popc(b & ((1u << lane) - 1u));
                if (on && idx < UC_MAX) {
                    map[f * 343 + q] = (uint8_t)idx;
                    const int vl = q % 7, vm = (q / 7) % 7, vz = q / 49;
                    ucl[f * UC_MAX + idx] = (uint16_t)(vl | (vm << 3) | (vz << 6));
                }
                base += __popc(b);
            }
            if (lane == 0) ucn[f] = base < UC_MAX ? base : UC_MAX;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NF * NP; t += blockDim.x) {
        const int f = t / NP, p = t - f * NP;
        const uint32_t k = key_of(f, p);
        ucidx[t] = map[f * 343 + (k & 7) + 7 * (((k >> 3) & 7) + 7 * (k >> 6))];
    }
    __syncthreads();
}

// Projection tables: rep[p] is the projection of point p (its code & keep), numbered in
// order of first occurrence, list[j] the first point of projection j (at most maxn of
// them).  Block-cooperative (every thread calls it; it synchronises); sdesc holds the
// point codes (point_variants); tmp: 2 np bytes of shared scratch.
__device__ inline void proj_tables(const uint32_t *sdesc, int np, uint32_t keep, uint8_t *rep,
                                   uint8_t *list, int maxn, uint8_t *tmp)
{
    uint8_t *first = tmp, *cidx = tmp + np;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        const uint32_t key = sdesc[p] & keep;
        int q = 0;
        while (q < p && (sdesc[q] & keep) != key) ++q;
        first[p] = (uint8_t)q;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // number the projections in point order
        const int lane = threadIdx.x;
        int base = 0;
        for (int c = 0; c < np; c += 32) {
            const int q = c + lane;
            const bool on = q < np && first[q] == q;
            const unsigned b = __ballot_sync(0xffffffffu, on);
            const int idx = base + __popc(b & ((1u << lane) - 1u));
            if (on && idx < maxn) {
                cidx[q] = (uint8_t)idx;
                list[idx] = (uint8_t)q;
            }
            base += __popc(b);
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < np; p += blockDim.x) rep[p] = cidx[first[p]];
    __syncthreads();
}

// Projection tables of the k3 u_NFW (u3_drop), per function f: u3rep[f][NP], u3list[f][U3_MAX]
template <int KIND, int TERM>
__device__ inline void u3_tables(const uint32_t *sdesc, uint8_t *u3rep, uint8_t *u3list,
                                 uint8_t *tmp)
{
    constexpr int NP = rule_points(TERM + 4);
    for (int f = 0; f < u3_nfun(TERM); ++f)
        proj_tables(sdesc, NP, ~u3_drop(KIND, TERM, f), u3rep + f * NP, u3list + f * U3_MAX,
                    U3_MAX, tmp);
}

// Projection tables of the auxiliary caches, per function a: auxrep[a][NP] (index within
// the function's values), auxlist[aux_off(a) + j] (first point of projection j)
template <int TERM>
__device__ inline void aux_tables(const uint32_t *sdesc, uint8_t *auxrep, uint8_t *auxlist,
                                  uint8_t *tmp)
{
    constexpr int NP = rule_points(TERM + 4);
    for (int a = 0; a < aux_nfun(TERM); ++a)
        proj_tables(sdesc, NP, aux_keep(TERM, a), auxrep + a * NP, auxlist + aux_off(TERM, a),
                    aux_count(TERM, a), tmp);
}

}  // namespace g3l
