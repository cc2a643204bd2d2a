// engine.cu -- device-resident refinement loop of the adaptive cubature.
//
// The reference's loop (rulecubature with parallel=1, src/hcubature.cpp:938-989)
// pops regions from a max-heap keyed on the error until the error left in the
// heap is within tolerance or the evaluation budget is spent, bisects them,
// evaluates the children and pushes them back.  Here each round is
//   k_select : one CTA per integral.  Sums the live regions' values and errors,
//              applies the reference's stopping tests (numEval >= maxEval,
//              converged(): err <= |val| rtol, src/converged.h:10-14) and picks
//              the regions the heap would pop: the largest errors, in order,
//              until the remaining error is <= rtol |val| (Gladwell), capped by
//              the evaluation budget.  Both cut-offs are found with an MSD radix
//              select on the IEEE bit pattern of the errors; the running error
//              sums use 64-bit fixed point, so the choice is deterministic and
//              independent of thread scheduling.
//   k_scan   : prefix sum of the per-integral pop counts -> flat work list; sets
//              the graph's WHILE condition (no host round trip).
//   k_eval*  : cut + rule evaluation (eval_fp64.cu / evalmx_impl.cuh).
// Compiled with -fmad=false.
#include <cuda_runtime.h>

#include "g3l_device.cuh"

namespace g3l {

constexpr int SEL_BS = 256;
constexpr int SEL_WARPS = SEL_BS / 32;

__device__ __forceinline__ unsigned long long ekey(const double *err, long long s)
{
    return (unsigned long long)__double_as_longlong(err[s]);
}

// deterministic block reduction (fixed pairing)
template <typename T>
__device__ T block_sum(T v, T *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < SEL_WARPS; ++w) r += sh[w];
        sh[0] = r;
    }
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

// exclusive block scan of 0/1 flags; returns prefix, writes the total
__device__ int block_flag_scan(int flag, int *sh, int &total)
{
    unsigned b = __ballot_sync(0xffffffffu, flag);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int pre = __popc(b & ((1u << lane) - 1u));
    if (lane == 0) sh[w] = __popc(b);
    __syncthreads();
    int off = 0, tot = 0;
    for (int k = 0; k < SEL_WARPS; ++k) {
        if (k < w) off += sh[k];
        tot += sh[k];
    }
    __syncthreads();
    total = tot;
    return off + pre;
}

__device__ float block_max(float v, float *sh)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x == 0) {
        for (int w = 0; w < SEL_WARPS; ++w) r = fmaxf(r, sh[w]);
        sh[0] = r;
    }
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

struct SelShared {
    unsigned int cnt[256];
    unsigned long long sum[256];
    unsigned long long prefix, mask;
    unsigned long long sum_above;
    unsigned int cnt_above;
    int chosen, unique;
    double dred[SEL_WARPS];
    unsigned long long ured[SEL_WARPS];
    int ired[SEL_WARPS];
    float fred[SEL_WARPS];
};

// MSD radix select over the live errors of one integral, descending.  by_sum:
// find the bucket where the cumulative fixed-point error first reaches `need`;
// otherwise where the cumulative count reaches `need`.  Returns the boundary key
// and the count/sum of strictly larger keys.
__device__ void radix_select(const double *err, const unsigned long long *q, long long base, int R,
                             bool by_sum, unsigned long long need, SelShared &sh,
                             unsigned long long &bkey, unsigned int &cnt_above,
                             unsigned long long &sum_above)
{
    if (threadIdx.x == 0) {
        sh.prefix = 0;
        sh.mask = 0;
        sh.sum_above = 0;
        sh.cnt_above = 0;
        sh.unique = 0;
    }
    __syncthreads();
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        sh.cnt[threadIdx.x] = 0;
        sh.sum[threadIdx.x] = 0;
        __syncthreads();
        const unsigned long long prefix = sh.prefix, mask = sh.mask;
        for (int j = threadIdx.x; j < R; j += SEL_BS) {
            unsigned long long k = ekey(err, base + j);
            if ((k & mask) == prefix) {
                int dg = (int)((k >> shift) & 255ull);
                atomicAdd(&sh.cnt[dg], 1u);
                if (by_sum) atomicAdd(&sh.sum[dg], q[base + j]);
            }
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            // lane l owns buckets 255-8l .. 248-8l (descending)
            const int lane = threadIdx.x;
            unsigned long long s = 0, c = 0;
            for (int b = 0; b < 8; ++b) {
                int dg = 255 - 8 * lane - b;
                s += sh.sum[dg];
                c += sh.cnt[dg];
            }
            unsigned long long v = by_sum ? s : c;
            unsigned long long inc = v;  // inclusive scan in descending bucket order
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            const unsigned long long base_v = by_sum ? sh.sum_above : sh.cnt_above;
            unsigned hit = __ballot_sync(0xffffffffu, base_v + inc >= need);
            int first = hit ? __ffs(hit) - 1 : 31;
            unsigned long long exs = 0, exc_c = 0;
            // exclusive sums of both quantities at the owning lane
            unsigned long long sc = s, cc = c;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long t1 = __shfl_up_sync(0xffffffffu, sc, o);
                unsigned long long t2 = __shfl_up_sync(0xffffffffu, cc, o);
                if (lane >= o) {
                    sc += t1;
                    cc += t2;
                }
            }
            exs = sc - s;
            exc_c = cc - c;
            if (lane == first) {
                unsigned long long sa = sh.sum_above + exs, ca = sh.cnt_above + exc_c;
                int chosen = 255 - 8 * lane - 7;
                for (int b = 0; b < 8; ++b) {
                    int dg = 255 - 8 * lane - b;
                    unsigned long long nv = by_sum ? sa + sh.sum[dg] : ca + sh.cnt[dg];
                    if (nv >= need) {
                        chosen = dg;
                        break;
                    }
                    sa += sh.sum[dg];
                    ca += sh.cnt[dg];
                }
                sh.sum_above = sa;
                sh.cnt_above = (unsigned int)ca;
                sh.chosen = chosen;
                sh.prefix = prefix | ((unsigned long long)chosen << shift);
                sh.mask = mask | (0xFFull << shift);
                sh.unique = (sh.cnt[chosen] == 1u);
            }
        }
        __syncthreads();
        if (sh.unique) {
            // a single element carries the boundary: find its full key
            const unsigned long long p2 = sh.prefix, m2 = sh.mask;
            for (int j = threadIdx.x; j < R; j += SEL_BS) {
                unsigned long long k = ekey(err, base + j);
                if ((k & m2) == p2) sh.prefix = k;  // exactly one writer
            }
            __syncthreads();
            break;
        }
    }
    bkey = sh.prefix;
    cnt_above = sh.cnt_above;
    sum_above = sh.sum_above;
    __syncthreads();
}

// Mixed precision: queue for FP64 re-evaluation the regions of integral i with the
// largest uncertainty keys (P.key, filled by the caller; U their sum), until the keys
// left sum to at most `keep`, and let the integral's selection wait for them.  Used
// when a threshold decision (convergence, the Gladwell count) lies within the FP32
// uncertainty of the sums it compares.
__device__ void escalate_keys(const IntDesc &d, IntState *S, const Pool &P, BatchHdr *H, int i,
                              long long base, int R, double U, double keep, SelShared &sh)
{
    const double sc = 1152921504606846976.0 / U;  // 2^60 / U
    unsigned long long ql = 0;
    for (int j = threadIdx.x; j < R; j += SEL_BS) {
        const double t = P.key[base + j] * sc;
        const unsigned long long qq = t >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)t;
        P.q[base + j] = qq;
        ql += qq;
    }
    const unsigned long long Qk = block_sum(ql, sh.ured);
    const double kq = keep * sc;
    const unsigned long long qk = kq >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)kq;
    const unsigned long long needp = Qk > qk ? Qk - qk : 1;
    unsigned long long pb, ps;
    unsigned int pc;
    radix_select(P.key, P.q, base, R, true, needp, sh, pb, pc, ps);
    for (int j = threadIdx.x; j < R; j += SEL_BS) {
        const unsigned long long kb = (unsigned long long)__double_as_longlong(P.key[base + j]);
        if (kb >= pb && P.key[base + j] > 0.0) push_esc(H, P, d.kind * 3 + d.term - 1, i, j | (1 << 30));
    }
    if (threadIdx.x == 0) {
        S[i].K = 0;
        S[i].defer = 1;
        atomicAdd(&H->deferred, 1ull);
        atomicAdd(&H->thr_checks, 1ull);
    }
    __syncthreads();
}

// pass 0 selects for every live integral; pass 1 (mixed precision) selects again, in
// the same round, for the integrals pass 0 deferred, once the FP64 re-evaluation of
// their ambiguous boundary regions has run.
__global__ void __launch_bounds__(SEL_BS) k_select(const IntDesc *__restrict__ D,
                                                   IntState *__restrict__ S, Pool P, BatchHdr *H,
                                                   double tau_sel, double tau_val, int pass)
{
    __shared__ SelShared sh;
    __shared__ int s_flag[4];  // fin, status, polish passes
    __shared__ double s_tot[4];
    __shared__ int s_cancel;
    // threshold guard (mixed precision): bound multiplier (gthr) and the value bounds' basis
    const double gthr = H->mixed ? (double)H->thr_ratio : 0.0;
    const double vr = (double)H->val_ratio;
    const int n = H->n;
    // a stop request: k_scan's (cancel or deadline), or a host cancel that arrived since
    // (one read of the host-mapped word per block)
    if (threadIdx.x == 0) {
        int cz = H->cancel;
        if (!cz && H->cancel_word && *H->cancel_word) cz = 1;
        s_cancel = cz;
    }
    __syncthreads();
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        if (pass == 1 && !S[i].defer) continue;  // block-uniform
        __syncthreads();
        if (threadIdx.x == 0) S[i].defer = 0;
        if (S[i].done) {
            if (threadIdx.x == 0) S[i].K = 0;
            continue;
        }
        const IntDesc &d = D[i];
        const long long base = d.base;
        const int R = S[i].nR;
        if (R == 0) {
            // fresh integral: its root region is this round's single work item
            if (threadIdx.x == 0) {
                P.cand[base] = -1;
                S[i].K = 1;
                S[i].nR = 1;
                S[i].neval = (unsigned long long)d.npts;
            }
            __syncthreads();
            continue;
        }
        // totals over live regions (mixed: and the FP32 uncertainty of each total)
        double sv = 0, se = 0, sue = 0, suv = 0;
        for (int j = threadIdx.x; j < R; j += SEL_BS) {
            const double v = P.val[base + j], e = P.err[base + j];
            sv += v;
            se += e;
            if (gthr > 0.0) {
                sue += e * (double)P.unc[base + j];
                suv += fabs(v) * (double)P.uval[base + j];
            }
        }
        double V = block_sum(sv, sh.dred);
        double E = block_sum(se, sh.dred);
        double UE = 0, UV = 0;
        if (gthr > 0.0) {
            UE = gthr * block_sum(sue, sh.dred);
            UV = gthr * vr * block_sum(suv, sh.dred);
        }
        if (threadIdx.x == 0) {
            IntState st = S[i];
            int fin = 0, status = ST_OK;
            if (s_cancel) {
                fin = 1;
                status = s_cancel == 2 ? ST_DEADLINE : ST_CANCELLED;
            } else if (!isfinite(V) || !isfinite(E)) {
                fin = 1;
                status = ST_NONFINITE;
            } else if (d.max_eval && st.neval >= d.max_eval) {
                fin = 1;
            } else if (!(E > 0 && E > fabs(V) * d.rtol)) {
                fin = 1;  // converged (src/converged.h:10-14 with reqAbsError = 0)
            } else if (st.rounds >= H->max_rounds) {
                fin = 1;
                status = ST_ROUNDS;
            }
            S[i].val = V;
            S[i].err = E;
            s_flag[0] = fin;
            s_flag[1] = status;
            s_flag[2] = st.pad;  // polish passes so far
            s_tot[0] = V;
            s_tot[1] = E;
            // the convergence test E <= rtol |V| decided within the FP32 uncertainty
            const bool tested = !s_cancel && isfinite(V) && isfinite(E) &&
                                !(d.max_eval && st.neval >= d.max_eval);
            s_flag[3] = gthr > 0.0 && tested && (UE + d.rtol * UV) > 0.0 &&
                        fabs(E - fabs(V) * d.rtol) <= UE + d.rtol * UV;
        }
        __syncthreads();
        if (s_flag[3]) {
            const double margin = fabs(s_tot[1] - fabs(s_tot[0]) * d.rtol);
            double ul = 0;
            for (int j = threadIdx.x; j < R; j += SEL_BS) {
                const double kj = gthr * (P.err[base + j] * (double)P.unc[base + j] +
                                         d.rtol * vr * fabs(P.val[base + j]) * (double)P.uval[base + j]);
                P.key[base + j] = kj;
                ul += kj;
            }
            const double U = block_sum(ul, sh.dred);
            escalate_keys(d, S, P, H, i, base, R, U, 0.9 * margin, sh);
            continue;
        }
        if (s_flag[0]) {
            // Mixed precision: before reporting, bound the FP32 noise left in the value.
            // If the regions' value bounds sum to more than tau_val |V|, re-evaluate in
            // FP64 the regions with the largest bounds until the rest is below half of it.
            bool polish = false;
            if (H->mixed && tau_val > 0.0 && s_flag[1] == ST_OK && s_flag[2] < 2) {
                const double Vt = s_tot[0];
                double uloc = 0;
                for (int j = threadIdx.x; j < R; j += SEL_BS) {
                    const double kj = fabs(P.val[base + j]) * (double)P.uval[base + j];
                    P.key[base + j] = kj;
                    uloc += kj;
                }
                const double U = block_sum(uloc, sh.dred);
                if (U > tau_val * fabs(Vt) && U > 0) {
                    polish = true;
                    const double sc = 1152921504606846976.0 / U;
                    unsigned long long ql = 0;
                    for (int j = threadIdx.x; j < R; j += SEL_BS) {
                        double t = P.key[base + j] * sc;
                        unsigned long long qq = t >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)t;
                        P.q[base + j] = qq;
                        ql += qq;
                    }
                    const unsigned long long Qk = block_sum(ql, sh.ured);
                    const double keep = 0.5 * tau_val * fabs(Vt) * sc;
                    const unsigned long long qk = keep >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)keep;
                    const unsigned long long needp = Qk > qk ? Qk - qk : 1;
                    unsigned long long pb;
                    unsigned int pc;
                    unsigned long long ps;
                    radix_select(P.key, P.q, base, R, true, needp, sh, pb, pc, ps);
                    for (int j = threadIdx.x; j < R; j += SEL_BS) {
                        const unsigned long long kb =
                            (unsigned long long)__double_as_longlong(P.key[base + j]);
                        if (kb >= pb && P.uval[base + j] > 0.f) {
                            push_esc(H, P, d.kind * 3 + d.term - 1, i, j | (1 << 30));
                        }
                    }
                    if (threadIdx.x == 0) {
                        S[i].K = 0;
                        S[i].pad += 1;
                        S[i].defer = 1;  // finish (or polish again) after the re-evaluation
                        atomicAdd(&H->polished, 1ull);
                    }
                }
            }
            if (!polish && threadIdx.x == 0) {
                S[i].done = 1;
                S[i].status = s_flag[1];
                S[i].K = 0;
            }
            __syncthreads();
            continue;
        }
        V = s_tot[0];
        E = s_tot[1];
        const unsigned long long neval = S[i].neval;
        const unsigned long long twoNp = 2ull * (unsigned long long)d.npts;
        unsigned long long Kcap = (unsigned long long)R;
        if (d.max_eval) {
            unsigned long long left = d.max_eval - neval;  // > 0 here
            unsigned long long kc = (left + twoNp - 1) / twoNp;
            if (kc < Kcap) Kcap = kc;
        }
        // fixed-point errors: q = floor(err * 2^60 / E)
        const double scale = 1152921504606846976.0 / E;  // 2^60 / E
        unsigned long long qs = 0;
        for (int j = threadIdx.x; j < R; j += SEL_BS) {
            double t = P.err[base + j] * scale;
            unsigned long long qq = t >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)t;
            P.q[base + j] = qq;
            qs += qq;
        }
        const unsigned long long Q = block_sum(qs, sh.ured);
        const double thr = fabs(V) * d.rtol * scale;
        const unsigned long long qthr = thr >= 1.8e19 ? 0xFFFFFFFFFFFFFFFFull : (unsigned long long)thr;
        const unsigned long long need = Q > qthr ? Q - qthr : 0;
        // K_conv: smallest k >= 1 whose popped error sum reaches `need`
        unsigned long long Kconv;
        unsigned long long bkey = 0, tneed = 0;
        unsigned int cnt_above = 0;
        unsigned long long sum_above = 0;
        if (need == 0) {
            Kconv = 1;
        } else {
            radix_select(P.err, P.q, base, R, true, need, sh, bkey, cnt_above, sum_above);
            // all keys equal to bkey carry the same q (any writer stores the same value)
            if (threadIdx.x == 0) sh.ured[0] = 0;
            __syncthreads();
            for (int j = threadIdx.x; j < R; j += SEL_BS)
                if (ekey(P.err, base + j) == bkey) sh.ured[0] = P.q[base + j];
            __syncthreads();
            unsigned long long qb = sh.ured[0];
            __syncthreads();
            unsigned long long rest = need - sum_above;
            tneed = qb ? (rest + qb - 1) / qb : 1;
            Kconv = (unsigned long long)cnt_above + tneed;
            // Mixed precision: the Gladwell count is the first k whose popped errors reach
            // `need` (the error left is <= rtol |V|).  If either neighbouring count is within
            // the FP32 uncertainty of the sums this compares (the errors not popped before
            // the boundary, and rtol |V|), and the choice can matter (it moves a region of
            // error b, and neighbours only where the budget allows), re-evaluate the regions
            // carrying that uncertainty first.
            const double b = __longlong_as_double((long long)bkey);
            if (gthr > 0.0 && qb && Kconv <= Kcap && b > H->tau_thr * fabs(V)) {
                const unsigned long long m_hi = sum_above + tneed * qb - need;  // < qb
                const unsigned long long m_lo = qb - m_hi;
                unsigned long long m = 0xFFFFFFFFFFFFFFFFull;
                if (Kconv < Kcap && Kconv < (unsigned long long)R) m = m_hi;
                if (Kconv > 1 && m_lo < m) m = m_lo;
                if (m != 0xFFFFFFFFFFFFFFFFull) {
                    double ur = 0;
                    for (int j = threadIdx.x; j < R; j += SEL_BS)
                        if (ekey(P.err, base + j) <= bkey)
                            ur += P.err[base + j] * (double)P.unc[base + j];
                    const double dlt = gthr * block_sum(ur, sh.dred) + d.rtol * UV;
                    const double m_abs = (double)m / scale;
                    if (dlt > 0.0 && m_abs <= dlt) {
                        double ul = 0;
                        for (int j = threadIdx.x; j < R; j += SEL_BS) {
                            const double e = P.err[base + j];
                            const double kj =
                                (ekey(P.err, base + j) <= bkey ? gthr * e * (double)P.unc[base + j] : 0.0) +
                                d.rtol * gthr * vr * fabs(P.val[base + j]) * (double)P.uval[base + j];
                            P.key[base + j] = kj;
                            ul += kj;
                        }
                        const double U = block_sum(ul, sh.dred);
                        escalate_keys(d, S, P, H, i, base, R, U, 0.9 * m_abs, sh);
                        continue;
                    }
                }
            }
        }
        unsigned long long K = Kconv < Kcap ? Kconv : Kcap;
        if (K < 1) K = 1;
        if (K > (unsigned long long)R) K = R;
        if (K != Kconv || need == 0) {
            if (K == (unsigned long long)R) {
                bkey = 0;
                cnt_above = 0;
                tneed = R;  // every key >= 0: take all
            } else {
                radix_select(P.err, P.q, base, R, false, K, sh, bkey, cnt_above, sum_above);
                tneed = K - cnt_above;
            }
        }
        // Mixed precision: if the boundary of this round's selection sits among regions
        // whose FP32-derived errors are uncertain (overlapping bounds), re-evaluate those
        // regions in FP64 first and select again next round.
        if (H->mixed && K < (unsigned long long)R) {
            const double b = __longlong_as_double((long long)bkey);
            if (b > tau_sel * fabs(V)) {
                float ub = 0.f;
                for (int j = threadIdx.x; j < R; j += SEL_BS)
                    if (ekey(P.err, base + j) == bkey) ub = fmaxf(ub, P.unc[base + j]);
                ub = block_max(ub, sh.fred);
                const double blo = b * (1.0 - ub), bhi = b * (1.0 + ub);
                int amb = 0;
                for (int j = threadIdx.x; j < R; j += SEL_BS) {
                    const unsigned long long k = ekey(P.err, base + j);
                    if (k == bkey) continue;
                    const double e = P.err[base + j];
                    const float u = P.unc[base + j];
                    if ((u > 0.f || ub > 0.f) && e * (1.0 + u) >= blo && e * (1.0 - u) <= bhi) ++amb;
                }
                amb = block_sum(amb, sh.ired);
                if (amb > 0) {
                    for (int j = threadIdx.x; j < R; j += SEL_BS) {
                        const double e = P.err[base + j];
                        const float u = P.unc[base + j];
                        if (u > 0.f && e * (1.0 + u) >= blo && e * (1.0 - u) <= bhi) {
                            push_esc(H, P, d.kind * 3 + d.term - 1, i, j | (1 << 30));
                        }
                    }
                    if (threadIdx.x == 0) {
                        S[i].K = 0;
                        S[i].defer = 1;
                        atomicAdd(&H->deferred, 1ull);
                    }
                    __syncthreads();
                    continue;
                }
            }
        }
        // pool capacity
        if ((long long)R + (long long)K > (long long)d.cap) {
            if (threadIdx.x == 0) {
                S[i].done = 1;
                S[i].status = ST_POOL;
                S[i].K = 0;
            }
            __syncthreads();
            continue;
        }
        // compact the selection in slot order
        int run_sel = 0, run_tie = 0;
        for (int c0 = 0; c0 < R; c0 += SEL_BS) {
            int j = c0 + threadIdx.x;
            unsigned long long k = j < R ? ekey(P.err, base + j) : 0;
            int is_eq = (j < R && k == bkey && !(K == (unsigned long long)R)) ? 1 : 0;
            int is_gt = (j < R && (K == (unsigned long long)R || k > bkey)) ? 1 : 0;
            int ntie;
            int tr = run_tie + block_flag_scan(is_eq, sh.ired, ntie);
            int sel = is_gt || (is_eq && (unsigned long long)tr < tneed);
            int nsel;
            int pos = run_sel + block_flag_scan(sel, sh.ired, nsel);
            if (sel) P.cand[base + pos] = j;
            run_tie += ntie;
            run_sel += nsel;
        }
        // Mixed precision: selected parents whose split is flagged unsettled get it
        // re-taken in FP64 before this round's cut.
        if (H->mixed) {
            __syncthreads();
            for (int j = threadIdx.x; j < (int)K; j += SEL_BS) {
                const int r = P.cand[base + j];
                if (P.split[base + r] & 0x80) {
                    push_esc(H, P, d.kind * 3 + d.term - 1, i, r);
                }
            }
        }
        if (threadIdx.x == 0) {
            S[i].K = (int)K;
            S[i].neval = neval + twoNp * K;
            S[i].nR = R + (int)K;
            S[i].rounds += 1;
        }
        __syncthreads();
    }
}

// prefix sum of K over integrals; work list offsets; loop condition
__global__ void __launch_bounds__(1024) k_scan(IntState *__restrict__ S, long long *woff,
                                               BatchHdr *H, cudaGraphConditionalHandle handle,
                                               int use_cond)
{
    __shared__ long long part[1024];
    const int n = H->n;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    long long loc = 0;
    for (int i = b; i < e; ++i) loc += S[i].K;
    part[threadIdx.x] = loc;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        long long t = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    long long run = part[threadIdx.x] - loc;
    for (int i = b; i < e; ++i) {
        woff[i] = run;
        run += S[i].K;
    }
    if (threadIdx.x == blockDim.x - 1) {
        long long tot = part[blockDim.x - 1];
        woff[n] = tot;
        H->total_work = tot;
        // keep looping while there is work or a deferred FP64 re-evaluation
        int pending = 0;
        for (int g = 0; g < NGROUPS; ++g) pending |= H->n_esc[g];
        const int more = tot > 0 || pending > 0;
        H->any_active = more;
        H->regions += 2ull * (unsigned long long)tot;
        if (more) H->rounds_done += 1;
        // a cancel from the host, or the deadline, stops every unfinished integral at the
        // next round's selection (this round's work still runs, so the pools stay whole)
        if (!H->cancel) {
            if (H->cancel_word && *H->cancel_word) H->cancel = 1;
            else if (H->deadline_ns && global_timer_ns() - H->t0_ns > H->deadline_ns)
                H->cancel = 2;
        }
        // a serving launch ends after chunk_rounds rounds; this round's body still runs,
        // so the states are consistent for the host between launches
        int go = more;
        if (more && H->chunk_rounds > 0 && ++H->chunk_count >= H->chunk_rounds) go = 0;
        if (use_cond) cudaGraphSetConditional(handle, go ? 1u : 0u);
    }
}

// root regions and fresh state
__global__ void k_init(const IntDesc *__restrict__ D, IntState *__restrict__ S, Pool P,
                       BatchHdr *H)
{
    const int n = H->n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const IntDesc &d = D[i];
        for (int k = 0; k < MAX_DIM; ++k) {
            if (k < d.dim) {
                P.center[k * P.stride + d.base] = d.c0[k];
                P.level[k * P.stride + d.base] = 0;
            }
        }
        IntState st;
        st.val = 0;
        st.err = 0;
        st.neval = 0;
        st.nR = 0;
        st.K = 0;
        st.done = 0;
        st.status = ST_OK;
        st.rounds = 0;
        st.pad = 0;
        st.defer = 0;
        st.pad2 = 0;
        S[i] = st;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        H->any_active = 1;
        H->total_work = 0;
        H->regions = (unsigned long long)n;
        H->rounds_done = 0;
        H->chunk_count = 0;
        H->ties = 0;
        H->small_arg = 0;
        for (int g = 0; g < NGROUPS; ++g) H->n_esc[g] = 0;
        H->escalated = 0;
        H->deferred = 0;
        H->polished = 0;
        H->esc_full = 0;
        H->thr_checks = 0;
        H->cancel = 0;
        H->t0_ns = global_timer_ns();
    }
}

// end of a mixed-precision round: the FP64 re-evaluation queue has been consumed
// End of a re-evaluation stage: count and clear the queues of every group (grp < 0) or
// of group grp alone (the per-group ends of concurrent branches, hence the atomic count)
__global__ void k_round_end(BatchHdr *H, int grp)
{
    for (int g = grp < 0 ? 0 : grp; g < (grp < 0 ? NGROUPS : grp + 1); ++g) {
        const int n = H->n_esc[g];
        atomicAdd(&H->escalated, (unsigned long long)(n < H->esc_cap[g] ? n : H->esc_cap[g]));
        H->n_esc[g] = 0;
    }
}

// Serving: place m integrals (packed descriptors Dn) into table slots idx[] and start
// each one at its root region.
__global__ void k_admit(const IntDesc *__restrict__ Dn, const int *__restrict__ idx, int m,
                        IntDesc *__restrict__ D, IntState *__restrict__ S, Pool P)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
        const IntDesc d = Dn[j];
        const int i = idx[j];
        D[i] = d;
        for (int k = 0; k < d.dim; ++k) {
            P.center[k * P.stride + d.base] = d.c0[k];
            P.level[k * P.stride + d.base] = 0;
        }
        IntState st;
        st.val = 0;
        st.err = 0;
        st.neval = 0;
        st.nR = 0;
        st.K = 0;
        st.done = 0;
        st.status = ST_OK;
        st.rounds = 0;
        st.pad = 0;
        st.defer = 0;
        st.pad2 = 0;
        S[i] = st;
    }
}

void *admit_kernel() { return (void *)k_admit; }
void *round_end_kernel() { return (void *)k_round_end; }
void *select_kernel() { return (void *)k_select; }
void *scan_kernel() { return (void *)k_scan; }
void *init_kernel() { return (void *)k_init; }

}  // namespace g3l
