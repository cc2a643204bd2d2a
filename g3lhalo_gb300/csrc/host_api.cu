// host_api.cu -- the C ABI: context, tables, HOD slots, batched evaluation.
//
// A call to g3l_eval turns its integrals into per-integral descriptors (sorted
// by kind and term so each rule-evaluation kernel sees one integrand), sizes
// the region pools from the evaluation caps, and runs one CUDA graph:
//   k_init -> WHILE(any work) { k_select -> k_scan -> k_eval per group }
// The loop condition is set on the device by k_scan, so the host waits once,
// at the end of the call.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <new>
#include <stdexcept>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "g3l_device.cuh"
#include "g3l_gpu.h"
#include "host_internal.h"

namespace g3l {
void *eval64_kernel(int kind, int term);
void *reeval64_kernel(int kind, int term);
void *reeval_phase_kernel(int kind, int term, int phase);
cudaError_t build_reeval_tables(unsigned char *out, cudaStream_t s);
void *round_end_kernel();
void *evalmx_kernel_k0(int term, int variant);
void *evalmx_kernel_k1(int term, int variant);
inline void *evalmx_kernel(int kind, int term, int variant = 0)
{
    return kind == 0 ? evalmx_kernel_k0(term, variant) : evalmx_kernel_k1(term, variant);
}
void *select_kernel();
void *scan_kernel();
void *init_kernel();
void *admit_kernel();
namespace host {
const char *last_error_cstr();
}
}  // namespace g3l

using namespace g3l;

namespace {

#define G3L_CK(call)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            host::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));              \
            return G3L_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

template <typename T>
int dalloc(T **p, size_t n)
{
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        host::set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        *p = nullptr;
        return G3L_ERR_NOMEM;
    }
    return G3L_OK;
}

// FP64 re-evaluation entries per group and round that take the device-wide passes
// (10.0 kB of scratch each): 4 per integral, between 8192 (82 MB per group) and 524288
// (5.2 GB per group); further entries take the batched kernel k_reeval64, which
// evaluates every point on its own.  G3L_REEVAL_CAP=<n> (read when a workspace is
// allocated) sets the count instead: 0 sends every entry through the batched kernel, so
// that tests can hold the passes' cached values against it.
int reeval_cap(int n_integrals)
{
    if (const char *e = std::getenv("G3L_REEVAL_CAP")) {
        const long long v = std::atoll(e);
        if (v >= 0) return (int)std::min<long long>(v, 524288);
    }
    return (int)std::min<long long>(std::max<long long>(4ll * n_integrals, 8192), 524288);
}

struct Workspace {
    size_t pool_cap = 0;
    int n_cap = 0;
    Pool P{};
    IntDesc *D = nullptr;
    IntState *S = nullptr;
    long long *woff = nullptr;
    BatchHdr *H = nullptr;
    int gen = 0;
};

struct GraphEntry {
    int gen, precision, gmask;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

}  // namespace

struct g3l_ctx {
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;
    host::Binning B{};
    double Om = 0, OL = 0, Ob = 0, s8 = 0, H0 = 0, ns = 0;
    std::vector<double> hmf_h, rho_h;
    std::vector<double> hod_h, nbar_h;
    std::vector<float> fnbar_h, fhodp_h;  // host copies of the mixed path's per-slot tables
    std::vector<char> hod_set;
    double A = 0, eps = 0;
    DevTables T{};
    std::vector<void *> allocs;
    double *d_hod = nullptr, *d_nbar = nullptr, *d_scale = nullptr;
    float *d_fscale = nullptr;
    // mixed path
    float *d_fnbar = nullptr, *d_fhodp = nullptr;
    std::vector<double> sn;  // per-slot n_bar scale
    double SH = 1, SP = 1, SZA = 1, SZB = 1;
    Workspace W;
    std::vector<GraphEntry> graphs;
    g3l_options opt{};
    g3l_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t tev[16] = {};
    // pinned staging for the per-call descriptor and result copies
    void *stage = nullptr;
    size_t stage_bytes = 0;
    long long *h_pinned = nullptr;
    size_t last_h2d = 0, last_d2h = 0;
    g3l_server *srv[2] = {nullptr, nullptr};  // serving loops behind g3l_submit, per precision
    std::mutex srv_mu;
    // last g3l_eval: descriptor, live region count and pool position of each item
    std::vector<IntDesc> last_D;
    std::vector<int> last_nR, last_pos;
    // in-flight cancel of g3l_eval: a host-mapped word the device loop reads once per
    // round; `running` (under run_mu) tells g3l_eval_cancel whether a call is in flight
    int *cancel_h = nullptr, *cancel_d = nullptr;
    unsigned char *retab_d = nullptr;  // re-evaluation point tables (NGROUPS * RETAB_BYTES)
    std::mutex run_mu;
    bool running = false;
    host::NbarDevice nbw;  // device buffers of the n_bar integrals (g3l_set_hod)
};

namespace {

// NVTX range for the lifetime of a scope (shown by Nsight tools; free without them)
struct NvtxScope {
    explicit NvtxScope(const char *name) { nvtxRangePushA(name); }
    ~NvtxScope() { nvtxRangePop(); }
};

// Marks a context's evaluation call as running for g3l_eval_cancel and clears any
// earlier cancel request, for the lifetime of the call.
struct RunGuard {
    g3l_ctx *c;
    explicit RunGuard(g3l_ctx *cc) : c(cc)
    {
        std::lock_guard<std::mutex> lk(c->run_mu);
        c->running = true;
        __atomic_store_n(c->cancel_h, 0, __ATOMIC_SEQ_CST);
    }
    ~RunGuard()
    {
        std::lock_guard<std::mutex> lk(c->run_mu);
        c->running = false;
    }
};

// the header fields that stop a call in flight
void set_stop_fields(const g3l_ctx *c, BatchHdr &H)
{
    H.thr_ratio = (float)c->opt.unc_thr;
    H.tau_thr = c->opt.unc_tau_thr;
    H.val_ratio = (float)(c->opt.unc_eps_sel / std::max(c->opt.unc_eps_val, 1e-30));
    H.cancel = 0;
    H.cancel_word = c->cancel_d;
    H.deadline_ns = c->opt.deadline_ms > 0
                        ? (unsigned long long)std::min(c->opt.deadline_ms * 1e6, 1.8e19)
                        : 0ull;
}

int upload(g3l_ctx *c, const double *src, size_t n, const double **dst)
{
    double *p;
    int st = dalloc(&p, n);
    if (st) return st;
    c->allocs.push_back(p);
    G3L_CK(cudaMemcpy(p, src, n * sizeof(double), cudaMemcpyHostToDevice));
    *dst = p;
    return G3L_OK;
}

float2 dsplit(double x)
{
    float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

template <typename T>
int upload_t(g3l_ctx *c, const std::vector<T> &src, const T **dst)
{
    T *p;
    int st = dalloc(&p, src.size());
    if (st) return st;
    c->allocs.push_back(p);
    G3L_CK(cudaMemcpy(p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    *dst = p;
    return G3L_OK;
}

constexpr double kL0 = 1e3;   // l unit of the FP32 integrand
constexpr double kM0 = 1e12;  // m unit of the FP32 integrand

// Mixed-path tables: FP32 in scaled units plus double-float constants.
int prepare_mixed(g3l_ctx *c, const g3l_tables *t)
{
    DevTables &T = c->T;
    const int Nz = t->Nz, Nm = t->Nm, Nk = t->Nk;
    double mh = 0, mp = 0, mza = 0, mzb = 0;
    for (size_t i = 0; i < (size_t)Nz * Nm; ++i) mh = std::max(mh, std::fabs(t->hmf[i]));
    for (size_t i = 0; i < (size_t)Nz * Nk; ++i) mp = std::max(mp, std::fabs(t->P_lin[i]));
    std::vector<double> zA(Nz), zB(Nz);
    for (int i = 0; i < Nz; ++i) {
        const double w = t->w[i], rho = c->rho_h[i];
        zA[i] = t->g[i] * t->p_lens1[i] * t->p_lens2[i] / (t->dwdz[i] * w * w * w * rho);
        zB[i] = t->g[i] * t->g[i] * t->p_lens1[i] / (t->dwdz[i] * w * w * rho * rho);
        if (std::isfinite(zA[i])) mza = std::max(mza, std::fabs(zA[i]));
        if (std::isfinite(zB[i])) mzb = std::max(mzb, std::fabs(zB[i]));
    }
    c->SH = mh > 0 ? 1 / mh : 1;
    c->SP = mp > 0 ? 1 / mp : 1;
    c->SZA = mza > 0 ? 1 / mza : 1;
    c->SZB = mzb > 0 ? 1 / mzb : 1;
    std::vector<float> fh(Nz * (size_t)Nm), fb(Nz * (size_t)Nm), fc(Nz * (size_t)Nm),
        fp(Nz * (size_t)Nk);
    for (size_t i = 0; i < fh.size(); ++i) {
        fh[i] = (float)(t->hmf[i] * c->SH);
        fb[i] = (float)t->b_h[i];
        fc[i] = (float)t->conc[i];
    }
    for (size_t i = 0; i < fp.size(); ++i) fp[i] = (float)(t->P_lin[i] * c->SP);
    std::vector<float> fza(Nz), fzb(Nz), fkw(Nz), fk200(Nz);
    std::vector<float2> fkb(Nz);
    const double kscale = Nk / std::log(t->kmax / t->kmin);
    for (int i = 0; i < Nz; ++i) {
        fza[i] = std::isfinite(zA[i]) ? (float)(zA[i] * c->SZA) : 0.f;
        fzb[i] = std::isfinite(zB[i]) ? (float)(zB[i] * c->SZB) : 0.f;
        fkw[i] = (float)(kL0 / t->w[i]);
        fk200[i] = (float)(0.239 * kM0 / (200 * c->rho_h[i]));
        fkb[i] = dsplit((std::log(t->w[i]) + std::log(t->kmin)) * kscale);
    }
    int st = 0;
    st |= upload_t(c, fh, &T.f_hmf);
    st |= upload_t(c, fb, &T.f_bh);
    st |= upload_t(c, fc, &T.f_conc);
    st |= upload_t(c, fp, &T.f_plin);
    st |= upload_t(c, fza, &T.f_zA);
    st |= upload_t(c, fzb, &T.f_zB);
    st |= upload_t(c, fkw, &T.f_kw);
    st |= upload_t(c, fk200, &T.f_k200);
    st |= upload_t(c, fkb, &T.f_kb);
    if (st) return st;
    T.k_a = dsplit(std::log(10.0) * kscale);
    T.kscale2 = dsplit(kscale);
    T.lnkmin2 = dsplit(std::log(t->kmin));
    T.m_x02 = dsplit(std::log10(t->mmin));
    T.m_s2 = dsplit(Nm / std::log10(t->mmax / t->mmin));
    T.z_02 = dsplit(t->zmin);
    T.z_s2 = dsplit(Nz / (t->zmax - t->zmin));
    T.small_arg = (float)c->opt.small_arg;
    T.unc_eps = (float)c->opt.unc_eps_rel;
    T.unc_abs = (float)c->opt.unc_tau_abs;
    T.tau_impact = c->opt.unc_tau_impact;
    T.tau_sel = c->opt.unc_tau_sel;
    T.tau_val = c->opt.unc_tau_val;
    T.unc_val_ratio = (float)(c->opt.unc_eps_val / c->opt.unc_eps_rel);
    T.unc_sel_ratio = (float)(c->opt.unc_eps_sel / c->opt.unc_eps_rel);
    st |= dalloc(&c->d_fnbar, (size_t)MAX_HOD_SLOTS * Nz);
    st |= dalloc(&c->d_fhodp, (size_t)MAX_HOD_SLOTS * 8);
    if (st) return st;
    c->allocs.push_back(c->d_fnbar);
    c->allocs.push_back(c->d_fhodp);
    G3L_CK(cudaMemset(c->d_fnbar, 0, sizeof(float) * MAX_HOD_SLOTS * Nz));
    G3L_CK(cudaMemset(c->d_fhodp, 0, sizeof(float) * MAX_HOD_SLOTS * 8));
    T.f_nbar = c->d_fnbar;
    T.f_hodp = c->d_fhodp;
    c->sn.assign(MAX_HOD_SLOTS, 1.0);
    host::TieTable tz = host::build_z_ties(c->B);
    std::vector<unsigned long long> zb(tz.bits);
    const unsigned long long *pb;
    const int *pr, *pt;
    st |= upload_t(c, zb, &pb);
    st |= upload_t(c, tz.round_ix, &pr);
    st |= upload_t(c, tz.trunc_ix, &pt);
    if (st) return st;
    T.tie_z_bits = pb;
    T.tie_z_round = pr;
    T.tie_z_trunc = pt;
    T.n_tie_z = (int)tz.bits.size();
    return G3L_OK;
}

// scale of the FP32 integrand of a term: true value = scaled value * scale
double mixed_scale(const g3l_ctx *c, int kind, int term, int h1, int h2)
{
    const int nm = kind == 0 ? term + 1 : term + 2;
    const double snf = kind == 0 ? c->sn[h1] * c->sn[h2] : c->sn[h1] * c->sn[h1];
    const double sz = kind == 0 ? c->SZA : c->SZB;
    return std::pow(kL0, 4) * std::pow(kM0, nm) * snf /
           (std::pow(c->SH, term) * std::pow(c->SP, term - 1) * sz);
}

bool finite_all(const double *a, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

void free_workspace(Workspace &W)
{
    void *ptrs[] = {W.P.center, W.P.level, W.P.val, W.P.err, W.P.split, W.P.cmask, W.P.q, W.P.cand,
                    W.P.unc,    W.P.esc,   W.P.uval, W.P.key, W.P.rscr, W.D, W.S, W.woff, W.H};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    const int gen = W.gen;
    W = Workspace{};
    W.gen = gen;
}

// Region pools for `pcap` slots and per-integral arrays for `ncap` integrals.
int alloc_workspace(Workspace &W, int ncap, size_t pcap, const unsigned char *retab)
{
    free_workspace(W);
    int st = 0;
    W.P.retab = retab;
    st |= dalloc(&W.P.center, pcap * MAX_DIM);
    st |= dalloc(&W.P.level, pcap * MAX_DIM);
    st |= dalloc(&W.P.val, pcap);
    st |= dalloc(&W.P.err, pcap);
    st |= dalloc(&W.P.split, pcap);
    st |= dalloc(&W.P.cmask, pcap);
    st |= dalloc(&W.P.q, pcap);
    st |= dalloc(&W.P.cand, pcap);
    st |= dalloc(&W.P.unc, pcap);
    st |= dalloc(&W.P.uval, pcap);
    st |= dalloc(&W.P.key, pcap);
    st |= dalloc(&W.P.esc, pcap);
    W.P.rcap = reeval_cap(ncap);
    W.P.rscr_group = reeval_scratch_group_bytes(W.P.rcap);
    st |= dalloc(&W.P.rscr, (size_t)(NGROUPS * W.P.rscr_group));
    st |= dalloc(&W.D, (size_t)ncap);
    st |= dalloc(&W.S, (size_t)ncap);
    st |= dalloc(&W.woff, (size_t)ncap + 1);
    st |= dalloc(&W.H, 1);
    if (st) {
        free_workspace(W);
        return G3L_ERR_NOMEM;
    }
    W.P.stride = (long long)pcap;
    W.pool_cap = pcap;
    W.n_cap = ncap;
    W.gen += 1;
    return G3L_OK;
}

int ensure_workspace(g3l_ctx *c, int n, size_t pool)
{
    Workspace &W = c->W;
    if (n <= W.n_cap && pool <= W.pool_cap) return G3L_OK;
    cudaStreamSynchronize(c->stream);
    int ncap = std::max(n, W.n_cap);
    size_t pcap = std::max(pool, W.pool_cap);
    if (n > W.n_cap) ncap = std::max(ncap, (int)(n * 1.25) + 16);
    if (pool > W.pool_cap) pcap = std::max(pcap, (size_t)(pool * 1.25) + 1024);
    for (auto &g : c->graphs) {
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
    }
    c->graphs.clear();
    return alloc_workspace(W, ncap, pcap, c->retab_d);
}

void *eval_fn(const g3l_ctx *c, int precision, int group)
{
    int kind = group / 3, term = group % 3 + 1;
    return precision == G3L_FP64 ? eval64_kernel(kind, term)
                                 : evalmx_kernel(kind, term, c->opt.evalmx_variant[group]);
}

int eval_grid(g3l_ctx *c, void *fn)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, 0) != cudaSuccess || nb < 1) nb = 1;
    if (c->opt.eval_blocks_per_sm > 0) nb = std::min(nb, c->opt.eval_blocks_per_sm);
    return nb * c->nsm;
}

int grid128(g3l_ctx *c, void *fn)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, 0) != cudaSuccess || nb < 1) nb = 1;
    return nb * c->nsm;
}

int reeval_grid(g3l_ctx *c, void *fn)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, 0) != cudaSuccess || nb < 1) nb = 1;
    return nb * c->nsm;
}

struct KernelArgs {
    DevTables T;
    IntDesc *D;
    IntState *S;
    Pool P;
    BatchHdr *H;
    long long *woff;
    cudaGraphConditionalHandle handle;
    int use_cond;
    double tau_sel;
    double tau_val;
    int pass0 = 0, pass1 = 1;
    int all_groups = -1;
    int grp_id[NGROUPS] = {0, 1, 2, 3, 4, 5};
};

int add_kernel(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *deps, size_t ndeps,
               void *fn, int grid, int block, void **args)
{
    cudaKernelNodeParams kp{};
    kp.func = fn;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    G3L_CK(cudaGraphAddKernelNode(node, g, deps, ndeps, &kp));
    return G3L_OK;
}

// FP64 re-evaluation queues: group g gets as many entries as its integrals have pool
// slots (a region is queued at most once per round), laid out group after group.
void set_esc_queues(const IntDesc *D, int n, BatchHdr &H)
{
    long long cnt[NGROUPS] = {};
    for (int r = 0; r < n; ++r) cnt[D[r].kind * 3 + D[r].term - 1] += D[r].cap;
    long long beg = 0;
    for (int g = 0; g < NGROUPS; ++g) {
        H.esc_beg[g] = beg;
        H.esc_cap[g] = (int)std::min<long long>(cnt[g], 0x7fffffff);
        beg += cnt[g];
    }
}

// The device loop as one graph: init, then WHILE (conditional node) { select, [mixed:
// FP64 re-evaluations, second selection pass], scan, [mixed: re-evaluations], rule
// evaluation per group }.  `init` = false leaves the states as they are (serving).
int build_graph_ws(g3l_ctx *c, Workspace &W, int precision, int gmask, bool init,
                   GraphEntry &out)
{
    KernelArgs a{c->T, W.D, W.S, W.P, W.H, W.woff, 0, 1, c->T.tau_sel, c->T.tau_val};
    cudaGraph_t g;
    G3L_CK(cudaGraphCreate(&g, 0));
    cudaGraphNode_t n_init;
    if (init) {
        void *args[] = {&a.D, &a.S, &a.P, &a.H};
        int st = add_kernel(g, &n_init, nullptr, 0, init_kernel(), c->nsm * 4, 256, args);
        if (st) return st;
    }
    G3L_CK(cudaGraphConditionalHandleCreate(&a.handle, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = a.handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t n_while;
    G3L_CK(cudaGraphAddNode(&n_while, g, init ? &n_init : nullptr, nullptr, init ? 1 : 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaGraphNode_t n_sel, n_scan, prev;
    // mixed: FP64 re-evaluations queued by a selection pass (unsettled splits of the
    // parents about to be cut, ambiguous boundary regions, polish), then the round end
    // (one branch per group, side by side: each group reads only its own queue).  With
    // ends != null each group's branch gets its own end node (ends[grp]) and dep is left
    // as it is: the rule kernel of a group then waits for its own re-evaluations only.
    auto add_reevals = [&](cudaGraphNode_t &dep, cudaGraphNode_t *ends) -> int {
        cudaGraphNode_t br[2 * NGROUPS];
        int nbr = 0;
        for (int grp = 0; grp < NGROUPS; ++grp) {
            if (!(gmask & (1 << grp))) continue;
            const int nbr0 = nbr;
            void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
            cudaGraphNode_t chain = dep;
            for (int ph = 0; ph < 4; ++ph) {
                void *fn = reeval_phase_kernel(grp / 3, grp % 3 + 1, ph);
                cudaGraphNode_t nd;
                int st = add_kernel(body, &nd, &chain, 1, fn, ph == 3 ? c->nsm : grid128(c, fn), 128,
                                    args);
                if (st) return st;
                chain = nd;
            }
            br[nbr++] = chain;
            void *fn = reeval_phase_kernel(grp / 3, grp % 3 + 1, 4);
            int st = add_kernel(body, &br[nbr], &dep, 1, fn, reeval_grid(c, fn), 128, args);
            if (st) return st;
            ++nbr;
            if (ends) {
                void *eargs[] = {&a.H, &a.grp_id[grp]};
                st = add_kernel(body, &ends[grp], &br[nbr0], 2, round_end_kernel(), 1, 1, eargs);
                if (st) return st;
            }
        }
        if (ends) return G3L_OK;
        void *args[] = {&a.H, &a.all_groups};
        cudaGraphNode_t n_end;
        int st = add_kernel(body, &n_end, nbr ? br : &dep, nbr ? nbr : 1, round_end_kernel(), 1,
                            1, args);
        if (st) return st;
        dep = n_end;
        return G3L_OK;
    };
    {
        void *args[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass0};
        int st = add_kernel(body, &n_sel, nullptr, 0, select_kernel(), c->nsm * 8, 256, args);
        if (st) return st;
    }
    prev = n_sel;
    if (precision == G3L_MIXED) {
        int st = add_reevals(prev, nullptr);
        if (st) return st;
        void *args[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass1};
        cudaGraphNode_t n_sel1;
        st = add_kernel(body, &n_sel1, &prev, 1, select_kernel(), c->nsm * 8, 256, args);
        if (st) return st;
        prev = n_sel1;
    }
    {
        void *args[] = {&a.S, &a.woff, &a.H, &a.handle, &a.use_cond};
        int st = add_kernel(body, &n_scan, &prev, 1, scan_kernel(), 1, 1024, args);
        if (st) return st;
    }
    prev = n_scan;
    cudaGraphNode_t ends[NGROUPS];
    if (precision == G3L_MIXED) {
        int st = add_reevals(prev, ends);
        if (st) return st;
    }
    // the groups' rule kernels in a chain (side-by-side branches measured slower: each
    // kernel fills the device, and concurrent ones contend for it); a group's kernel
    // waits for the previous one and its own re-evaluations, so the other groups'
    // re-evaluations run beside it
    for (int grp = 0; grp < NGROUPS; ++grp) {
        if (!(gmask & (1 << grp))) continue;
        void *fn = eval_fn(c, precision, grp);
        void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
        cudaGraphNode_t n_ev, deps[2] = {prev, ends[grp]};
        int st = add_kernel(body, &n_ev, deps, precision == G3L_MIXED ? 2 : 1, fn,
                            eval_grid(c, fn), 128, args);
        if (st) return st;
        prev = n_ev;
    }
    cudaGraphExec_t ex;
    G3L_CK(cudaGraphInstantiate(&ex, g, 0));
    out = GraphEntry{W.gen, precision, gmask, g, ex};
    return G3L_OK;
}

int build_graph(g3l_ctx *c, int precision, int gmask, GraphEntry &out)
{
    return build_graph_ws(c, c->W, precision, gmask, true, out);
}

// descriptor of one integral: bounds and root geometry as the reference computes them
// (src/NNMap_Model.cu:46-49, 313-314; src/hcubature.cpp:160-172), plus the
// mixed-precision constants
bool item_ok(const g3l_ctx *c, const g3l_integral &it)
{
    bool ok = (it.kind == G3L_NNMAP || it.kind == G3L_NMAPMAP) && it.term >= 1 && it.term <= 3 &&
              it.hod1 >= 0 && it.hod1 < MAX_HOD_SLOTS && c->hod_set[it.hod1] &&
              std::isfinite(it.rtol) && it.rtol >= 0;
    if (ok && it.kind == G3L_NNMAP)
        ok = it.hod2 >= 0 && it.hod2 < MAX_HOD_SLOTS && c->hod_set[it.hod2];
    for (int k = 0; k < 3 && ok; ++k) ok = std::isfinite(it.theta[k]) && it.theta[k] > 0;
    return ok;
}

void fill_desc(const g3l_ctx *c, const g3l_integral &it, int precision, IntDesc &d)
{
    std::memset(&d, 0, sizeof d);
    for (int k = 0; k < 3; ++k) d.theta[k] = it.theta[k];
    double lo[MAX_DIM], hi[MAX_DIM];
    d.dim = c->B.bounds(it.term, lo, hi);
    for (int k = 0; k < d.dim; ++k) {
        d.c0[k] = 0.5 * (lo[k] + hi[k]);
        d.hw0[k] = 0.5 * (hi[k] - lo[k]);
    }
    double vol = 1;
    for (int k = 0; k < d.dim; ++k) vol *= 2 * d.hw0[k];
    d.rootvol = vol;
    if (precision == G3L_MIXED) {
        static const double lam[3] = {G3L_LAMBDA2, G3L_LAMBDA4, G3L_LAMBDA5};
        for (int k = 0; k < d.dim; ++k)
            for (int q = 0; q < 3; ++q) d.hwl[k][q] = dsplit(d.hw0[k] * lam[q]);
        for (int k = 0; k < 3; ++k) d.th_s[k] = (float)(it.theta[k] * kL0);
        const int h2 = it.kind == G3L_NNMAP ? it.hod2 : it.hod1;
        d.rootvol_mx = vol * mixed_scale(c, it.kind, it.term, it.hod1, h2);
    }
    d.rtol = it.rtol;
    d.scale = 1.0;
    d.max_eval = it.max_eval;
    d.kind = it.kind;
    d.term = it.term;
    d.npts = rule_points(d.dim);
    d.hod1 = it.hod1;
    d.hod2 = it.kind == G3L_NNMAP ? it.hod2 : it.hod1;
    d.same = d.hod1 == d.hod2;
}

int run_host_loop(g3l_ctx *c, int precision, int gmask, int *launches)
{
    Workspace &W = c->W;
    KernelArgs a{c->T, W.D, W.S, W.P, W.H, W.woff, 0, 0, c->T.tau_sel, c->T.tau_val};
    cudaStream_t s = c->stream;
    {
        void *args[] = {&a.D, &a.S, &a.P, &a.H};
        G3L_CK(cudaLaunchKernel(init_kernel(), dim3(c->nsm * 4), dim3(256), args, 0, s));
        ++*launches;
    }
    for (int g = 0; g < NGROUPS; ++g) c->stats.group_ms[g] = 0;
    c->stats.reeval_ms = 0;
    c->stats.select_ms = 0;
    float ms;
    auto reevals = [&]() -> int {
        G3L_CK(cudaEventRecord(c->tev[12], s));
        for (int grp = 0; grp < NGROUPS; ++grp) {
            if (!(gmask & (1 << grp))) continue;
            void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
            for (int ph = 0; ph < 5; ++ph) {
                void *fn = reeval_phase_kernel(grp / 3, grp % 3 + 1, ph);
                const int grid = ph == 3 ? c->nsm : (ph == 4 ? reeval_grid(c, fn) : grid128(c, fn));
                G3L_CK(cudaLaunchKernel(fn, dim3(grid), dim3(128), args, 0, s));
                ++*launches;
            }
        }
        G3L_CK(cudaEventRecord(c->tev[13], s));
        void *eargs[] = {&a.H, &a.all_groups};
        G3L_CK(cudaLaunchKernel(round_end_kernel(), dim3(1), dim3(1), eargs, 0, s));
        ++*launches;
        G3L_CK(cudaEventSynchronize(c->tev[13]));
        cudaEventElapsedTime(&ms, c->tev[12], c->tev[13]);
        c->stats.reeval_ms += ms;
        return G3L_OK;
    };
    for (int r = 0; r < c->opt.max_rounds + 4; ++r) {
        NvtxScope nv("round");
        void *sargs[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass0};
        G3L_CK(cudaEventRecord(c->tev[14], s));
        G3L_CK(cudaLaunchKernel(select_kernel(), dim3(c->nsm * 8), dim3(256), sargs, 0, s));
        G3L_CK(cudaEventRecord(c->tev[15], s));
        ++*launches;
        G3L_CK(cudaEventSynchronize(c->tev[15]));
        cudaEventElapsedTime(&ms, c->tev[14], c->tev[15]);
        c->stats.select_ms += ms;
        if (precision == G3L_MIXED) {
            int st = reevals();
            if (st) return st;
            void *sargs1[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass1};
            G3L_CK(cudaEventRecord(c->tev[14], s));
            G3L_CK(cudaLaunchKernel(select_kernel(), dim3(c->nsm * 8), dim3(256), sargs1, 0, s));
            ++*launches;
        } else {
            G3L_CK(cudaEventRecord(c->tev[14], s));
        }
        void *cargs[] = {&a.S, &a.woff, &a.H, &a.handle, &a.use_cond};
        G3L_CK(cudaLaunchKernel(scan_kernel(), dim3(1), dim3(1024), cargs, 0, s));
        G3L_CK(cudaEventRecord(c->tev[15], s));
        ++*launches;
        G3L_CK(cudaEventSynchronize(c->tev[15]));
        cudaEventElapsedTime(&ms, c->tev[14], c->tev[15]);
        c->stats.select_ms += ms;
        if (precision == G3L_MIXED) {
            int st = reevals();
            if (st) return st;
        }
        for (int grp = 0; grp < NGROUPS; ++grp) {
            if (!(gmask & (1 << grp))) continue;
            void *fn = eval_fn(c, precision, grp);
            void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
            G3L_CK(cudaEventRecord(c->tev[2 * grp], s));
            G3L_CK(cudaLaunchKernel(fn, dim3(eval_grid(c, fn)), dim3(128), args, 0, s));
            G3L_CK(cudaEventRecord(c->tev[2 * grp + 1], s));
            ++*launches;
        }
        G3L_CK(cudaMemcpyAsync(c->h_pinned, &W.H->any_active, sizeof(int),
                               cudaMemcpyDeviceToHost, s));
        G3L_CK(cudaStreamSynchronize(s));
        for (int grp = 0; grp < NGROUPS; ++grp)
            if (gmask & (1 << grp)) {
                cudaEventElapsedTime(&ms, c->tev[2 * grp], c->tev[2 * grp + 1]);
                c->stats.group_ms[grp] += ms;
            }
        if (*(int *)c->h_pinned == 0) break;
    }
    return G3L_OK;
}

}  // namespace

// ------------------------------------------------------------------ serving
//
// A server keeps a table of integral slots (one segment per kind x term group, so the
// rule kernels see each group contiguously) and a region pool on the device, and runs
// the same device loop as g3l_eval in launches of a few rounds.  Between launches its
// driver thread collects finished integrals, completes their requests, returns their
// slots and pool ranges, and admits waiting requests (first come, first served) as
// slots and pool space allow.  The trajectory of every integral depends only on its
// own regions, so a result is the same alone and in any mix.
namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct SrvReq {
    std::vector<IntDesc> desc;  // per item; base filled at admission
    std::vector<int> slot;      // table slot per item (-1 before admission)
    std::vector<g3l_result> res;
    int remaining = 0;
    bool admitted = false, done = false, cancel = false;
    double t_submit = 0, t_done = 0;
    nvtxRangeId_t range = 0;  // NVTX range from submission to completion
};

// a request is complete: close its NVTX range and record the time
void req_done(SrvReq &q, double t)
{
    q.done = true;
    q.t_done = t;
    if (q.range) nvtxRangeEnd(q.range);
    q.range = 0;
}

// First-fit allocator of pool slot ranges.
struct RangeAlloc {
    std::map<long long, long long> free_;  // start -> length
    long long total_free = 0;
    void init(long long n)
    {
        free_.clear();
        free_[0] = n;
        total_free = n;
    }
    long long take(long long n)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                const long long b = it->first, len = it->second;
                free_.erase(it);
                if (len > n) free_[b + n] = len - n;
                total_free -= n;
                return b;
            }
        return -1;
    }
    void give(long long b, long long n)
    {
        total_free += n;
        auto it = free_.emplace(b, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

}  // namespace

struct g3l_server {
    g3l_ctx *c = nullptr;
    int precision = G3L_MIXED;
    int per_group = 0, n = 0, chunk = 4;
    size_t pool = 0;
    cudaStream_t s = nullptr;
    Workspace W;
    GraphEntry G{};
    bool graph_ok = false;
    std::vector<IntState> Sh;       // host copy of the states after each launch
    std::vector<int64_t> slot_req;  // slot -> ticket (0 = free)
    std::vector<int> slot_item;
    std::vector<std::vector<int>> free_slots;  // per group
    RangeAlloc ra;
    std::map<int64_t, SrvReq> reqs;
    std::deque<int64_t> pending;
    int64_t next_ticket = 1;
    int active = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread th;
    bool stop = false;
    int fatal = G3L_OK;
    std::string fatal_msg;
    IntDesc *d_new = nullptr;  // admission staging (device)
    int *d_idx = nullptr;
    uint64_t launches = 0, admitted_total = 0, completed_total = 0;
};

namespace {

// Admit waiting requests in order while their items fit (caller holds the lock).
void srv_admit(g3l_server *v, std::vector<IntDesc> &nd, std::vector<int> &ni)
{
    while (!v->pending.empty()) {
        const int64_t t = v->pending.front();
        SrvReq &q = v->reqs[t];
        if (q.cancel) {
            v->pending.pop_front();
            for (auto &r : q.res) r.status = G3L_ERR_CANCELLED;
            req_done(q, now_s());
            continue;
        }
        const int m = (int)q.desc.size();
        int need[NGROUPS] = {};
        for (const IntDesc &d : q.desc) ++need[d.kind * 3 + d.term - 1];
        bool ok = true;
        for (int g = 0; g < NGROUPS; ++g) ok &= (int)v->free_slots[g].size() >= need[g];
        if (!ok) break;
        std::vector<long long> bases(m, -1);
        for (int k = 0; k < m && ok; ++k) {
            bases[k] = v->ra.take(q.desc[k].cap);
            if (bases[k] < 0) ok = false;
        }
        if (!ok) {
            for (int k = 0; k < m; ++k)
                if (bases[k] >= 0) v->ra.give(bases[k], q.desc[k].cap);
            break;
        }
        v->pending.pop_front();
        for (int k = 0; k < m; ++k) {
            IntDesc &d = q.desc[k];
            auto &fs = v->free_slots[d.kind * 3 + d.term - 1];
            const int sl = fs.back();
            fs.pop_back();
            d.base = bases[k];
            q.slot[k] = sl;
            v->slot_req[sl] = t;
            v->slot_item[sl] = k;
            v->Sh[sl] = IntState{};
            nd.push_back(d);
            ni.push_back(sl);
        }
        q.admitted = true;
        v->active += m;
        v->admitted_total += 1;
    }
}

void srv_fail_all(g3l_server *v, int st, const std::string &msg)
{
    std::lock_guard<std::mutex> lk(v->mu);
    v->fatal = st;
    v->fatal_msg = msg;
    for (auto &kv : v->reqs)
        if (!kv.second.done) {
            for (auto &r : kv.second.res) r.status = st;
            req_done(kv.second, now_s());
        }
    v->pending.clear();
    v->cv_done.notify_all();
}

#define SRV_CK(x)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            srv_fail_all(v, G3L_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
            return;                                                                 \
        }                                                                           \
    } while (0)

void srv_loop(g3l_server *v)
{
    cudaSetDevice(v->c->device);
    std::vector<IntDesc> nd;
    std::vector<int> ni;
    std::vector<int> cancel_slots;
    BatchHdr H{};
    for (;;) {
        nd.clear();
        ni.clear();
        cancel_slots.clear();
        long long cnt[NGROUPS] = {};
        {
            std::unique_lock<std::mutex> lk(v->mu);
            v->cv_work.wait(lk, [&] { return v->stop || !v->pending.empty() || v->active > 0; });
            if (v->stop) return;
            srv_admit(v, nd, ni);
            v->cv_done.notify_all();  // requests cancelled while queued
            for (int i = 0; i < v->n; ++i) {
                const int64_t t = v->slot_req[i];
                if (!t) continue;
                const SrvReq &q = v->reqs[t];
                if (q.cancel && !v->Sh[i].done) cancel_slots.push_back(i);
                const IntDesc &d = q.desc[v->slot_item[i]];
                cnt[d.kind * 3 + d.term - 1] += d.cap;
            }
            if (v->active == 0) continue;
        }
        cudaStream_t s = v->s;
        if (!nd.empty()) {
            const int m = (int)nd.size();
            SRV_CK(cudaMemcpyAsync(v->d_new, nd.data(), sizeof(IntDesc) * m, cudaMemcpyHostToDevice, s));
            SRV_CK(cudaMemcpyAsync(v->d_idx, ni.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s));
            void *args[] = {&v->d_new, &v->d_idx, (void *)&m, &v->W.D, &v->W.S, &v->W.P};
            SRV_CK(cudaLaunchKernel(admit_kernel(), dim3((m + 127) / 128), dim3(128), args, 0, s));
            SRV_CK(cudaStreamSynchronize(s));  // m and the staging must outlive the launch
        }
        for (int i : cancel_slots) {
            IntState st{};
            st.done = 1;
            st.status = G3L_ERR_CANCELLED;
            SRV_CK(cudaMemcpyAsync(v->W.S + i, &st, sizeof st, cudaMemcpyHostToDevice, s));
        }
        // header: fixed table layout, this launch's re-evaluation queues and round budget
        H = BatchHdr{};
        H.n = v->n;
        for (int g = 0; g <= NGROUPS; ++g) H.gbeg[g] = g * v->per_group;
        H.max_rounds = v->c->opt.max_rounds;
        H.mixed = v->precision == G3L_MIXED ? 1 : 0;
        H.chunk_rounds = v->chunk;
        H.thr_ratio = (float)v->c->opt.unc_thr;
        H.tau_thr = v->c->opt.unc_tau_thr;
        H.val_ratio = (float)(v->c->opt.unc_eps_sel / std::max(v->c->opt.unc_eps_val, 1e-30));
        long long beg = 0;
        for (int g = 0; g < NGROUPS; ++g) {
            H.esc_beg[g] = beg;
            H.esc_cap[g] = (int)std::min<long long>(cnt[g], 0x7fffffff);
            beg += cnt[g];
        }
        SRV_CK(cudaMemcpyAsync(v->W.H, &H, sizeof H, cudaMemcpyHostToDevice, s));
        NvtxScope nv("server launch");
        SRV_CK(cudaGraphLaunch(v->G.exec, s));
        SRV_CK(cudaMemcpyAsync(v->Sh.data(), v->W.S, sizeof(IntState) * v->n, cudaMemcpyDeviceToHost, s));
        SRV_CK(cudaStreamSynchronize(s));
        SRV_CK(cudaGetLastError());
        {
            std::lock_guard<std::mutex> lk(v->mu);
            v->launches += 1;
            const double t = now_s();
            for (int i = 0; i < v->n; ++i) {
                const int64_t tk = v->slot_req[i];
                if (!tk || !v->Sh[i].done) continue;
                SrvReq &q = v->reqs[tk];
                const int k = v->slot_item[i];
                const IntDesc &d = q.desc[k];
                const IntState &sr = v->Sh[i];
                g3l_result &o = q.res[k];
                o.val = sr.val * d.scale;
                o.err = sr.err * d.scale;
                o.neval = sr.neval;
                o.status = sr.status;
                o.rounds = sr.rounds;
                o.result = host::apply_prefactor(d.kind, d.term, v->c->H0, v->c->Om, o.val);
                v->slot_req[i] = 0;
                v->free_slots[d.kind * 3 + d.term - 1].push_back(i);
                v->ra.give(d.base, d.cap);
                v->active -= 1;
                if (--q.remaining == 0) {
                    req_done(q, t);
                    v->completed_total += 1;
                }
            }
            v->cv_done.notify_all();
        }
    }
}

void srv_destroy(g3l_server *v)
{
    if (!v) return;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        v->stop = true;
    }
    v->cv_work.notify_all();
    if (v->th.joinable()) v->th.join();
    for (auto &kv : v->reqs)
        if (kv.second.range) nvtxRangeEnd(kv.second.range);
    cudaSetDevice(v->c->device);
    if (v->s) cudaStreamSynchronize(v->s);
    if (v->graph_ok) {
        cudaGraphExecDestroy(v->G.exec);
        cudaGraphDestroy(v->G.graph);
    }
    free_workspace(v->W);
    if (v->d_new) cudaFree(v->d_new);
    if (v->d_idx) cudaFree(v->d_idx);
    if (v->s) cudaStreamDestroy(v->s);
    delete v;
}

int srv_create(g3l_ctx *c, int precision, int per_group, uint64_t pool_regions, int chunk,
               g3l_server **out)
{
    if (!c || !out || (precision != G3L_FP64 && precision != G3L_MIXED) || per_group < 1 ||
        per_group > (1 << 20) || pool_regions < 64 || pool_regions > (1ull << 31) || chunk < 1) {
        host::set_error("g3l_server_create: invalid arguments");
        return G3L_ERR_INVALID;
    }
    if (precision == G3L_MIXED && !evalmx_kernel(0, 1)) {
        host::set_error("g3l_server_create: mixed-precision kernels not built");
        return G3L_ERR_INVALID;
    }
    G3L_CK(cudaSetDevice(c->device));
    auto *v = new g3l_server;
    v->c = c;
    v->precision = precision;
    v->per_group = per_group;
    v->n = NGROUPS * per_group;
    v->pool = (size_t)pool_regions;
    v->chunk = chunk;
    int st = G3L_OK;
    if (cudaStreamCreateWithFlags(&v->s, cudaStreamNonBlocking) != cudaSuccess) st = G3L_ERR_CUDA;
    if (!st) st = alloc_workspace(v->W, v->n, v->pool, c->retab_d);
    if (!st) st = dalloc(&v->d_new, (size_t)v->n) | dalloc(&v->d_idx, (size_t)v->n);
    if (!st) st = build_graph_ws(c, v->W, precision, (1 << NGROUPS) - 1, false, v->G);
    if (!st) v->graph_ok = true;
    if (!st) {
        // every slot starts free: a finished state, never selected
        v->Sh.assign(v->n, IntState{});
        for (auto &x : v->Sh) x.done = 1;
        if (cudaMemcpy(v->W.S, v->Sh.data(), sizeof(IntState) * v->n, cudaMemcpyHostToDevice) !=
            cudaSuccess)
            st = G3L_ERR_CUDA;
    }
    if (st) {
        if (st == G3L_ERR_NOMEM) host::set_error("g3l_server_create: device allocation failed");
        srv_destroy(v);
        return st;
    }
    v->slot_req.assign(v->n, 0);
    v->slot_item.assign(v->n, 0);
    v->free_slots.assign(NGROUPS, {});
    for (int g = 0; g < NGROUPS; ++g)
        for (int k = per_group - 1; k >= 0; --k) v->free_slots[g].push_back(g * per_group + k);
    v->ra.init((long long)v->pool);
    v->th = std::thread(srv_loop, v);
    *out = v;
    return G3L_OK;
}

int srv_submit(g3l_server *v, const g3l_integral *items, int n, int64_t *ticket)
{
    if (!v || !ticket || n < 1 || !items) {
        host::set_error("g3l_server_submit: invalid arguments");
        return G3L_ERR_INVALID;
    }
    SrvReq q;
    q.desc.resize(n);
    q.slot.assign(n, -1);
    q.res.assign(n, g3l_result{});
    q.remaining = n;
    int need[NGROUPS] = {};
    for (int i = 0; i < n; ++i) {
        if (!item_ok(v->c, items[i])) {
            host::set_error("g3l_server_submit: invalid integral " + std::to_string(i));
            return G3L_ERR_INVALID;
        }
        IntDesc &d = q.desc[i];
        fill_desc(v->c, items[i], v->precision, d);
        unsigned long long cap = items[i].max_eval
                                     ? 3 + (items[i].max_eval + d.npts) / (2ull * d.npts)
                                     : v->c->opt.unlimited_pool;
        if (cap > v->pool) {
            host::set_error("g3l_server_submit: integral " + std::to_string(i) +
                            " needs more region slots than the server's pool");
            return G3L_ERR_INVALID;
        }
        d.cap = (int)cap;
        ++need[d.kind * 3 + d.term - 1];
    }
    for (int g = 0; g < NGROUPS; ++g)
        if (need[g] > v->per_group) {
            host::set_error("g3l_server_submit: more integrals of one kind and term than the "
                            "server's slots for it");
            return G3L_ERR_INVALID;
        }
    std::lock_guard<std::mutex> lk(v->mu);
    if (v->fatal) {
        host::set_error("g3l_server_submit: server stopped: " + v->fatal_msg);
        return v->fatal;
    }
    q.t_submit = now_s();
    const int64_t t = v->next_ticket++;
    {
        char nm[40];
        std::snprintf(nm, sizeof nm, "request %lld", (long long)t);
        q.range = nvtxRangeStartA(nm);
    }
    v->reqs.emplace(t, std::move(q));
    v->pending.push_back(t);
    *ticket = t;
    v->cv_work.notify_all();
    return G3L_OK;
}

int srv_poll(g3l_server *v, int64_t ticket, g3l_result *out, int wait_ms, double *latency_ms)
{
    if (!v) {
        host::set_error("g3l_server_poll: no server");
        return G3L_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lk(v->mu);
    auto it = v->reqs.find(ticket);
    if (it == v->reqs.end()) {
        host::set_error("g3l_server_poll: unknown ticket");
        return G3L_ERR_INVALID;
    }
    if (!it->second.done && wait_ms != 0) {
        auto pred = [&] { return v->reqs.at(ticket).done; };
        if (wait_ms < 0) v->cv_done.wait(lk, pred);
        else v->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), pred);
    }
    it = v->reqs.find(ticket);
    if (!it->second.done) return G3L_ERR_BUSY;
    SrvReq &q = it->second;
    int first_bad = G3L_OK;
    for (auto &r : q.res)
        if (r.status && !first_bad) first_bad = r.status;
    if (out) std::copy(q.res.begin(), q.res.end(), out);
    if (latency_ms) *latency_ms = 1e3 * (q.t_done - q.t_submit);
    v->reqs.erase(it);
    if (first_bad) host::set_error("g3l_server_poll: an integral ended with status " + std::to_string(first_bad));
    return first_bad;
}

int srv_cancel(g3l_server *v, int64_t ticket)
{
    if (!v) {
        host::set_error("g3l_server_cancel: no server");
        return G3L_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(v->mu);
    auto it = v->reqs.find(ticket);
    if (it == v->reqs.end()) {
        host::set_error("g3l_server_cancel: unknown or already polled ticket");
        return G3L_ERR_INVALID;
    }
    if (it->second.done) return G3L_OK;  // finished before the cancel: its results stand
    SrvReq &q = it->second;
    q.cancel = true;
    if (!q.admitted) {  // still queued: finish it now
        v->pending.erase(std::find(v->pending.begin(), v->pending.end(), ticket));
        for (auto &r : q.res) r.status = G3L_ERR_CANCELLED;
        q.done = true;
        q.t_done = now_s();
        v->cv_done.notify_all();
    }
    v->cv_work.notify_all();
    return G3L_OK;
}

g3l_server *ctx_server(g3l_ctx *c, int precision, int *st)
{
    std::lock_guard<std::mutex> lk(c->srv_mu);
    g3l_server *&v = c->srv[precision == G3L_MIXED ? 1 : 0];
    if (!v) *st = srv_create(c, precision, 1024, 1ull << 22, 4, &v);
    return v;
}

}  // namespace

extern "C" {

const char *g3l_last_error(void) { return host::last_error_cstr(); }
int g3l_abi_version(void) { return G3L_ABI_VERSION; }
int g3l_max_hod_slots(void) { return MAX_HOD_SLOTS; }

int g3l_host_densities(const g3l_tables *t, const double hod[6], double *rho_bar, double *n_bar)
try {
    if (!t || !hod || !rho_bar || !n_bar || t->Nz < 2 || t->Nm < 2) {
        host::set_error("g3l_host_densities: invalid arguments");
        return G3L_ERR_INVALID;
    }
    host::Binning B{t->Nz, t->Nm, t->Nk, t->zmin, t->zmax, t->mmin, t->mmax, t->kmin, t->kmax};
    host::rho_bar(B, t->Om, t->OL, t->H0, rho_bar);
    if (host::n_bar(B, t->hmf, hod, n_bar)) return G3L_ERR_INVALID;
    return G3L_OK;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_host_densities: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_host_densities: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_ctx_create(const g3l_tables *t, int device, g3l_ctx **out)
try {
    if (!out) return G3L_ERR_INVALID;
    *out = nullptr;
    if (!t || t->Nz < 2 || t->Nm < 2 || t->Nk < 2 || !t->g || !t->p_lens1 || !t->p_lens2 || !t->w ||
        !t->dwdz || !t->hmf || !t->b_h || !t->conc || !t->P_lin) {
        host::set_error("g3l_ctx_create: missing tables or bins < 2");
        return G3L_ERR_INVALID;
    }
    if (!(t->zmax > t->zmin) || !(t->mmax > t->mmin) || !(t->mmin > 0) || !(t->kmax > t->kmin) ||
        !(t->kmin > 0) || !(t->H0 > 0)) {
        host::set_error("g3l_ctx_create: invalid binning or cosmology");
        return G3L_ERR_INVALID;
    }
    const size_t Nz = t->Nz, Nm = t->Nm, Nk = t->Nk;
    const double *z1[] = {t->g, t->p_lens1, t->p_lens2, t->w, t->dwdz};
    for (const double *a : z1)
        if (!finite_all(a, Nz)) {
            host::set_error("g3l_ctx_create: non-finite value in a redshift table");
            return G3L_ERR_INVALID;
        }
    if (!finite_all(t->hmf, Nz * Nm) || !finite_all(t->b_h, Nz * Nm) || !finite_all(t->conc, Nz * Nm) ||
        !finite_all(t->P_lin, Nz * Nk)) {
        host::set_error("g3l_ctx_create: non-finite value in a 2-D table");
        return G3L_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
        host::set_error("g3l_ctx_create: no CUDA device");
        return G3L_ERR_NO_DEVICE;
    }
    std::unique_ptr<g3l_ctx> c(new g3l_ctx);
    c->device = device;
    G3L_CK(cudaSetDevice(device));
    G3L_CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
    G3L_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    G3L_CK(cudaEventCreate(&c->ev0));
    G3L_CK(cudaEventCreate(&c->ev1));
    for (auto &e : c->tev) G3L_CK(cudaEventCreate(&e));
    G3L_CK(cudaMallocHost(&c->h_pinned, 64));
    G3L_CK(cudaHostAlloc((void **)&c->cancel_h, 64, cudaHostAllocMapped));
    *c->cancel_h = 0;
    G3L_CK(cudaHostGetDevicePointer((void **)&c->cancel_d, c->cancel_h, 0));
    G3L_CK(cudaMalloc((void **)&c->retab_d, (size_t)NGROUPS * RETAB_BYTES));
    G3L_CK(build_reeval_tables(c->retab_d, c->stream));
    G3L_CK(cudaStreamSynchronize(c->stream));
    c->B = host::Binning{t->Nz, t->Nm, t->Nk, t->zmin, t->zmax, t->mmin, t->mmax, t->kmin, t->kmax};
    c->Om = t->Om;
    c->OL = t->OL;
    c->Ob = t->Ob;
    c->s8 = t->sigma8;
    c->H0 = t->H0;
    c->ns = t->ns;
    c->hmf_h.assign(t->hmf, t->hmf + Nz * Nm);
    c->rho_h.resize(Nz);
    host::rho_bar(c->B, t->Om, t->OL, t->H0, c->rho_h.data());
    c->hod_h.assign((size_t)MAX_HOD_SLOTS * 6, 0.0);
    c->nbar_h.assign((size_t)MAX_HOD_SLOTS * Nz, 0.0);
    c->fnbar_h.assign((size_t)MAX_HOD_SLOTS * Nz, 0.f);
    c->fhodp_h.assign((size_t)MAX_HOD_SLOTS * 8, 0.f);
    c->hod_set.assign(MAX_HOD_SLOTS, 0);
    c->opt.eval_blocks_per_sm = 0;
    c->opt.eval_warps_per_block = 0;
    c->opt.use_graph = 1;
    c->opt.max_rounds = 4096;
    c->opt.unlimited_pool = 1 << 20;
    c->opt.small_arg = 1e-7;
    // Point-value bounds: FP32 chains with tail amplification (aperture filter,
    // occupation tails) reach ~1e-5 relative, so decisions use 5e-5; the value-noise
    // estimate uses the typical 5e-6.  Every unsettled split is re-evaluated
    // (impact 0); finished integrals whose value noise may exceed 5e-5 of the value
    // are polished in FP64.
    c->opt.unc_eps_rel = 5e-5;
    c->opt.unc_tau_abs = 1e-34;
    c->opt.unc_tau_impact = 0.0;
    c->opt.unc_tau_sel = 1e-7;
    c->opt.unc_tau_val = 5e-5;
    c->opt.unc_eps_val = 5e-6;
    c->opt.unc_eps_sel = 5e-5;
    c->opt.unc_thr = 0.1;
    c->opt.unc_tau_thr = 1e-6;
    // register-budget variant of the rule kernels per kind x term (autotuned default:
    // 8 blocks per SM for the 1-halo terms, 6 for the 2- and 3-halo terms)
    for (int g = 0; g < NGROUPS; ++g) c->opt.evalmx_variant[g] = g % 3 == 0 ? 2 : 1;

    DevTables &T = c->T;
    T.Nz = t->Nz;
    T.Nm = t->Nm;
    T.Nk = t->Nk;
    T.clamp_k = t->clamp_k ? 1 : 0;
    T.zmin = t->zmin;
    T.zmax = t->zmax;
    T.mmin = t->mmin;
    T.mmax = t->mmax;
    T.kmin = t->kmin;
    T.kmax = t->kmax;
    T.ln_mratio = std::log(t->mmax / t->mmin);
    T.ln_kratio = std::log(t->kmax / t->kmin);
    T.m_x0 = std::log10(t->mmin);
    T.m_scale = t->Nm / std::log10(t->mmax / t->mmin);
    int st = 0;
    st |= upload(c.get(), t->g, Nz, &T.g);
    st |= upload(c.get(), t->p_lens1, Nz, &T.p1);
    st |= upload(c.get(), t->p_lens2, Nz, &T.p2);
    st |= upload(c.get(), t->w, Nz, &T.w);
    st |= upload(c.get(), t->dwdz, Nz, &T.dwdz);
    st |= upload(c.get(), c->rho_h.data(), Nz, &T.rho_bar);
    st |= upload(c.get(), t->hmf, Nz * Nm, &T.hmf);
    st |= upload(c.get(), t->b_h, Nz * Nm, &T.b_h);
    st |= upload(c.get(), t->conc, Nz * Nm, &T.conc);
    st |= upload(c.get(), t->P_lin, Nz * Nk, &T.P_lin);
    if (st) return st;
    st |= dalloc(&c->d_hod, (size_t)MAX_HOD_SLOTS * 6);
    st |= dalloc(&c->d_nbar, (size_t)MAX_HOD_SLOTS * Nz);
    if (st) return st;
    c->allocs.push_back(c->d_hod);
    c->allocs.push_back(c->d_nbar);
    G3L_CK(cudaMemset(c->d_hod, 0, sizeof(double) * MAX_HOD_SLOTS * 6));
    G3L_CK(cudaMemset(c->d_nbar, 0, sizeof(double) * MAX_HOD_SLOTS * Nz));
    T.hod = c->d_hod;
    T.nbar = c->d_nbar;
    // satellite-variance rescaling per slot, s = 1 (FP32: s^2 - 1 = 0) until set
    st |= dalloc(&c->d_scale, (size_t)MAX_HOD_SLOTS * Nm);
    st |= dalloc(&c->d_fscale, (size_t)MAX_HOD_SLOTS * Nm);
    if (st) return st;
    c->allocs.push_back(c->d_scale);
    c->allocs.push_back(c->d_fscale);
    {
        std::vector<double> ones((size_t)MAX_HOD_SLOTS * Nm, 1.0);
        G3L_CK(cudaMemcpy(c->d_scale, ones.data(), ones.size() * sizeof(double),
                          cudaMemcpyHostToDevice));
    }
    G3L_CK(cudaMemset(c->d_fscale, 0, sizeof(float) * MAX_HOD_SLOTS * Nm));
    T.scale = c->d_scale;
    T.f_scale = c->d_fscale;
    // tie-prone mass-centre indices
    host::TieTable tt = host::build_m_ties(c->B);
    unsigned long long *tb;
    int *tr, *tq;
    st |= dalloc(&tb, tt.bits.size());
    st |= dalloc(&tr, tt.bits.size());
    st |= dalloc(&tq, tt.bits.size());
    if (st) return st;
    c->allocs.push_back(tb);
    c->allocs.push_back(tr);
    c->allocs.push_back(tq);
    G3L_CK(cudaMemcpy(tb, tt.bits.data(), tt.bits.size() * 8, cudaMemcpyHostToDevice));
    G3L_CK(cudaMemcpy(tr, tt.round_ix.data(), tt.bits.size() * 4, cudaMemcpyHostToDevice));
    G3L_CK(cudaMemcpy(tq, tt.trunc_ix.data(), tt.bits.size() * 4, cudaMemcpyHostToDevice));
    T.tie_m_bits = tb;
    T.tie_m_round = tr;
    T.tie_m_trunc = tq;
    T.n_tie_m = (int)tt.bits.size();
    st = prepare_mixed(c.get(), t);
    if (st) return st;
    *out = c.release();
    return G3L_OK;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_ctx_create: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_ctx_create: ") + e.what());
    return G3L_ERR_INVALID;
}

void g3l_ctx_destroy(g3l_ctx *c)
{
    if (!c) return;
    srv_destroy(c->srv[0]);
    srv_destroy(c->srv[1]);
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &g : c->graphs) {
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
    }
    Workspace &W = c->W;
    void *ptrs[] = {W.P.center, W.P.level, W.P.val, W.P.err, W.P.split, W.P.cmask, W.P.q, W.P.cand,
                    W.P.unc,    W.P.esc,   W.P.uval, W.P.key, W.P.rscr, W.D, W.S, W.woff, W.H};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (void *p : c->allocs) cudaFree(p);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->cancel_h) cudaFreeHost(c->cancel_h);
    if (c->retab_d) cudaFree(c->retab_d);
    host::free_nbar_device(c->nbw);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (auto &e : c->tev)
        if (e) cudaEventDestroy(e);
    if (c->stage) cudaFreeHost(c->stage);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // extern "C"

namespace {

bool hod_ok(const double *params, std::string &why)
{
    for (int k = 0; k < 6; ++k)
        if (!std::isfinite(params[k])) {
            why = "non-finite HOD parameter";
            return false;
        }
    if (!(params[2] > 0) || !(params[3] != 0) || !(params[4] > 0)) {
        why = "Mth, M' must be > 0 and sigma != 0";
        return false;
    }
    return true;
}

// A slot's HOD vector and its n_bar(z): the FP64 tables and the mixed path's scaled FP32
// n_bar and occupation constants, copied on the context's stream (not synchronised).
int store_hod(g3l_ctx *c, int slot, const double params[6], const double *nb)
{
    const int Nz = c->B.Nz;
    std::copy(params, params + 6, c->hod_h.begin() + 6 * slot);
    std::copy(nb, nb + Nz, c->nbar_h.begin() + (size_t)Nz * slot);
    c->hod_set[slot] = 1;
    G3L_CK(cudaMemcpyAsync(c->d_hod + 6 * slot, c->hod_h.data() + 6 * slot, 6 * sizeof(double),
                           cudaMemcpyHostToDevice, c->stream));
    G3L_CK(cudaMemcpyAsync(c->d_nbar + (size_t)Nz * slot, c->nbar_h.data() + (size_t)Nz * slot,
                           Nz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    // mixed path: n_bar scaled to max 1 and the occupation constants in FP32
    double mx = 0;
    for (int i = 0; i < Nz; ++i) mx = std::max(mx, std::fabs(nb[i]));
    c->sn[slot] = mx > 0 ? 1 / mx : 1;
    float *fnb = c->fnbar_h.data() + (size_t)Nz * slot;
    for (int i = 0; i < Nz; ++i) fnb[i] = (float)(nb[i] * c->sn[slot]);
    const float2 lmth = dsplit(std::log10(params[2])), lmp = dsplit(std::log10(params[4]));
    float *hp = c->fhodp_h.data() + 8 * slot;
    const float h8[8] = {(float)params[0], (float)params[1], lmth.x, lmth.y,
                         (float)(std::log(10.0) / (params[3] * 1.414213562)), lmp.x, lmp.y,
                         (float)params[5]};
    std::copy(h8, h8 + 8, hp);
    G3L_CK(cudaMemcpyAsync(c->d_fnbar + (size_t)Nz * slot, fnb, Nz * sizeof(float),
                           cudaMemcpyHostToDevice, c->stream));
    G3L_CK(cudaMemcpyAsync(c->d_fhodp + 8 * slot, hp, 8 * sizeof(float), cudaMemcpyHostToDevice,
                           c->stream));
    return G3L_OK;
}

// n_bar of n HOD vectors on the device, stored in their slots; one synchronisation
int set_hods_impl(g3l_ctx *c, int n, const int *slots, const double *params, const char *who)
{
    for (int k = 0; k < n; ++k) {
        std::string why;
        if (slots[k] < 0 || slots[k] >= MAX_HOD_SLOTS) {
            host::set_error(std::string(who) + ": slot out of range");
            return G3L_ERR_INVALID;
        }
        if (!hod_ok(params + 6 * k, why)) {
            host::set_error(std::string(who) + ": " + why);
            return G3L_ERR_INVALID;
        }
    }
    G3L_CK(cudaSetDevice(c->device));
    NvtxScope nv("n_bar");
    const int Nz = c->B.Nz;
    std::vector<double> nb((size_t)n * Nz);
    int st = host::n_bar_device(c->nbw, c->B, c->T.hmf, params, n, (void *)c->stream, c->nsm,
                                nb.data());
    if (st) return st;
    // the host copies must not be overwritten while an earlier slot's copy is in flight
    for (int k = 0; k < n; ++k) {
        st = store_hod(c, slots[k], params + 6 * k, nb.data() + (size_t)Nz * k);
        if (st) return st;
    }
    G3L_CK(cudaStreamSynchronize(c->stream));
    return G3L_OK;
}

}  // namespace

extern "C" {

int g3l_set_hod(g3l_ctx *c, int slot, const double params[6])
try {
    if (!c || !params) {
        host::set_error("g3l_set_hod: invalid arguments");
        return G3L_ERR_INVALID;
    }
    return set_hods_impl(c, 1, &slot, params, "g3l_set_hod");
} catch (const std::bad_alloc &) {
    host::set_error("g3l_set_hod: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_set_hod: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_set_hods(g3l_ctx *c, int n, const int *slots, const double *params)
try {
    if (!c || n < 0 || (n > 0 && (!slots || !params))) {
        host::set_error("g3l_set_hods: invalid arguments");
        return G3L_ERR_INVALID;
    }
    if (n == 0) return G3L_OK;
    return set_hods_impl(c, n, slots, params, "g3l_set_hods");
} catch (const std::bad_alloc &) {
    host::set_error("g3l_set_hods: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_set_hods: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_set_correlation(g3l_ctx *c, double A, double eps)
{
    if (!c || !std::isfinite(A) || !std::isfinite(eps)) return G3L_ERR_INVALID;
    c->A = A;
    c->eps = eps;
    c->T.A = A;
    c->T.eps = eps;
    c->T.fA = (float)A;
    c->T.feps = (float)eps;
    for (auto &g : c->graphs) {  // the tables struct is baked into the graph's kernel args
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
    }
    c->graphs.clear();
    return G3L_OK;
}

int g3l_set_scaling(g3l_ctx *c, int slot, const double *scaling)
try {
    if (!c || slot < 0 || slot >= MAX_HOD_SLOTS) {
        host::set_error("g3l_set_scaling: invalid arguments");
        return G3L_ERR_INVALID;
    }
    const int Nm = c->B.Nm;
    std::vector<double> s(Nm, 1.0);
    if (scaling) {
        for (int j = 0; j < Nm; ++j)
            if (!std::isfinite(scaling[j])) {
                host::set_error("g3l_set_scaling: non-finite value");
                return G3L_ERR_INVALID;
            }
        std::copy(scaling, scaling + Nm, s.begin());
    }
    std::vector<float> q(Nm);
    for (int j = 0; j < Nm; ++j) q[j] = (float)(s[j] * s[j] - 1.0);
    G3L_CK(cudaSetDevice(c->device));
    G3L_CK(cudaMemcpyAsync(c->d_scale + (size_t)Nm * slot, s.data(), Nm * sizeof(double),
                           cudaMemcpyHostToDevice, c->stream));
    G3L_CK(cudaMemcpyAsync(c->d_fscale + (size_t)Nm * slot, q.data(), Nm * sizeof(float),
                           cudaMemcpyHostToDevice, c->stream));
    G3L_CK(cudaStreamSynchronize(c->stream));
    return G3L_OK;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_set_scaling: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_set_scaling: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_get_densities(g3l_ctx *c, int slot, double *rho, double *nbar)
{
    if (!c || slot < 0 || slot >= MAX_HOD_SLOTS || !c->hod_set[slot]) return G3L_ERR_INVALID;
    const int Nz = c->B.Nz;
    if (rho) std::copy(c->rho_h.begin(), c->rho_h.end(), rho);
    if (nbar) std::copy(c->nbar_h.begin() + (size_t)Nz * slot, c->nbar_h.begin() + (size_t)Nz * (slot + 1), nbar);
    return G3L_OK;
}

int g3l_get_options(g3l_ctx *c, g3l_options *o)
{
    if (!c || !o) return G3L_ERR_INVALID;
    *o = c->opt;
    return G3L_OK;
}

int g3l_set_options(g3l_ctx *c, const g3l_options *o)
{
    if (!c || !o || o->max_rounds < 1 || o->unlimited_pool < 16 || !(o->small_arg >= 0) ||
        !(o->unc_eps_rel > 0) || !(o->unc_eps_val >= 0) || !(o->unc_eps_sel >= 0) ||
        !(o->deadline_ms >= 0) || !std::isfinite(o->deadline_ms) ||
        !(o->unc_thr >= 0) || !std::isfinite(o->unc_thr) || !(o->unc_tau_thr >= 0) ||
        std::any_of(o->evalmx_variant, o->evalmx_variant + NGROUPS,
                    [](int v) { return v < 0 || v > 2; })) {
        host::set_error("g3l_set_options: invalid option value");
        return G3L_ERR_INVALID;
    }
    c->opt = *o;
    c->T.small_arg = (float)o->small_arg;
    c->T.unc_eps = (float)o->unc_eps_rel;
    c->T.unc_abs = (float)o->unc_tau_abs;
    c->T.tau_impact = o->unc_tau_impact;
    c->T.tau_sel = o->unc_tau_sel;
    c->T.tau_val = o->unc_tau_val;
    c->T.unc_val_ratio = (float)(o->unc_eps_val / o->unc_eps_rel);
    c->T.unc_sel_ratio = (float)(o->unc_eps_sel / o->unc_eps_rel);
    for (auto &g : c->graphs) {
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
    }
    c->graphs.clear();
    return G3L_OK;
}

int g3l_autotune(g3l_ctx *c, const g3l_integral *items, int n, int variant_out[6],
                 double *ms_out)
try {
    if (!c || !items || n < 1 || !variant_out) {
        host::set_error("g3l_autotune: invalid arguments");
        return G3L_ERR_INVALID;
    }
    const g3l_options keep = c->opt;
    double ms[NGROUPS][3] = {};
    uint64_t pts[NGROUPS] = {};
    std::vector<g3l_result> res(n);
    int st = G3L_OK;
    for (int v = 0; v < 3 && !st; ++v) {
        g3l_options o = keep;
        o.use_graph = 0;
        for (int g = 0; g < NGROUPS; ++g) o.evalmx_variant[g] = v;
        st = g3l_set_options(c, &o);
        for (int rep = 0; rep < 2 && !st; ++rep) {  // the first pass warms the kernels
            st = g3l_eval(c, items, n, G3L_MIXED, res.data());
            if (st == G3L_ERR_POOL || st == G3L_ERR_ROUNDS || st == G3L_ERR_NONFINITE) st = G3L_OK;
        }
        for (int g = 0; g < NGROUPS; ++g) {
            ms[g][v] = c->stats.group_ms[g];
            pts[g] = c->stats.group_points[g];
        }
    }
    g3l_options best = keep;
    for (int g = 0; g < NGROUPS; ++g) {
        if (!st && pts[g]) {
            int b = 0;
            for (int v = 1; v < 3; ++v)
                if (ms[g][v] < ms[g][b]) b = v;
            best.evalmx_variant[g] = b;
        }
        variant_out[g] = best.evalmx_variant[g];
        if (ms_out)
            for (int v = 0; v < 3; ++v) ms_out[g * 3 + v] = ms[g][v];
    }
    const int st2 = g3l_set_options(c, &best);
    return st ? st : st2;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_autotune: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_autotune: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_eval_terms(g3l_ctx *c, int kind, const double *triplets, int n, int hod1, int hod2,
                   int term_mask, double rtol, uint64_t max_eval, int precision, double *val,
                   double *err, double *result, uint64_t *neval)
try {
    if (!c || n < 0 || (n > 0 && (!triplets || !val || !err || !result)) || term_mask < 0 ||
        term_mask > 7) {
        host::set_error("g3l_eval_terms: invalid arguments");
        return G3L_ERR_INVALID;
    }
    std::vector<g3l_integral> items;
    std::vector<int> where;
    for (int i = 0; i < n; ++i)
        for (int t = 1; t <= 3; ++t) {
            val[3 * i + t - 1] = err[3 * i + t - 1] = result[3 * i + t - 1] = 0;
            if (!(term_mask >> (t - 1) & 1)) continue;
            g3l_integral it{};
            it.kind = kind;
            it.term = t;
            it.hod1 = hod1;
            it.hod2 = hod2;
            for (int k = 0; k < 3; ++k) it.theta[k] = triplets[3 * i + k];
            it.rtol = rtol;
            it.max_eval = max_eval;
            items.push_back(it);
            where.push_back(3 * i + t - 1);
        }
    if (neval) *neval = 0;
    if (items.empty()) return G3L_OK;
    std::vector<g3l_result> out(items.size());
    const int st = g3l_eval(c, items.data(), (int)items.size(), precision, out.data());
    if (st == G3L_ERR_INVALID || st == G3L_ERR_CUDA || st == G3L_ERR_NOMEM) return st;
    uint64_t ne = 0;
    for (size_t k = 0; k < items.size(); ++k) {
        val[where[k]] = out[k].val;
        err[where[k]] = out[k].err;
        result[where[k]] = out[k].result;
        ne += out[k].neval;
    }
    if (neval) *neval = ne;
    return st;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_eval_terms: host allocation failed");
    return G3L_ERR_NOMEM;
}

int g3l_eval_cancel(g3l_ctx *c)
{
    if (!c) {
        host::set_error("g3l_eval_cancel: invalid context");
        return G3L_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(c->run_mu);
    if (c->running) __atomic_store_n(c->cancel_h, 1, __ATOMIC_SEQ_CST);
    return G3L_OK;
}

int g3l_get_stats(g3l_ctx *c, g3l_stats *s)
{
    if (!c || !s) return G3L_ERR_INVALID;
    *s = c->stats;
    return G3L_OK;
}

int g3l_eval(g3l_ctx *c, const g3l_integral *items, int n, int precision, g3l_result *out)
try {
    if (!c || n < 0 || (n > 0 && (!items || !out)) ||
        (precision != G3L_FP64 && precision != G3L_MIXED)) {
        host::set_error("g3l_eval: invalid arguments");
        return G3L_ERR_INVALID;
    }
    if (n == 0) return G3L_OK;
    if (precision == G3L_MIXED && !evalmx_kernel(0, 1)) {
        host::set_error("g3l_eval: mixed-precision kernels not built");
        return G3L_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) {
        if (!item_ok(c, items[i])) {
            host::set_error("g3l_eval: invalid integral " + std::to_string(i) +
                            " (kind, term, unset HOD slot, theta or rtol)");
            return G3L_ERR_INVALID;
        }
    }
    G3L_CK(cudaSetDevice(c->device));
    NvtxScope nv("g3l_eval");
    RunGuard run(c);
    // order by group
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto grp = [&](int i) { return items[i].kind * 3 + items[i].term - 1; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return grp(a) < grp(b); });
    std::vector<IntDesc> D(n);
    BatchHdr H{};
    H.n = n;
    int gmask = 0;
    long long base = 0;
    for (int r = 0; r < n; ++r) {
        const g3l_integral &it = items[order[r]];
        IntDesc &d = D[r];
        fill_desc(c, it, precision, d);
        unsigned long long cap;
        if (it.max_eval) {
            unsigned long long np = d.npts;
            cap = 3 + (it.max_eval + np) / (2 * np);
        } else {
            cap = c->opt.unlimited_pool;
        }
        if (cap > (1ull << 30)) {
            host::set_error("g3l_eval: max_eval too large for one region pool");
            return G3L_ERR_INVALID;
        }
        d.cap = (int)cap;
        d.base = base;
        base += (long long)cap;
        gmask |= 1 << grp(order[r]);
    }
    for (int g = 0, r = 0; g <= NGROUPS; ++g) {
        while (r < n && grp(order[r]) < g) ++r;
        H.gbeg[g] = r;
    }
    H.gbeg[NGROUPS] = n;
    H.max_rounds = c->opt.max_rounds;
    H.mixed = precision == G3L_MIXED ? 1 : 0;
    int st = ensure_workspace(c, n, (size_t)base);
    if (st) return st;
    Workspace &W = c->W;
    set_esc_queues(D.data(), n, H);
    set_stop_fields(c, H);
    H.dbg = nullptr;
    // stage through pinned host memory: descriptors + header in, states + header out
    const size_t in_bytes = sizeof(IntDesc) * n + sizeof(BatchHdr);
    const size_t out_bytes = sizeof(IntState) * n + sizeof(BatchHdr);
    if (c->stage_bytes < in_bytes + out_bytes) {
        if (c->stage) cudaFreeHost(c->stage);
        c->stage_bytes = (in_bytes + out_bytes) * 5 / 4 + 4096;
        if (cudaMallocHost(&c->stage, c->stage_bytes) != cudaSuccess) {
            c->stage = nullptr;
            c->stage_bytes = 0;
            host::set_error("g3l_eval: pinned staging allocation failed");
            return G3L_ERR_NOMEM;
        }
    }
    char *stg = (char *)c->stage;
    std::memcpy(stg, D.data(), sizeof(IntDesc) * n);
    std::memcpy(stg + sizeof(IntDesc) * n, &H, sizeof(BatchHdr));
    c->last_h2d = in_bytes;
    c->last_d2h = out_bytes;
    G3L_CK(cudaMemcpyAsync(W.D, stg, sizeof(IntDesc) * n, cudaMemcpyHostToDevice, c->stream));
    G3L_CK(cudaMemcpyAsync(W.H, stg + sizeof(IntDesc) * n, sizeof(BatchHdr),
                           cudaMemcpyHostToDevice, c->stream));
    int launches = 0;
    G3L_CK(cudaEventRecord(c->ev0, c->stream));
    if (c->opt.use_graph) {
        GraphEntry *ge = nullptr;
        for (auto &g : c->graphs)
            if (g.gen == W.gen && g.precision == precision && g.gmask == gmask) ge = &g;
        if (!ge) {
            GraphEntry e;
            st = build_graph(c, precision, gmask, e);
            if (st) return st;
            c->graphs.push_back(e);
            ge = &c->graphs.back();
        }
        G3L_CK(cudaGraphLaunch(ge->exec, c->stream));
        launches = -1;  // filled from the round count below
    } else {
        st = run_host_loop(c, precision, gmask, &launches);
        if (st) return st;
    }
    G3L_CK(cudaEventRecord(c->ev1, c->stream));
    char *ostg = stg + in_bytes;
    G3L_CK(cudaMemcpyAsync(ostg, W.S, sizeof(IntState) * n, cudaMemcpyDeviceToHost, c->stream));
    G3L_CK(cudaMemcpyAsync(ostg + sizeof(IntState) * n, W.H, sizeof(BatchHdr),
                           cudaMemcpyDeviceToHost, c->stream));
    G3L_CK(cudaStreamSynchronize(c->stream));
    std::vector<IntState> S(n);
    std::memcpy(S.data(), ostg, sizeof(IntState) * n);
    BatchHdr Hout;
    std::memcpy(&Hout, ostg + sizeof(IntState) * n, sizeof(BatchHdr));
    G3L_CK(cudaGetLastError());
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    int ngroups = __builtin_popcount((unsigned)gmask);
    g3l_stats &sx = c->stats;
    {
        g3l_stats keep = sx;
        sx = g3l_stats{};
        if (!c->opt.use_graph) {
            for (int g = 0; g < NGROUPS; ++g) sx.group_ms[g] = keep.group_ms[g];
            sx.reeval_ms = keep.reeval_ms;
            sx.select_ms = keep.select_ms;
        }
    }
    sx.rounds = (uint64_t)Hout.rounds_done;
    sx.kernel_launches = launches >= 0 ? (uint64_t)launches
                                       : (uint64_t)(1 + (Hout.rounds_done + 1) *
                                                           (2 + ngroups +
                                                            (precision == G3L_MIXED
                                                                 ? 2 * (ngroups + 1) + 1
                                                                 : 0)));
    sx.regions_evaluated = Hout.regions;
    sx.tie_fallbacks = Hout.ties;
    sx.small_arg_fp64 = Hout.small_arg;
    sx.escalated = Hout.escalated;
    sx.h2d_bytes = c->last_h2d;
    sx.d2h_bytes = c->last_d2h;
    sx.deferred = Hout.deferred;
    sx.polished = Hout.polished;
    sx.escalated_full = Hout.esc_full;
    sx.thr_checks = Hout.thr_checks;
    sx.device_ms = ms;
    int first_bad = G3L_OK;
    uint64_t pts = 0;
    for (int r = 0; r < n; ++r) {
        const IntDesc &d = D[r];
        const IntState &s = S[r];
        sx.group_points[d.kind * 3 + d.term - 1] += s.neval;
        g3l_result &o = out[order[r]];
        o.val = s.val * d.scale;
        o.err = s.err * d.scale;
        o.neval = s.neval;
        o.status = s.done ? s.status : G3L_ERR_ROUNDS;
        o.rounds = s.rounds;
        o.result = host::apply_prefactor(d.kind, d.term, c->H0, c->Om, o.val);
        pts += s.neval;
        if (o.status && !first_bad) first_bad = o.status;
    }
    sx.points_evaluated = pts;
    c->last_D = D;
    c->last_nR.resize(n);
    c->last_pos.resize(n);
    for (int r = 0; r < n; ++r) {
        c->last_nR[r] = S[r].nR;
        c->last_pos[order[r]] = r;
    }
    if (first_bad) host::set_error("g3l_eval: an integral ended with status " + std::to_string(first_bad));
    return first_bad;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_eval: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_eval: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_debug_pool(g3l_ctx *c, int index, int max_regions, double *centers, int *levels,
                   double *val, double *err, int *split, float *unc, int *n_regions)
try {
    if (!c || !n_regions || index < 0 || index >= (int)c->last_pos.size() || max_regions < 0) {
        host::set_error("g3l_debug_pool: invalid arguments or no previous g3l_eval");
        return G3L_ERR_INVALID;
    }
    const int r = c->last_pos[index];
    const IntDesc &d = c->last_D[r];
    const int nR = c->last_nR[r];
    *n_regions = nR;
    if (max_regions < nR) return G3L_OK;  // size query
    if (!centers || !levels || !val || !err || !split) {
        host::set_error("g3l_debug_pool: null output array");
        return G3L_ERR_INVALID;
    }
    G3L_CK(cudaSetDevice(c->device));
    G3L_CK(cudaStreamSynchronize(c->stream));
    const Workspace &W = c->W;
    const long long stride = W.P.stride;
    std::vector<unsigned char> b(nR);
    for (int k = 0; k < d.dim; ++k) {
        G3L_CK(cudaMemcpy(centers + (size_t)k * nR, W.P.center + k * stride + d.base,
                          nR * sizeof(double), cudaMemcpyDeviceToHost));
        G3L_CK(cudaMemcpy(b.data(), W.P.level + k * stride + d.base, nR, cudaMemcpyDeviceToHost));
        for (int j = 0; j < nR; ++j) levels[(size_t)k * nR + j] = b[j];
    }
    G3L_CK(cudaMemcpy(val, W.P.val + d.base, nR * sizeof(double), cudaMemcpyDeviceToHost));
    G3L_CK(cudaMemcpy(err, W.P.err + d.base, nR * sizeof(double), cudaMemcpyDeviceToHost));
    G3L_CK(cudaMemcpy(b.data(), W.P.split + d.base, nR, cudaMemcpyDeviceToHost));
    for (int j = 0; j < nR; ++j) {
        split[j] = b[j] & 0x7F;
        val[j] *= d.scale;
        err[j] *= d.scale;
    }
    if (unc) {
        G3L_CK(cudaMemcpy(unc, W.P.unc + d.base, nR * sizeof(float), cudaMemcpyDeviceToHost));
        G3L_CK(cudaMemcpy(unc + nR, W.P.uval + d.base, nR * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return G3L_OK;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_debug_pool: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_debug_pool: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_debug_region(g3l_ctx *c, const g3l_integral *item, const double *center,
                     const int *levels, int precision, double *values, double out[3])
try {
    if (!c || !item || !center || !levels || !values || !out ||
        (precision != G3L_FP64 && precision != G3L_MIXED) || !item_ok(c, *item)) {
        host::set_error("g3l_debug_region: invalid arguments");
        return G3L_ERR_INVALID;
    }
    G3L_CK(cudaSetDevice(c->device));
    IntDesc d;
    fill_desc(c, *item, precision, d);
    for (int k = 0; k < d.dim; ++k)
        if (levels[k] < 0 || levels[k] > 60 || !std::isfinite(center[k])) {
            host::set_error("g3l_debug_region: invalid region");
            return G3L_ERR_INVALID;
        }
    d.base = 0;
    d.cap = 2;
    int st = ensure_workspace(c, 1, 4);
    if (st) return st;
    Workspace &W = c->W;
    const int grp = item->kind * 3 + item->term - 1;
    double *dbg;
    st = dalloc(&dbg, 2 * (size_t)d.npts);
    if (st) return st;
    BatchHdr H{};
    H.n = 1;
    for (int g = 0; g <= NGROUPS; ++g) H.gbeg[g] = g <= grp ? 0 : 1;
    H.max_rounds = 1;
    H.mixed = precision == G3L_MIXED;
    H.esc_cap[grp] = 2;
    H.dbg = dbg;
    IntState S{};
    S.nR = 1;
    S.K = 1;
    long long woff[2] = {0, 1};
    const int cand = -1;
    cudaStream_t s = c->stream;
    int rc = G3L_OK;
    do {
        if (cudaMemcpyAsync(W.D, &d, sizeof d, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(W.H, &H, sizeof H, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(W.S, &S, sizeof S, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(W.woff, woff, sizeof woff, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(W.P.cand, &cand, sizeof cand, cudaMemcpyHostToDevice, s)) {
            rc = G3L_ERR_CUDA;
            break;
        }
        for (int k = 0; k < d.dim; ++k) {
            unsigned char lv = (unsigned char)levels[k];
            if (cudaMemcpyAsync(W.P.center + (size_t)k * W.P.stride, center + k, sizeof(double),
                                cudaMemcpyHostToDevice, s) ||
                cudaMemcpyAsync(W.P.level + (size_t)k * W.P.stride, &lv, 1, cudaMemcpyHostToDevice,
                                s)) {
                rc = G3L_ERR_CUDA;
                break;
            }
        }
        if (rc) break;
        KernelArgs a{c->T, W.D, W.S, W.P, W.H, W.woff, 0, 0, 0.0, 0.0};
        void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
        if (cudaLaunchKernel(eval_fn(c, precision, grp), dim3(1), dim3(128), args, 0, s)) {
            rc = G3L_ERR_CUDA;
            break;
        }
        double vv[2];
        unsigned char sp = 0;
        if (cudaMemcpyAsync(values, dbg, sizeof(double) * d.npts, cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(&vv[0], W.P.val, sizeof(double), cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(&vv[1], W.P.err, sizeof(double), cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(&sp, W.P.split, 1, cudaMemcpyDeviceToHost, s) ||
            cudaStreamSynchronize(s)) {
            rc = G3L_ERR_CUDA;
            break;
        }
        out[0] = vv[0];
        out[1] = vv[1];
        out[2] = sp & 0x7F;
    } while (0);
    if (rc) host::set_error(std::string("g3l_debug_region: ") + cudaGetErrorString(cudaGetLastError()));
    cudaFree(dbg);
    return rc;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_debug_region: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_debug_region: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_measure_peaks(g3l_ctx *c, double *fp32_tflops, double *fp64_tflops)
{
    if (!c || !fp32_tflops || !fp64_tflops) return G3L_ERR_INVALID;
    G3L_CK(cudaSetDevice(c->device));
    extern int g3l_probe_peaks(int, cudaStream_t, double *, double *);
    return g3l_probe_peaks(c->device, c->stream, fp32_tflops, fp64_tflops);
}

int g3l_submit(g3l_ctx *c, const g3l_integral *items, int n, int precision, int64_t *ticket)
try {
    if (!c || !ticket || (precision != G3L_FP64 && precision != G3L_MIXED)) {
        host::set_error("g3l_submit: invalid arguments");
        return G3L_ERR_INVALID;
    }
    int st = G3L_OK;
    g3l_server *v = ctx_server(c, precision, &st);
    if (!v) return st ? st : G3L_ERR_INVALID;
    int64_t t = 0;
    st = srv_submit(v, items, n, &t);
    if (!st) *ticket = 2 * t + (precision == G3L_MIXED ? 1 : 0);
    return st;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_submit: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_submit: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_poll(g3l_ctx *c, int64_t ticket, g3l_result *out, int wait)
try {
    if (!c || ticket < 2) return G3L_ERR_INVALID;
    g3l_server *v = c->srv[ticket & 1];
    if (!v) return G3L_ERR_INVALID;
    return srv_poll(v, ticket >> 1, out, wait ? -1 : 0, nullptr);
} catch (const std::bad_alloc &) {
    host::set_error("g3l_poll: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_poll: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_cancel(g3l_ctx *c, int64_t ticket)
{
    if (!c || ticket < 2) return G3L_ERR_INVALID;
    g3l_server *v = c->srv[ticket & 1];
    if (!v) return G3L_ERR_INVALID;
    return srv_cancel(v, ticket >> 1);
}

int g3l_server_create(g3l_ctx *ctx, int precision, int max_items_per_term, uint64_t pool_regions,
                      int rounds_per_launch, g3l_server **out)
try {
    return srv_create(ctx, precision, max_items_per_term, pool_regions, rounds_per_launch, out);
} catch (const std::bad_alloc &) {
    host::set_error("g3l_server_create: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_server_create: ") + e.what());
    return G3L_ERR_INVALID;
}

void g3l_server_destroy(g3l_server *srv) { srv_destroy(srv); }

int g3l_server_submit(g3l_server *srv, const g3l_integral *items, int n, int64_t *ticket)
try {
    return srv_submit(srv, items, n, ticket);
} catch (const std::bad_alloc &) {
    host::set_error("g3l_server_submit: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_server_submit: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_server_poll(g3l_server *srv, int64_t ticket, g3l_result *out, int wait_ms,
                    double *latency_ms)
try {
    return srv_poll(srv, ticket, out, wait_ms, latency_ms);
} catch (const std::bad_alloc &) {
    host::set_error("g3l_server_poll: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_server_poll: ") + e.what());
    return G3L_ERR_INVALID;
}

int g3l_server_cancel(g3l_server *srv, int64_t ticket) { return srv_cancel(srv, ticket); }

int g3l_server_info(g3l_server *srv, g3l_server_stats *st)
{
    if (!srv || !st) return G3L_ERR_INVALID;
    std::lock_guard<std::mutex> lk(srv->mu);
    *st = g3l_server_stats{};
    st->launches = srv->launches;
    st->admitted = srv->admitted_total;
    st->completed = srv->completed_total;
    st->queued = (int)srv->pending.size();
    st->running_integrals = srv->active;
    st->free_regions = (uint64_t)srv->ra.total_free;
    return G3L_OK;
}

}  // extern "C"

// ------------------------------------------------------------- fixed-scratch entry point
//
// g3l_eval_static runs the same device engine as g3l_eval, but every per-call device
// buffer (batch header, descriptors, states, work offsets and the region pools) is
// carved out of one file-scope __device__ array instead of the context's workspace,
// and the refinement rounds are driven from the host with plain kernel launches.  The
// call therefore allocates no device memory, no pinned host memory and no graph: it is
// for callers that must not allocate at evaluation time (a process whose device memory
// is owned by another allocator, or a latency-critical loop that cannot afford an
// allocation's implicit synchronisation).
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kStaticMaxItems = 1024;
constexpr int kStaticMaxDevices = 64;
constexpr int kStaticReevalCap = 512;  // re-evaluation entries per group and round (device-wide passes)

static __device__ __align__(256) unsigned char g3l_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void *g_static_base[kStaticMaxDevices];  // device address of the scratch, per device

// Host staging of one call, one set per device beside that device's scratch (static
// storage: the entry point allocates nothing).  The per-device lock serialises calls on
// one device, which share both; calls on different devices proceed side by side.
struct StaticStage {
    std::mutex mu;
    IntDesc desc[kStaticMaxItems];
    IntState state[kStaticMaxItems];
    int order[kStaticMaxItems];
};
StaticStage g_st[kStaticMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of scratch a call with n integrals and `pool` region slots needs, and the
// offsets of its arrays (same arrays as the context workspace).
struct StaticLayout {
    size_t H, D, S, woff, center, level, val, err, split, cmask, q, cand, unc, uval, key, esc, rscr, end;
};

StaticLayout static_layout(int n, size_t pool)
{
    StaticLayout L{};
    size_t o = 0;
    L.H = o;      o = align256(o + sizeof(BatchHdr));
    L.D = o;      o = align256(o + sizeof(IntDesc) * (size_t)n);
    L.S = o;      o = align256(o + sizeof(IntState) * (size_t)n);
    L.woff = o;   o = align256(o + sizeof(long long) * ((size_t)n + 1));
    L.center = o; o = align256(o + sizeof(double) * pool * MAX_DIM);
    L.level = o;  o = align256(o + pool * MAX_DIM);
    L.val = o;    o = align256(o + sizeof(double) * pool);
    L.err = o;    o = align256(o + sizeof(double) * pool);
    L.split = o;  o = align256(o + pool);
    L.cmask = o;  o = align256(o + pool);
    L.q = o;      o = align256(o + sizeof(unsigned long long) * pool);
    L.cand = o;   o = align256(o + sizeof(int) * pool);
    L.unc = o;    o = align256(o + sizeof(float) * pool);
    L.uval = o;   o = align256(o + sizeof(float) * pool);
    L.key = o;    o = align256(o + sizeof(double) * pool);
    L.esc = o;    o = align256(o + sizeof(int2) * pool);
    L.rscr = o;   o = align256(o + (size_t)(NGROUPS * reeval_scratch_group_bytes(kStaticReevalCap)));
    L.end = o;
    return L;
}

// Resolve the scratch address on the current device (once per device).
int static_scratch(int device, unsigned char **base)
{
    if (device < 0 || device >= kStaticMaxDevices) {
        host::set_error("g3l_eval_static: device ordinal beyond the supported range");
        return G3L_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_base[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g3l_static_scratch);
        if (e != cudaSuccess || !p) {
            host::set_error(std::string("g3l_eval_static: cudaGetSymbolAddress failed: ") +
                            cudaGetErrorString(e));
            return G3L_ERR_CUDA;
        }
        g_static_base[device] = p;
    }
    *base = (unsigned char *)g_static_base[device];
    return G3L_OK;
}

// One call on the device of `c`, with that device's staging `G` held by the caller.
int eval_static_locked(g3l_ctx *c, const g3l_integral *items, int n, int precision,
                       g3l_result *out, StaticStage &G, unsigned char *base)
{
    // descriptors in group order (stable counting sort, no temporary buffer), pool
    // capacities as g3l_eval
    auto grp = [&](int i) { return items[i].kind * 3 + items[i].term - 1; };
    {
        int cnt[NGROUPS + 1] = {};
        for (int i = 0; i < n; ++i) ++cnt[grp(i) + 1];
        for (int g = 0; g < NGROUPS; ++g) cnt[g + 1] += cnt[g];
        for (int i = 0; i < n; ++i) G.order[cnt[grp(i)]++] = i;
    }
    BatchHdr H{};  // zero: every counter of the header starts at zero
    H.n = n;
    int gmask = 0;
    size_t pool = 0;
    for (int r = 0; r < n; ++r) {
        const g3l_integral &it = items[G.order[r]];
        IntDesc &d = G.desc[r];
        fill_desc(c, it, precision, d);
        unsigned long long cap;
        if (it.max_eval) {
            unsigned long long np = d.npts;
            cap = 3 + (it.max_eval + np) / (2 * np);
        } else {
            cap = c->opt.unlimited_pool;
        }
        if (cap > (1ull << 30)) {
            host::set_error("g3l_eval_static: max_eval too large for one region pool");
            return G3L_ERR_INVALID;
        }
        d.cap = (int)cap;
        d.base = (long long)pool;
        pool += cap;
        gmask |= 1 << grp(G.order[r]);
    }
    const StaticLayout L = static_layout(n, pool);
    if (L.end > kStaticScratchBytes) {
        host::set_error("g3l_eval_static: the batch needs " + std::to_string(L.end) +
                        " bytes of scratch (" + std::to_string(pool) +
                        " region slots); the fixed scratch holds " +
                        std::to_string(kStaticScratchBytes) + " bytes -- lower max_eval or split "
                        "the batch");
        return G3L_ERR_INVALID;
    }
    for (int g = 0, r = 0; g <= NGROUPS; ++g) {
        while (r < n && grp(G.order[r]) < g) ++r;
        H.gbeg[g] = r;
    }
    H.gbeg[NGROUPS] = n;
    H.max_rounds = c->opt.max_rounds;
    H.mixed = precision == G3L_MIXED ? 1 : 0;
    set_esc_queues(G.desc, n, H);
    set_stop_fields(c, H);
    H.dbg = nullptr;

    KernelArgs a{};
    a.T = c->T;
    a.H = (BatchHdr *)(base + L.H);
    a.D = (IntDesc *)(base + L.D);
    a.S = (IntState *)(base + L.S);
    a.woff = (long long *)(base + L.woff);
    a.P.center = (double *)(base + L.center);
    a.P.level = base + L.level;
    a.P.val = (double *)(base + L.val);
    a.P.err = (double *)(base + L.err);
    a.P.split = base + L.split;
    a.P.cmask = base + L.cmask;
    a.P.q = (unsigned long long *)(base + L.q);
    a.P.cand = (int *)(base + L.cand);
    a.P.unc = (float *)(base + L.unc);
    a.P.uval = (float *)(base + L.uval);
    a.P.key = (double *)(base + L.key);
    a.P.esc = (int2 *)(base + L.esc);
    a.P.rscr = base + L.rscr;
    a.P.retab = c->retab_d;
    a.P.rcap = kStaticReevalCap;
    a.P.rscr_group = reeval_scratch_group_bytes(kStaticReevalCap);
    a.P.stride = (long long)pool;
    a.handle = 0;
    a.use_cond = 0;
    a.tau_sel = c->T.tau_sel;
    a.tau_val = c->T.tau_val;
    cudaStream_t s = c->stream;
    // The uploaded header and the init kernel's states are all that must start at a
    // known value; the pools are written before they are read.
    G3L_CK(cudaMemcpyAsync(a.D, G.desc, sizeof(IntDesc) * n, cudaMemcpyHostToDevice, s));
    G3L_CK(cudaMemcpyAsync(a.H, &H, sizeof(BatchHdr), cudaMemcpyHostToDevice, s));
    int launches = 0, st = G3L_OK;
    {
        void *args[] = {&a.D, &a.S, &a.P, &a.H};
        G3L_CK(cudaLaunchKernel(init_kernel(), dim3(c->nsm * 4), dim3(256), args, 0, s));
        ++launches;
    }
    int active = 1;
    auto reevals = [&]() -> int {
        for (int g = 0; g < NGROUPS; ++g) {
            if (!(gmask & (1 << g))) continue;
            void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
            for (int ph = 0; ph < 5; ++ph) {
                void *fn = reeval_phase_kernel(g / 3, g % 3 + 1, ph);
                const int grid = ph == 3 ? c->nsm : (ph == 4 ? reeval_grid(c, fn) : grid128(c, fn));
                G3L_CK(cudaLaunchKernel(fn, dim3(grid), dim3(128), args, 0, s));
                ++launches;
            }
        }
        void *eargs[] = {&a.H, &a.all_groups};
        G3L_CK(cudaLaunchKernel(round_end_kernel(), dim3(1), dim3(1), eargs, 0, s));
        ++launches;
        return G3L_OK;
    };
    for (int r = 0; r < c->opt.max_rounds + 4 && active; ++r) {
        void *sargs[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass0};
        G3L_CK(cudaLaunchKernel(select_kernel(), dim3(c->nsm * 8), dim3(256), sargs, 0, s));
        ++launches;
        if (precision == G3L_MIXED) {
            if ((st = reevals())) return st;
            void *sargs1[] = {&a.D, &a.S, &a.P, &a.H, &a.tau_sel, &a.tau_val, &a.pass1};
            G3L_CK(cudaLaunchKernel(select_kernel(), dim3(c->nsm * 8), dim3(256), sargs1, 0, s));
            ++launches;
        }
        void *cargs[] = {&a.S, &a.woff, &a.H, &a.handle, &a.use_cond};
        G3L_CK(cudaLaunchKernel(scan_kernel(), dim3(1), dim3(1024), cargs, 0, s));
        ++launches;
        if (precision == G3L_MIXED)
            if ((st = reevals())) return st;
        for (int g = 0; g < NGROUPS; ++g) {
            if (!(gmask & (1 << g))) continue;
            void *fn = eval_fn(c, precision, g);
            void *args[] = {&a.T, &a.D, &a.S, &a.P, &a.H, &a.woff};
            G3L_CK(cudaLaunchKernel(fn, dim3(eval_grid(c, fn)), dim3(128), args, 0, s));
            ++launches;
        }
        G3L_CK(cudaMemcpyAsync(&active, &a.H->any_active, sizeof(int), cudaMemcpyDeviceToHost, s));
        G3L_CK(cudaStreamSynchronize(s));
    }
    BatchHdr Hout;
    G3L_CK(cudaMemcpyAsync(G.state, a.S, sizeof(IntState) * n, cudaMemcpyDeviceToHost, s));
    G3L_CK(cudaMemcpyAsync(&Hout, a.H, sizeof(BatchHdr), cudaMemcpyDeviceToHost, s));
    G3L_CK(cudaStreamSynchronize(s));
    G3L_CK(cudaGetLastError());
    // statistics as g3l_eval reports them for host-driven rounds (without the per-kernel
    // timings, which would need events)
    g3l_stats sx{};
    int first_bad = G3L_OK;
    uint64_t pts = 0;
    for (int r = 0; r < n; ++r) {
        const IntDesc &d = G.desc[r];
        const IntState &sr = G.state[r];
        sx.group_points[d.kind * 3 + d.term - 1] += sr.neval;
        g3l_result &o = out[G.order[r]];
        o.val = sr.val * d.scale;
        o.err = sr.err * d.scale;
        o.neval = sr.neval;
        o.status = sr.done ? sr.status : G3L_ERR_ROUNDS;
        o.rounds = sr.rounds;
        o.result = host::apply_prefactor(d.kind, d.term, c->H0, c->Om, o.val);
        pts += sr.neval;
        if (o.status && !first_bad) first_bad = o.status;
    }
    sx.kernel_launches = (uint64_t)launches;
    sx.rounds = (uint64_t)Hout.rounds_done;
    sx.regions_evaluated = Hout.regions;
    sx.points_evaluated = pts;
    sx.tie_fallbacks = Hout.ties;
    sx.small_arg_fp64 = Hout.small_arg;
    sx.escalated = Hout.escalated;
    sx.escalated_full = Hout.esc_full;
    sx.thr_checks = Hout.thr_checks;
    sx.deferred = Hout.deferred;
    sx.polished = Hout.polished;
    sx.h2d_bytes = sizeof(IntDesc) * n + sizeof(BatchHdr);
    sx.d2h_bytes = sizeof(IntState) * n + sizeof(BatchHdr) + sizeof(int) * Hout.rounds_done;
    c->stats = sx;
    if (first_bad)
        host::set_error("g3l_eval_static: an integral ended with status " + std::to_string(first_bad));
    return first_bad;
}

}  // namespace

extern "C" int g3l_eval_static(g3l_ctx *c, const g3l_integral *items, int n, int precision,
                               g3l_result *out)
try {
    if (!c || n < 0 || (n > 0 && (!items || !out)) ||
        (precision != G3L_FP64 && precision != G3L_MIXED)) {
        host::set_error("g3l_eval_static: invalid arguments");
        return G3L_ERR_INVALID;
    }
    if (n == 0) return G3L_OK;
    if (precision == G3L_MIXED && !evalmx_kernel(0, 1)) {
        host::set_error("g3l_eval_static: mixed-precision kernels not built");
        return G3L_ERR_INVALID;
    }
    if (n > kStaticMaxItems) {
        host::set_error("g3l_eval_static: " + std::to_string(n) + " integrals exceed the limit of " +
                        std::to_string(kStaticMaxItems) + " per call");
        return G3L_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i)
        if (!item_ok(c, items[i])) {
            host::set_error("g3l_eval_static: invalid integral " + std::to_string(i));
            return G3L_ERR_INVALID;
        }
    G3L_CK(cudaSetDevice(c->device));
    unsigned char *base = nullptr;
    int st = static_scratch(c->device, &base);
    if (st) return st;
    StaticStage &G = g_st[c->device];
    std::lock_guard<std::mutex> lk(G.mu);
    NvtxScope nv("g3l_eval_static");
    RunGuard run(c);
    st = eval_static_locked(c, items, n, precision, out, G, base);
    // A call that failed part-way may have kernels still queued: let them finish before
    // the next call on this device reuses the scratch.
    if (st) cudaStreamSynchronize(c->stream);
    return st;
} catch (const std::bad_alloc &) {
    host::set_error("g3l_eval_static: host allocation failed");
    return G3L_ERR_NOMEM;
} catch (const std::exception &e) {
    host::set_error(std::string("g3l_eval_static: ") + e.what());
    return G3L_ERR_INVALID;
}
