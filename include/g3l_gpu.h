/*
 * g3l_gpu.h -- C ABI of libg3lgpu.so, the GB300 (sm_103a) engine for the
 * halo-model aperture statistics <N N M_ap> (NNMap) and <N M_ap M_ap> (NMapMap).
 *
 * The reference computes each term by calling the host cubature hcubature_v
 * (src/hcubature.cpp:1059-1067) with a vectorised integrand callback that
 * copies the points to the GPU every refinement round
 * (src/NNMap_Model.cu:418-542).  This library keeps the whole adaptive
 * Genz-Malik cubature on the device: region pools, rule evaluation,
 * bisection, error bookkeeping and the refinement loop (a CUDA-graph
 * conditional WHILE node) never return to the host until every integral of a
 * call is finished.
 *
 * Conventions
 *  - Plain C types only; all pointers are host pointers unless stated.
 *  - Every entry point returns an int status (G3L_OK = 0); the library never
 *    calls exit() (the reference does, src/cuda_helpers.h:11-19).
 *    g3l_last_error() returns a thread-local message for the last failure.
 *  - Thread safety: one context may be used by one host thread at a time;
 *    distinct contexts are independent.
 */
#ifndef G3L_GPU_H
#define G3L_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G3L_ABI_VERSION 2  /* 2: g3l_options.deadline_ms, g3l_eval_cancel, G3L_ERR_DEADLINE */

enum g3l_status {
    G3L_OK = 0,
    G3L_ERR_INVALID = 1,    /* bad argument */
    G3L_ERR_CUDA = 2,       /* CUDA runtime error (see g3l_last_error) */
    G3L_ERR_NOMEM = 3,      /* device or host allocation failed */
    G3L_ERR_POOL = 4,       /* region pool exhausted (maxEval == 0 beyond the pool cap) */
    G3L_ERR_NONFINITE = 5,  /* an integral's running value or error became NaN/Inf */
    G3L_ERR_CANCELLED = 6,  /* cancelled (g3l_eval_cancel, g3l_cancel, g3l_server_cancel) */
    G3L_ERR_ROUNDS = 7,     /* refinement-round cap reached */
    G3L_ERR_NO_DEVICE = 8,  /* no usable CUDA device */
    G3L_ERR_BUSY = 9,       /* serving queue full */
    G3L_ERR_DEADLINE = 10   /* the call's deadline (g3l_options.deadline_ms) passed */
};

enum g3l_kind { G3L_NNMAP = 0, G3L_NMAPMAP = 1 };

enum g3l_precision {
    G3L_FP64 = 0,  /* all-FP64 integrand, same operation order as the reference */
    G3L_MIXED = 1  /* FP32 integrand, FP64-class accumulation and decisions */
};

/* Lookup tables and binning (src/NNMap_Model.h:36-58).  The reference uses one
 * Nbins for z, m and k; Nz, Nm and Nk may differ here.  Grids:
 *   z_i = zmin + i (zmax-zmin)/Nz,   m_j = mmin (mmax/mmin)^(j/Nm),
 *   k_j = kmin (kmax/kmin)^(j/Nk).
 * 2-D tables are z-major: hmf[i*Nm + j], P_lin[i*Nk + j].  The arrays are
 * copied at creation; the caller keeps ownership. */
typedef struct g3l_tables {
    int Nz, Nm, Nk;
    double zmin, zmax, mmin, mmax, kmin, kmax;
    const double *g, *p_lens1, *p_lens2, *w, *dwdz; /* [Nz] */
    const double *hmf, *b_h, *conc;                 /* [Nz*Nm] */
    const double *P_lin;                            /* [Nz*Nk] */
    double Om, OL, Ob, sigma8, H0, ns;              /* flat LCDM (src/Cosmology.h:18-24) */
    int clamp_k; /* nonzero: clamp the P_lin k index at Nk-1.  The reference reads
                    past the row instead (src/NNMap_Model.cu:826-839). */
} g3l_tables;

/* One integral: a term of NNMap or NMapMap for one aperture triplet. */
typedef struct g3l_integral {
    int kind;          /* G3L_NNMAP or G3L_NMAPMAP */
    int term;          /* 1, 2 or 3 (1-, 2-, 3-halo: 5, 6, 7 dimensions) */
    int hod1, hod2;    /* HOD slots of the two lens populations (NMapMap: hod1 only).
                          hod1 == hod2 selects the same-population satellite-pair
                          branch, as the reference's pointer test does (src/HOD.cu:82). */
    double theta[3];   /* aperture radii [rad] */
    double rtol;       /* relative tolerance */
    uint64_t max_eval; /* evaluation cap; 0 = unlimited (bounded by the pool cap) */
} g3l_integral;

typedef struct g3l_result {
    double val, err;   /* raw integral and error estimate (before the prefactor) */
    double result;     /* val times the reference's prefactor chain */
    uint64_t neval;    /* integrand evaluations */
    int32_t status;    /* g3l_status of this integral */
    int32_t rounds;    /* refinement rounds */
} g3l_result;

typedef struct g3l_ctx g3l_ctx;

/* Create a context on `device`: copies the tables to device memory and sets up
 * one stream.  Replaces the table uploads in the NNMap_Model / NMapMap_Model
 * constructors (src/NNMap_Model.cu:15-101, src/NMapMap_Model.cu:14-91). */
int g3l_ctx_create(const g3l_tables *tables, int device, g3l_ctx **out);
void g3l_ctx_destroy(g3l_ctx *ctx);

/* Set HOD slot `slot` (0 <= slot < g3l_max_hod_slots()) to
 * params = {f, alpha, Mth, sigma, M', beta} (the reference's device order,
 * src/HOD.cu:15-20) and compute n_bar(z) for it with the 1-D adaptive Gauss-Kronrod
 * integral of the reference (updateDensities, src/NNMap_Model.cu:244-297), on the
 * device: one integral per z bin, the reference's refinement, FP64. */
int g3l_set_hod(g3l_ctx *ctx, int slot, const double params[6]);
/* g3l_set_hod for n slots at once (slots[n], params[n][6]): the n_bar integrals of all
 * of them run in one device launch (the reference updates one model's HODs at a time,
 * src/NNMap_Model.cu:236-297). */
int g3l_set_hods(g3l_ctx *ctx, int n, const int *slots, const double *params);
int g3l_max_hod_slots(void);
/* Satellite-pair correlation parameters A, epsilon (src/HOD.cu:90). */
int g3l_set_correlation(g3l_ctx *ctx, double A, double epsilon);
/* Satellite-variance rescaling of HOD slot `slot` (the reference's SCALING build:
 * src/NNMap_Model.cu:103-200, src/NNMap_Model.h:59-62): scaling[j], j < Nm, at the
 * mass grid m_j.  In the same-population branch of NNMap 1h and 2h the satellite-
 * pair count becomes (N_s + s^2 - 1) N_s with s = scaling[round mass index] of the
 * item's hod1 slot (src/HOD.cu:78-87, src/NNMap_Model.cu:563,808).  NULL resets the
 * slot to s = 1 (no rescaling, the default).  Finite values only.  Like a HOD slot,
 * it must not change while a queued or running request uses the slot. */
int g3l_set_scaling(g3l_ctx *ctx, int slot, const double *scaling);
/* n_bar(z) of a slot and rho_bar(z) as computed by g3l_set_hod ([Nz] each). */
int g3l_get_densities(g3l_ctx *ctx, int slot, double *rho_bar, double *n_bar);

/* Integrate n items in one device-resident launch (all items refine
 * concurrently; the host waits once at the end).  Replaces the per-term
 * methods NNMap_1h/2h/3h and NMapMap_1h/2h/3h (src/NNMap_Model.cu:299-373,
 * src/NMapMap_Model.cu:169-238) and the batch loop calculateAll
 * (src/NNMap_Model.cu:382-415).  Returns the first non-OK item status, or OK. */
int g3l_eval(g3l_ctx *ctx, const g3l_integral *items, int n, int precision,
             g3l_result *out);
/* Stop the g3l_eval (or g3l_eval_terms, g3l_eval_static) call that is running on the
 * context, from any other thread.  The device loop reads the request once per
 * refinement round: every unfinished integral ends at the next round's selection with
 * status G3L_ERR_CANCELLED and the value and error of its regions so far; integrals that
 * had already finished keep their results and G3L_OK.  The call returns
 * G3L_ERR_CANCELLED, and the context stays usable.  With no call running this does
 * nothing (a call starts uncancelled).  The reference has no counterpart: its term
 * methods run to completion or exit (src/cuda_helpers.h:11-19). */
int g3l_eval_cancel(g3l_ctx *ctx);

/* g3l_eval in the per-term methods' shape: the terms in term_mask (bit t-1 = term t) of
 * one kind for n aperture triplets (triplets[3*i + k], radians) and one HOD slot pair,
 * all in one launch.  val, err and result: [n*3], entry 3*i + t-1, before and after the
 * prefactor (terms outside the mask are set to 0); neval: the evaluations of all of
 * them (may be NULL).  Returns the first non-OK status, like g3l_eval. */
int g3l_eval_terms(g3l_ctx *ctx, int kind, const double *triplets, int n, int hod1, int hod2,
                   int term_mask, double rtol, uint64_t max_eval, int precision, double *val,
                   double *err, double *result, uint64_t *neval);

/* Serving with continuous batching.  A server owns a table of integral slots
 * (max_items_per_term for each kind x term) and a pool of pool_regions region slots
 * on the device, and a driver thread that runs the device loop of g3l_eval in
 * launches of rounds_per_launch refinement rounds.  Between launches it completes
 * the integrals that finished, frees their slots and pool ranges, and admits waiting
 * requests first come, first served, as slots and pool space allow (an integral with
 * max_eval M and a P-point rule takes 3 + (M + P) / (2P) pool slots).  Requests that
 * arrive while others run are therefore integrated concurrently with them, and every
 * integral's result is the same as from g3l_eval alone (its trajectory depends only
 * on its own regions).  The server reads the context's tables, HOD slots and options
 * as they are at creation; a HOD slot used by a queued or running request must not
 * be changed until that request completes.  Submit, poll and cancel may be called
 * from any thread.  The reference evaluates one term per blocking call
 * (src/NNMap_Model.cu:299-373); this replaces its calculateAll loop for callers that
 * issue many model evaluations (src/NNMap_Model.cu:382-415). */
typedef struct g3l_server g3l_server;
typedef struct g3l_server_stats {
    uint64_t launches;        /* device-loop launches so far */
    uint64_t admitted;        /* requests admitted */
    uint64_t completed;       /* requests whose integrals all finished */
    int32_t queued;           /* requests waiting for slots or pool space */
    int32_t running_integrals;/* integrals on the device now */
    uint64_t free_regions;    /* unallocated pool slots */
} g3l_server_stats;
int g3l_server_create(g3l_ctx *ctx, int precision, int max_items_per_term, uint64_t pool_regions,
                      int rounds_per_launch, g3l_server **out);
void g3l_server_destroy(g3l_server *srv); /* waits for the running launch, drops the rest */
/* Queue n integrals as one request.  Fails (G3L_ERR_INVALID) if the request could
 * never fit the server's slots or pool. */
int g3l_server_submit(g3l_server *srv, const g3l_integral *items, int n, int64_t *ticket);
/* G3L_ERR_BUSY while the request runs (after waiting up to wait_ms; -1 = until done,
 * 0 = do not wait).  Once done: copies the n results to out, releases the ticket and
 * returns the first non-OK integral status, or OK; latency_ms (optional) receives the
 * time from submit to completion. */
int g3l_server_poll(g3l_server *srv, int64_t ticket, g3l_result *out, int wait_ms,
                    double *latency_ms);
/* A queued request finishes at once; a running one at the next launch boundary.  Its
 * integrals report G3L_ERR_CANCELLED unless they had already finished.  A request that
 * has finished but not been polled is left as it is (G3L_OK); a ticket that is unknown
 * or already polled is G3L_ERR_INVALID. */
int g3l_server_cancel(g3l_server *srv, int64_t ticket);
int g3l_server_info(g3l_server *srv, g3l_server_stats *st);

/* The same on a context: g3l_submit starts (on first use) one server per precision
 * with 1024 slots per kind x term, 4M pool slots and 4 rounds per launch.  g3l_poll
 * with wait != 0 blocks until the request is done; otherwise it returns G3L_ERR_BUSY
 * while it runs.  g3l_ctx_destroy stops these servers. */
int g3l_submit(g3l_ctx *ctx, const g3l_integral *items, int n, int precision,
               int64_t *ticket);
int g3l_poll(g3l_ctx *ctx, int64_t ticket, g3l_result *out, int wait);
int g3l_cancel(g3l_ctx *ctx, int64_t ticket);

/* Engine options. */
typedef struct g3l_options {
    int eval_blocks_per_sm;  /* 0 = automatic */
    int eval_warps_per_block;/* 0 = automatic */
    int use_graph;           /* 1 (default): device-resident loop in a CUDA graph;
                                0: host-driven rounds (diagnostics only) */
    int max_rounds;          /* refinement-round cap (default 4096) */
    uint64_t unlimited_pool; /* region-pool capacity per integral when max_eval == 0 */
    double small_arg;        /* mixed precision: NFW profile arguments k r_s below this
                                are evaluated in FP64 (default 1e-7) */
    /* Mixed precision: every FP32 point value v carries the error bound
     * unc_eps_rel |v| + unc_tau_abs (defaults 5e-5, 1e-34).  A region whose split
     * decision is not settled under these bounds, or that sits on an unsettled
     * selection boundary, is re-evaluated in FP64 when its error exceeds
     * unc_tau_impact (split, default 0: always) or unc_tau_sel (selection, default
     * 1e-7) times the integral's running value. */
    double unc_eps_rel, unc_tau_abs, unc_tau_impact, unc_tau_sel;
    /* A finished integral whose regions' value bounds sum to more than
     * unc_tau_val |value| has its largest-bound regions re-evaluated in FP64, at
     * most twice (default 5e-5; 0 = off). */
    double unc_tau_val;
    /* Relative bound on the FP32 error of one point value used for the value-noise
     * estimate of unc_tau_val (decisions use unc_eps_rel; default 5e-6). */
    double unc_eps_val;
    /* Relative bound on the FP32 error of one point value used for the bound on a
     * region's error estimate, which decides whether a selection boundary is settled
     * (split decisions use unc_eps_rel). */
    double unc_eps_sel;
    /* Register budget of the mixed-precision rule kernel per kind x term
     * (kind * 3 + term - 1): 0, 1, 2 = 7, 6, 8 blocks per SM (72, 80, 64 registers
     * per thread).  Set by g3l_autotune; default 2 for the 1-halo terms, 1 for the 2- and
     * 3-halo terms. */
    int evalmx_variant[6];
    /* Deadline of a g3l_eval / g3l_eval_terms / g3l_eval_static call in milliseconds,
     * measured on the device from the start of its refinement loop (0 = none, the
     * default).  When it passes, every unfinished integral ends at the next round's
     * selection with status G3L_ERR_DEADLINE and its value so far, as with
     * g3l_eval_cancel. */
    double deadline_ms;
    /* Mixed precision: the threshold decisions of the refinement loop -- the
     * convergence test err <= rtol |val| and the number of regions the Gladwell rule
     * pops -- compare sums over many regions of FP32-derived values.  When one is closer
     * to its threshold than unc_thr times the sum of the regions' bounds (the bounds of
     * the selection, unc_eps_sel, and of the values, unc_eps_val), the regions carrying
     * that uncertainty are re-evaluated in FP64 before deciding (default 0.1: the errors
     * of many regions do not all add up; 0 = off).  The count is checked only where it
     * moves a region whose error exceeds unc_tau_thr |val| (default 1e-6). */
    double unc_thr, unc_tau_thr;
} g3l_options;
int g3l_get_options(g3l_ctx *ctx, g3l_options *opt);
int g3l_set_options(g3l_ctx *ctx, const g3l_options *opt);

/* Autotuner: runs the batch once per register-budget variant of the mixed-precision
 * rule kernels (after one warm-up pass each; host-driven rounds with CUDA events around
 * every launch), and keeps for each kind x term present the variant with the least
 * rule-kernel time in the context's options (evalmx_variant).  variant_out[6] receives
 * the choice; ms_out (optional, [6][3]) the rule-kernel milliseconds per group and
 * variant.  The number of regions refined per round is not tuned: it is fixed by the
 * reference's algorithm (src/hcubature.cpp:904-1021), which the results must follow. */
int g3l_autotune(g3l_ctx *ctx, const g3l_integral *items, int n, int variant_out[6],
                 double *ms_out);

/* Per-call diagnostics of the last g3l_eval: kernel launches, rounds, regions,
 * device time, and counters of the exact-index fallbacks. */
typedef struct g3l_stats {
    uint64_t kernel_launches;
    uint64_t rounds;
    uint64_t regions_evaluated;
    uint64_t points_evaluated;
    uint64_t tie_fallbacks;   /* nearest-bin indices resolved by the exact FP64 path */
    uint64_t small_arg_fp64;  /* NFW profile evaluations on the small-k r_s FP64 branch */
    double device_ms;         /* device time of the whole call (CUDA events) */
    double eval_ms;           /* of which in the rule-evaluation kernels */
    uint64_t escalated;       /* mixed precision: regions re-evaluated in FP64 */
    uint64_t deferred;        /* mixed precision: selections deferred for re-evaluation */
    uint64_t polished;        /* mixed precision: finished integrals polished in FP64 */
    /* host-driven rounds only (use_graph = 0): device time and points of the
     * rule-evaluation kernel of each group (kind * 3 + term - 1), CUDA events */
    double group_ms[6];
    uint64_t group_points[6];
    double reeval_ms;         /* FP64 re-evaluation kernels */
    double select_ms;         /* selection + scan kernels */
    uint64_t h2d_bytes, d2h_bytes; /* bytes copied in / out by the call */
    uint64_t escalated_full;  /* of escalated: whole-rule re-evaluations (selection, polish) */
    uint64_t thr_checks;      /* mixed precision: threshold decisions re-taken after FP64
                                 re-evaluation (unc_thr) */
} g3l_stats;
int g3l_get_stats(g3l_ctx *ctx, g3l_stats *st);

/* Evaluate the Genz-Malik rule of one region of one integral on the device and
 * return its integrand values at the rule points, in the reference's point order
 * (src/hcubature.cpp:476-503), plus {val, err, split}.  center[dim] is the region
 * centre, levels[dim] its bisection depth per dimension (half-width = root
 * half-width * 2^-level).  Used by the parity tests to compare the device
 * integrand with the CPU oracle point by point. */
int g3l_debug_region(g3l_ctx *ctx, const g3l_integral *item, const double *center,
                     const int *levels, int precision, double *values, double out[3]);

/* g3l_eval without allocation (no counterpart in the reference, whose term methods
 * copy their points through a fresh device buffer every round).  Same items, results
 * and statuses as g3l_eval, for callers that must not allocate device or pinned host
 * memory while evaluating -- e.g. a process whose device memory is owned by another
 * allocator, or a loop that cannot take an allocation's implicit synchronisation.
 *  - Scratch: one fixed 64 MiB device array per device, built into the library.  A
 *    call may hold at most 1024 integrals and as many region slots as fit beside them
 *    and the ~31 MB of re-evaluation scratch (about 117 bytes per slot; each integral
 *    takes 3 + (max_eval + P) / (2 P) slots for its P-point rule, so ~305k slots, e.g.
 *    145 seven-dimensional integrals at max_eval = 1e6).  An item with max_eval = 0
 *    takes the context's unlimited_pool slots (g3l_options; 1 << 20 by default, more
 *    than the scratch holds), so such items need unlimited_pool lowered to ~300k or
 *    less.  Larger calls fail with G3L_ERR_INVALID and a message stating the bytes
 *    needed; nothing is evaluated.
 *  - Set-up: the first call on a device looks up the scratch's device address (with
 *    that device current); make that first call before capturing any stream.
 *  - The scratch (and the host staging beside it) is shared by every context on a
 *    device and keeps the last call's contents.  Two calls whose kernels were on the
 *    GPU at once would race on it; the library prevents that by serialising the calls
 *    on one device with a lock, and every call waits for its own kernels before it
 *    returns.  Calls on different devices run side by side.
 *  - Rounds are driven from the host with plain kernel launches (one small
 *    device-to-host read per round).  The context's workspace (its pools and graphs)
 *    is not touched; its statistics (g3l_get_stats) are replaced by this call's. */
int g3l_eval_static(g3l_ctx *ctx, const g3l_integral *items, int n, int precision,
                    g3l_result *out);

/* Copy the live regions of item `index` of the last g3l_eval (before any other
 * call on the context): centres and levels dimension-major ([dim][n]), value and
 * error in the integral's units, and the stored split dimension; unc (optional,
 * [2][n]) receives the mixed path's relative bounds on the FP32 error of err and
 * of val (0 for regions evaluated in FP64).  With max_regions below the region
 * count only *n_regions is written.  Used by the tests to compare the region
 * sets of the two precisions. */
int g3l_debug_pool(g3l_ctx *ctx, int index, int max_regions, double *centers, int *levels,
                   double *val, double *err, int *split, float *unc, int *n_regions);

/* Issue-rate probe on the context's device: FP32 and FP64 fused multiply-add
 * throughput in TFLOP/s (2 flops per FMA), measured with CUDA events. */
int g3l_measure_peaks(g3l_ctx *ctx, double *fp32_tflops, double *fp64_tflops);

const char *g3l_last_error(void);
int g3l_abi_version(void);

/* The reference's cubature entry point for host integrands (the 1-D
 * precomputations and Cosmology::comovingDistance call it), with the same
 * contract as src/cubature.h:55-57 and :90-94. */
typedef int (*g3l_integrand_v)(unsigned ndim, size_t npt, const double *x, void *fdata,
                               unsigned fdim, double *fval);
int g3l_hcubature_v(unsigned fdim, g3l_integrand_v f, void *fdata, unsigned dim,
                    const double *xmin, const double *xmax, size_t maxEval, double reqAbsError,
                    double reqRelError, int norm, double *val, double *err);

/* The reference's table precomputation (doPrecomputations.x,
 * src/doPrecomputations.cpp:40-134) on the device: from a flat LCDM cosmology and a
 * source redshift distribution, the lensing efficiency, comoving distance and its
 * derivative on nbins z bins (src/Cosmology.cpp:74-193), the linear power spectrum
 * (Eisenstein & Hu transfer function normalised to sigma8, src/Powerspectrum.cpp:9-196)
 * on z x k, and the concentration, Sheth-Tormen mass function and halo bias on z x m
 * (src/Powerspectrum.cpp:117-150, src/HMF.cpp:7-84).  Grids as the reference's:
 * z_i = zmin + i (zmax-zmin)/nbins, m_j and k_j logarithmic from mmin and kmin.
 * Every adaptive 1-D integral (sigma^2, dsigma^2/dm, M*, the amplitude, the comoving
 * distances) runs on the device with the reference's refinement.  The lens
 * distributions p_lens1/2 are inputs of the model, not outputs of this step. */
typedef struct g3l_precompute_in {
    double cosmo[6];            /* Om, OL, Ob, sigma8, H0 [km/s/Mpc], ns */
    const double *nz_z, *nz_v;  /* source n(z): redshifts and values [n_nz], as read
                                   from the reference's n(z) file */
    int n_nz;
    double zmin, zmax, mmin, mmax, kmin, kmax;
    int nbins;                  /* 1..4096 */
} g3l_precompute_in;
typedef struct g3l_precompute_out {
    double *g, *w, *dwdz;              /* caller's arrays [nbins] */
    double *P_lin, *conc, *hmf, *b_h;  /* caller's arrays [nbins*nbins], z-major */
    double amplitude;                  /* P(k) normalisation [Mpc^3] */
    double device_ms;                  /* device time of the computation */
    long long integrals, points;       /* 1-D integrals and integrand evaluations */
} g3l_precompute_out;
int g3l_precompute_tables(const g3l_precompute_in *in, int device, g3l_precompute_out *out);

/* The reference's ASCII inputs, read as its drivers read them (host only, no device
 * work).  Numbers are parsed by C++ stream extraction; reading stops at the first
 * token that is not a number.  Where the reference exits or reads undefined values,
 * these return G3L_ERR_INVALID with g3l_last_error().
 *
 * A 1-D table of "x y" lines (g3lhalo::Function, src/Function.cpp:6-39), sampled at
 * nbins bins: linear interpolation, default_value outside [x_first, x_last).
 * log_bins = 0: x_i = min + i (max-min)/nbins (Function::read, src/Function.cpp:89-105,
 * the z tables and the SCALING arrays); 1: x_i = exp(log min + i log(max/min)/nbins)
 * (Function::readLog, src/Function.cpp:108-124).  out: [nbins]. */
int g3l_read_function(const char *path, double default_value, int nbins, double min, double max,
                      int log_bins, double *out);
/* A 2-D table of "x1 x2 y" lines (g3lhalo::Function2D) on nbins x nbins bins, x1
 * linear in [min1, max1), x2 logarithmic in [min2, max2) (Function2D::read,
 * src/Function2D.cpp:46-95: the hmf, b_h and concentration tables over (z, m), P_lin
 * over (z, k)).  out: [nbins * nbins], first index x1. */
int g3l_read_function2d(const char *path, double default_value, int nbins, double min1,
                        double max1, double min2, double max2, double *out);
/* A HOD parameter file ("M_min", "sigma", "M'", "beta", "alpha", "f" lines,
 * src/Params.cpp:7-74) as {f, alpha, Mth, sigma, M', beta}. */
int g3l_read_hod_params(const char *path, double params[6]);
/* A cosmology file ("Omega_m", "Omega_Lambda", "Omega_b", "sigma8", "H0", "ns" lines,
 * src/Cosmology.cpp:11-72) as {Om, OL, Ob, sigma8, H0, ns}. */
int g3l_read_cosmology(const char *path, double cosmo[6]);
/* Aperture triplets "theta1 theta2 theta3" in arcmin (src/calculateNNMap.cu:121-129).
 * Stores up to cap triplets in thetas[3*cap] and the number in the file in *n. */
int g3l_read_triplets(const char *path, double *thetas, int cap, int *n);

#ifdef __cplusplus
}
#endif
#endif /* G3L_GPU_H */
