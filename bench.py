"""Benchmark: NNMap model evaluations per second on one GB300.

One step = one model evaluation of <N N M_ap>: the 1-, 2- and 3-halo terms of
all 220 aperture triplets theta1 <= theta2 <= theta3 from 10 log-spaced radii in
[0.5', 16'] (660 adaptive Genz-Malik integrals over 5/6/7 dimensions), rtol 1e-4,
an evaluation cap of 1e6 per integral (the reference's integrals never reach
rtol 1e-4, so the cap decides the work), on synthetic tables (64 z x 128 m x
256 k bins) and one HOD vector per step (seeded draws from the fit-sweep box).

Reported (one JSON line on rank 0):
  value       mixed-precision evals/s, device time (CUDA events) of the whole
              refinement loop, inputs resident
  e2e         the same through the public call (HOD update + descriptors in,
              results out, host wall clock)
  fp64        the plain all-FP64 form on the same device (the >= 5x comparison)
  parity      max relative deviation of every mixed term from the FP64 form
  roofline    the dominant rule kernel (NNMap 2-halo) against the measured FP32
              FMA rate of this device
  cpu_baseline the CPU oracle (restated reference CPU path, OpenMP over all host
              cores) on 11 of the 220 triplets, timed; value = 11/220 of an evaluation
              per measured second
Further legs: serving (continuous batching at a sweep of Poisson arrival rates, each
served result checked against g3l_eval; the same stream on an FP64 server, with every
term compared), sweep (256 HOD vectors in one launch; the first 16 again in FP64, every
term compared), nmapmap_twopop (NMapMap plus two-population NNMap), config0 (the FP64
1-halo term of 5 equal-scale triplets on the host cores and on the device), precompute
(the table precomputation on 64 bins).
--impl reference times the reference's CPU path alone (the oracle restatement) on the
same workload: the timed steps split the 220 triplets round robin, so 20 steps time one
whole model evaluation, measured, not extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NNMap evals/s (220 triplets,1h+2h+3h,rtol 1e-4) mixed vs FP64; p50/p99 ms"
MAX_EVAL = 1_000_000
RTOL = 1e-4
# FP32 operations per integrand point of the NNMap 2-halo rule (algorithmic): the
# integrand with its u_NFW calls de-duplicated within a point, counted by ncu as thread-
# level fadd + fmul + 2 ffma on the kernel version that evaluated every u_NFW per point
# (3.434e11 over 2.2005e8 points of the benchmark).  DRAM traffic per launch (read +
# write): three launches of the kernel on the 110-triplet case (7.9 MB per ms of kernel
# time), scaled by duration to the benchmark's mean launch (17.65 ms / 28 launches);
# profiles/k_evalmx_nnmap2h.md.
FLOPS_PER_POINT = {"nnmap_2h": 1561.0}
DRAM_BYTES_PER_LAUNCH = {"nnmap_2h": 5.0e6}
# Pipe utilisation (% of peak while the SMs are active) of the dominant kernels, from one
# `ncu --set full` capture of three launches each (profiles/k_evalmx_nnmap2h.md,
# profiles/k_re_points_nnmap3h.md, profiles/k_nbar_densities.md,
# profiles/k_pc_integrate_precompute.md).
PIPES_NCU = {
    "k_evalmx<NNMap,2h> (FP32 rule)": {"fma": 38.7, "alu": 36.6, "xu_mufu": 8.1, "fp64": 9.1,
                                       "issue_active": 70.5, "warps_active": 33.4},
    "k_re_ucache<NNMap,2h> (FP64 re-evaluation, u_NFW)": {"fp64": 81.0},
    "k_re_points<NNMap,3h> (FP64 re-evaluation, points)": {"fp64": 46.3},
    "k_nbar (n_bar integrals)": {"fp64": 57.7},
    "k_pc_integrate (table precompute)": {"fp64": 79.2, "fma": 0.5, "xu_mufu": 0.1},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--max-eval", type=int, default=MAX_EVAL)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    # smaller cases for profiler captures: N evenly spaced triplets, host-driven rounds
    ap.add_argument("--triplets", type=int, default=0)
    ap.add_argument("--host-loop", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-config2", action="store_true")
    ap.add_argument("--no-precompute", action="store_true")
    # batched fit sweep: this many HOD vectors in one launch (0 = skip)
    ap.add_argument("--sweep", type=int, default=256)
    # of which this many are integrated again in the FP64 form and compared term by term
    ap.add_argument("--sweep-parity", type=int, default=16)
    ap.add_argument("--no-config0", action="store_true")
    return ap.parse_args()


def W_hod_default():
    from g3lhalo_gb300 import workloads as W
    return W.hod_default()


def workload():
    from g3lhalo_gb300 import workloads as W
    from g3lhalo_gb300.tables import make_tables
    T = make_tables(Nz=64, Nm=128, Nk=256)
    trip = W.triplets_all()
    hods = W.hod_sweep(64, seed=12345)
    return T, trip, hods


def config(n_trip, me, extra=None):
    c = {"workload": "NNMap <N1 N2 Map> 1h+2h+3h, 220 triplets theta1<=theta2<=theta3 from 10 "
                     "log-spaced radii in [0.5,16] arcmin, rtol 1e-4, maxEval %d per integral, "
                     "tables 64 z x 128 m x 256 k, one HOD vector per step" % me,
         "integrals_per_step": 3 * n_trip, "max_eval": me, "rtol": RTOL,
         "tables": {"Nz": 64, "Nm": 128, "Nk": 256, "zmin": 0.001, "zmax": 2.0,
                    "mmin": 1e10, "mmax": 1e17, "k_h_per_mpc": [1e-4, 1e3]},
         "l2": "no flush: each step rewrites ~0.3 GB of region pools (> 129 MB L2)"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """Samples nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.rows, self.proc = [], None
        self.device = device

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle(T, hod):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as P
    # one population (hod1 == hod2): the same-population branch, as the device runs it
    return P.Oracle(T, hod, None, clamp_k=True)


def _cpu_terms(O, trip, idx, me, terms=(1, 2, 3)):
    """The oracle's FP64 terms of triplets idx (NNMap, one population); wall seconds and
    integrand points."""
    t0 = time.perf_counter()
    pts = 0
    for i in idx:
        for t in terms:
            pts += O.term(0, t, trip[i], 1, 2, maxEval=me, rtol=RTOL)[2]
    return time.perf_counter() - t0, pts


def cpu_sample(T, trip, hod, me, n_trip):
    """Oracle on the host cores: n_trip evenly spaced triplets x 3 terms, timed; the
    rate is the fraction of a model evaluation they make (n_trip / 220) per second."""
    O = _oracle(T, hod)
    idx = np.linspace(0, len(trip) - 1, n_trip).astype(int)
    dt, pts = _cpu_terms(O, trip, idx, me)
    return {"value": (n_trip / len(trip)) / dt, "unit": "evals/s", "cores": os.cpu_count(),
            "kind": "port", "seconds": dt, "points_per_s": pts / dt,
            "sample": "%d evenly spaced of the 220 triplets x 3 terms at maxEval %d (oracle "
                      "restatement of the reference CPU path, OpenMP over all host cores); "
                      "value = %d/220 of an evaluation / the measured seconds" % (n_trip, me, n_trip)}


def reference_steps(n_trip, steps):
    """Triplets of each timed step of the reference arm: step s takes every triplet
    j with j % steps == s % steps, so `steps` consecutive steps cover all of them."""
    k = max(1, min(steps, n_trip))
    return [list(range(s % k, n_trip, k)) for s in range(steps)]


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle restatement, OpenMP over all host cores) on
    the benchmark's model evaluation, measured: the timed steps split the 220 triplets
    between them (round robin), so --steps 20 time exactly one whole evaluation; the
    value is the evaluations covered / the measured seconds.  Warm-up steps take one
    triplet each."""
    if rank != 0:
        return
    T, trip, hods = workload()
    O = _oracle(T, hods[0])
    for s in range(args.warmup):
        _cpu_terms(O, trip, [(7 * s) % len(trip)], args.max_eval)
    parts = reference_steps(len(trip), args.steps)
    res, covered = [], 0
    for idx in parts:
        dt, _ = _cpu_terms(O, trip, idx, args.max_eval)
        res.append(dt)
        covered += len(idx)
    total = float(np.sum(res))
    evals = covered / len(trip)
    value = evals / total
    sample = ("%d timed steps of %s triplets x 3 terms each (round robin over the 220), "
              "%.3g model evaluations in %.1f s measured, no extrapolation"
              % (args.steps, "/".join(sorted({str(len(p)) for p in parts})), evals, total))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": config(len(trip), args.max_eval),
            "evaluations_timed": evals,
            "p50_ms": float(np.percentile(np.array(res) * 1e3, 50)),
            "p99_ms": float(np.percentile(np.array(res) * 1e3, 99)),
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(dev_s, wall_s, dist=None):
    """Device and wall time of the timed steps, the maximum over the replicas (one
    rank per GPU; the replicas share no data, so this is the only collective)."""
    if dist is None:
        return dev_s, wall_s
    import torch
    tt = torch.tensor([dev_s, wall_s], dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt[0]), float(tt[1])


def parity(mixed, fp64):
    """Largest relative deviation of every mixed-precision term from the FP64 form."""
    rel = np.abs(mixed["val"] - fp64["val"]) / np.abs(fp64["val"])
    return {"max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
            "terms": int(rel.size), "terms_over_1e-4": int((rel > 1e-4).sum()),
            "neval_identical": bool(np.array_equal(mixed["neval"], fp64["neval"])),
            "status_ok": bool((mixed["status"] == 0).all() and (fp64["status"] == 0).all())}


def sweep_leg(G, ctx, trip, hods, n_hod, max_eval, n_parity):
    """Batched fit sweep: n_hod HOD vectors x 220 triplets x 3 terms in one launch; the
    first n_parity vectors are integrated again in the FP64 form (one call) and every
    one of their terms compared."""
    from g3lhalo_gb300 import workloads as W
    hs = hods[:n_hod] if n_hod <= len(hods) else W.hod_sweep(n_hod, seed=12345)
    t0 = time.perf_counter()
    ctx.set_hods(16 + np.arange(n_hod), hs)  # n_bar of every vector in one device launch
    t_hod = time.perf_counter() - t0
    specs = [(G.NNMAP, t, 16 + k, 16 + k, tuple(th), RTOL, max_eval)
             for k in range(n_hod) for th in trip for t in (1, 2, 3)]
    ctx.eval(specs[:3 * len(trip)], G.MIXED)  # warm the graph shapes
    t0 = time.perf_counter()
    r = ctx.eval(specs, G.MIXED)
    wall = time.perf_counter() - t0
    st = ctx.stats()
    out = {"hod_vectors": n_hod, "integrals": len(specs),
           "model_evals_per_s": n_hod / (st["device_ms"] * 1e-3),
           "device_ms": st["device_ms"], "wall_s": wall, "hod_update_s": t_hod,
           "points_per_s": st["points_evaluated"] / (st["device_ms"] * 1e-3),
           "rounds": st["rounds"], "status_ok": bool((r["status"] == 0).all()),
           "workload": "%d seeded HOD vectors (the fit-sweep box) x 220 triplets x 1h+2h+3h, "
                       "rtol 1e-4, maxEval %d, one g3l_eval call" % (n_hod, max_eval)}
    if n_parity:
        m = min(n_parity, n_hod) * 3 * len(trip)
        r64 = ctx.eval(specs[:m], G.FP64)
        par = parity(r[:m], r64)
        par["hod_vectors"] = min(n_parity, n_hod)
        par["fp64_device_ms"] = ctx.stats()["device_ms"]
        out["parity_vs_fp64"] = par
    return out


def config0_leg(G, T, hod, max_eval):
    """SURVEY config 0: the FP64 NNMap 1-halo term on the 5 equal-scale triplets
    (0.5', 1', 2', 4', 8'), rtol 1e-4, maxEval 1e6, on the host cores (the oracle
    restatement of the reference CPU path, OpenMP over all cores) and on the device in
    both forms, with the device results against the host's."""
    from g3lhalo_gb300 import workloads as W
    tri = W.triplets_equal()
    O = _oracle(T, hod)
    t0 = time.perf_counter()
    cpu = [O.term(0, 1, tuple(th), 1, 2, maxEval=max_eval, rtol=RTOL) for th in tri]
    cpu_s = time.perf_counter() - t0
    c = G.Context(T, device=0)
    c.set_hod(0, hod)
    specs = [(G.NNMAP, 1, 0, 0, tuple(th), RTOL, max_eval) for th in tri]
    out = {"integrals": len(specs), "cpu_s": cpu_s, "cpu_cores": os.cpu_count(),
           "cpu_kind": "port"}
    vc = np.array([x[0] for x in cpu])
    nc = np.array([x[2] for x in cpu])
    for name, prec in (("fp64", G.FP64), ("mixed", G.MIXED)):
        c.eval(specs, prec)
        ms = []
        for _ in range(3):
            r = c.eval(specs, prec)
            ms.append(c.stats()["device_ms"])
        out[name] = {"device_ms": float(np.median(ms)), "speedup_vs_cpu": cpu_s / (np.median(ms) * 1e-3),
                     "max_rel_vs_cpu": float(np.max(np.abs(r["val"] - vc) / np.abs(vc))),
                     "neval_identical_to_cpu": bool(np.array_equal(r["neval"], nc))}
    c.close()
    out["workload"] = ("NNMap 1-halo, FP64, theta1=theta2=theta3 in {0.5,1,2,4,8} arcmin, rtol "
                       "1e-4, maxEval %d, benchmark tables, default HOD" % max_eval)
    return out


def config2_leg(G, trip, max_eval, reps=3):
    """NMapMap 1h+2h+3h plus two-population NNMap (second HOD and a second lens
    distribution, Gaussian mu 0.5 sigma 0.07) on all 220 triplets: 1320 integrals per
    evaluation, mixed precision against the FP64 form."""
    from g3lhalo_gb300 import workloads as W
    from g3lhalo_gb300.tables import make_tables
    T2 = make_tables(Nz=64, Nm=128, Nk=256, lens2=(0.5, 0.07))
    c2 = G.Context(T2)
    c2.set_hod(0, W.hod_default())
    c2.set_hod(1, W.hod_second())
    specs = [(G.NMAPMAP, t, 0, 0, tuple(th), RTOL, max_eval) for th in trip for t in (1, 2, 3)]
    specs += [(G.NNMAP, t, 0, 1, tuple(th), RTOL, max_eval) for th in trip for t in (1, 2, 3)]
    c2.eval(specs, G.MIXED)
    ms = []
    for _ in range(reps):
        r = c2.eval(specs, G.MIXED)
        ms.append(c2.stats()["device_ms"])
    st = c2.stats()
    r64 = c2.eval(specs, G.FP64)
    ms64 = c2.stats()["device_ms"]
    rel = np.abs(r["val"] - r64["val"]) / np.abs(r64["val"])
    c2.close()
    return {"integrals": len(specs), "evals_per_s": 1e3 / float(np.mean(ms)),
            "ms": float(np.mean(ms)), "fp64_evals_per_s": 1e3 / ms64,
            "mixed_over_fp64": ms64 / float(np.mean(ms)),
            "max_rel_vs_fp64": float(rel.max()), "terms_over_1e-4": int((rel > 1e-4).sum()),
            "neval_identical": bool(np.array_equal(r["neval"], r64["neval"])),
            "small_arg_fp64_evaluations": int(st["small_arg_fp64"]),
            "workload": "NMapMap (HOD 1, lens 1) + NNMap two populations (HOD 1 and 2, lens "
                        "1 and lens 2 = Gaussian 0.5/0.07), 220 triplets x 3 terms each, rtol "
                        "1e-4, maxEval %d" % max_eval}


PRECOMPUTE_ARGS = (0.001, 2.0, 1e10, 1e17, 1e-4 * 0.7, 1e3 * 0.7, 64)
PRECOMPUTE_COSMO = (0.3, 0.7, 0.045, 0.8, 70.0, 0.96)


def precompute_source_nz():
    z = np.linspace(0.0, 3.0, 60)
    nz = z * z * np.exp(-(z / 0.5) ** 1.5)
    return z, nz / (nz.sum() * (z[1] - z[0]))


def precompute_leg(G, reps=3):
    """The reference's table precomputation (doPrecomputations) for 64 bins on the
    device: ~25k adaptive 1-D integrals (sigma^2, dsigma^2/dm, M*, distances); device
    time (CUDA events) of the best of `reps` runs."""
    z, nz = precompute_source_nz()
    runs = [G.precompute_tables(PRECOMPUTE_COSMO, z, nz, *PRECOMPUTE_ARGS) for _ in range(reps)]
    best = min(runs, key=lambda r: r["device_ms"])
    return best, {"nbins": 64, "device_ms": best["device_ms"], "integrals": best["integrals"],
                  "points": best["points"],
                  "points_per_s": best["points"] / (best["device_ms"] * 1e-3),
                  "workload": "doPrecomputations: g, w, dw/dz, P_lin, concentration (M* from "
                              "256 sigma^2 per z), Sheth-Tormen n(m, z) and b_h on 64 bins; FP64"}


def precompute_cpu(dev):
    """The oracle restatement of the same precomputation on the host cores (OpenMP over
    the integrals), and the device tables' largest deviation from it."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle"))
    import pyoracle as P
    z, nz = precompute_source_nz()
    t0 = time.perf_counter()
    o = P.precompute(PRECOMPUTE_COSMO, z, nz, *PRECOMPUTE_ARGS)
    dt = time.perf_counter() - t0
    rel = max(float(np.max(np.abs(dev[k] - o[k]) / np.maximum(np.abs(o[k]), 1e-300)))
              for k in ("g", "w", "dwdz", "P_lin", "conc", "hmf", "b_h"))
    return {"seconds": dt, "cores": os.cpu_count(), "kind": "port",
            "device_max_rel_vs_port": rel}


SERVING_RATES = (10.0, 100.0, 1000.0, 2000.0)
SERVING_RTOLS = (1e-3, 1e-4, 1e-5)


def serving_requests(trip, n_req, max_eval, rng):
    """Model evaluations from the config-4 distribution: triplet count log-uniform in
    1..220, NNMap or NMapMap, rtol in {1e-3, 1e-4, 1e-5}, one of 8 HOD slots."""
    reqs = []
    for _ in range(n_req):
        nt = int(np.clip(np.round(np.exp(rng.uniform(0, np.log(220)))), 1, 220))
        idx = np.sort(rng.choice(len(trip), nt, replace=False))
        kind = int(rng.integers(0, 2))
        slot = 8 + int(rng.integers(0, 8))
        rtol = SERVING_RTOLS[int(rng.integers(0, len(SERVING_RTOLS)))]
        reqs.append([(kind, t, slot, slot, tuple(trip[i]), rtol, max_eval)
                     for i in idx for t in (1, 2, 3)])
    return reqs


def serve_stream(G, ctx, precision, reqs, rate, rng):
    """Submit `reqs` with seeded Poisson gaps while earlier ones run; latency = submit
    to completion of each request."""
    srv = G.Server(ctx, precision, max_items_per_term=2048, pool_regions=1 << 24,
                   rounds_per_launch=4)
    gaps = rng.exponential(1.0 / rate, len(reqs))
    tickets, lat, res = [], [], []
    t0 = time.perf_counter()
    for q, gap in zip(reqs, gaps):
        time.sleep(gap)
        tickets.append(srv.submit(q))
    for t in tickets:
        r, ms = srv.poll(t)
        lat.append(ms)
        res.append(r)
    wall = time.perf_counter() - t0
    info = srv.info()
    srv.close()
    n_int = sum(len(q) for q in reqs)
    out = {"arrival_rate_per_s": rate, "requests": len(reqs), "integrals": n_int,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(np.mean(lat)), "wall_s": wall,
           "requests_per_s": len(reqs) / wall,
           "model_evals_per_s": n_int / 660.0 / wall, "launches": info["launches"]}
    return out, res


def served_equals_eval(G, ctx, precision, reqs, res):
    """Every served request against g3l_eval of the same integrals in the same form (one
    call): integrals whose value or evaluation count differ."""
    flat = [it for q in reqs for it in q]
    ref = ctx.eval(flat, precision)
    got = np.concatenate(res)
    return {"integrals": len(flat),
            "differ": int(np.sum((got["val"] != ref["val"]) | (got["neval"] != ref["neval"])))}


def serving_leg(G, ctx, trip, hods, args, n_req=48, n_fp64=6, seed=7):
    """Continuous batching at a sweep of Poisson arrival rates (config 4), and the same
    stream's saturated throughput with an all-FP64 server for comparison."""
    for k in range(8):
        ctx.set_hod(8 + k, hods[(40 + k) % len(hods)])
    rates = []
    for i, rate in enumerate(SERVING_RATES):
        rng = np.random.default_rng(seed + i)
        reqs = serving_requests(trip, n_req, args.max_eval, rng)
        o, res = serve_stream(G, ctx, G.MIXED, reqs, rate, rng)
        # continuous batching must not change a result: served == g3l_eval, bit for bit
        o["vs_eval_mixed"] = served_equals_eval(G, ctx, G.MIXED, reqs, res)
        rates.append(o)
    rng = np.random.default_rng(seed + 100)
    reqs = serving_requests(trip, n_fp64, args.max_eval, rng)
    mixed, rm = serve_stream(G, ctx, G.MIXED, reqs, SERVING_RATES[-1], np.random.default_rng(1))
    fp64, rf = serve_stream(G, ctx, G.FP64, reqs, SERVING_RATES[-1], np.random.default_rng(1))
    low = rates[0]
    return {"p50_ms": low["p50_ms"], "p99_ms": low["p99_ms"],
            "arrival_rate_per_s": low["arrival_rate_per_s"], "rates": rates,
            "saturated_same_stream": {"requests": n_fp64, "mixed": mixed, "fp64": fp64,
                                      "mixed_over_fp64": mixed["model_evals_per_s"] /
                                                         fp64["model_evals_per_s"],
                                      "parity_vs_fp64": parity(np.concatenate(rm),
                                                               np.concatenate(rf))},
            "workload": "seeded Poisson arrivals at %s req/s, %d requests each; triplets per "
                        "request log-uniform 1..220, NNMap or NMapMap 1h+2h+3h, rtol in "
                        "{1e-3, 1e-4, 1e-5}, maxEval %d, 8 HOD vectors from the fit-sweep box; "
                        "model_evals_per_s counts 660 integrals as one evaluation"
                        % ("/".join("%g" % r for r in SERVING_RATES), n_req, args.max_eval)}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
        return

    import g3lhalo_gb300 as G
    T, trip, hods = workload()
    if args.triplets:
        trip = [trip[i] for i in np.linspace(0, len(trip) - 1, args.triplets).astype(int)]
    ctx = G.Context(T, device=local)
    ctx.set_hod(1, hods[0])
    if args.host_loop:
        ctx.set_options(use_graph=0)

    def specs(slot):
        return [(G.NNMAP, t, slot, slot, tuple(th), RTOL, args.max_eval) for th in trip
                for t in (1, 2, 3)]

    # the fit loop: each step sets a new HOD vector and evaluates the model
    def step(s, precision):
        ctx.set_hod(0, hods[s % len(hods)])
        return ctx.eval(specs(0), precision)

    for s in range(args.warmup):
        step(s, G.MIXED)
    # timed region
    clocks = Clocks(local)
    clocks.start()
    if dist:
        dist.barrier()
    dev_ms, wall_ms, launches = [], [], 0
    results = []
    t0 = time.perf_counter()
    for s in range(args.steps):
        w0 = time.perf_counter()
        r = step(args.warmup + s, G.MIXED)
        wall_ms.append((time.perf_counter() - w0) * 1e3)
        st = ctx.stats()
        dev_ms.append(st["device_ms"])
        launches += int(st["kernel_launches"])
        results.append(r)
    total = time.perf_counter() - t0
    if dist:
        dist.barrier()
    dev_total, total = max_over_ranks(sum(dev_ms) / 1e3, total, dist)
    clk = clocks.stop()
    st_last = ctx.stats()
    value = world * args.steps / dev_total
    e2e = world * args.steps / total
    out = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * dev_total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 integrand, f64 accumulation/decisions",
           "data": "synthetic: seeded tables (Sheth-Tormen, Eisenstein-Hu no-wiggle) and HOD "
                   "vectors; no public dataset",
           "p50_ms": float(np.percentile(dev_ms, 50)), "p99_ms": float(np.percentile(dev_ms, 99)),
           "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": int(st_last["h2d_bytes"]),
                   "d2h_bytes_per_step": int(st_last["d2h_bytes"]),
                   "p50_ms": float(np.percentile(wall_ms, 50)),
                   "p99_ms": float(np.percentile(wall_ms, 99)),
                   "includes": "HOD update (device n_bar integrals, copies), descriptor H2D, "
                               "device loop, result D2H"},
           "gpu_launches": launches, "clocks": clk,
           "stats_last_step": {k: st_last[k] for k in ("rounds", "regions_evaluated",
                                                        "points_evaluated", "escalated",
                                                        "escalated_full", "deferred", "polished",
                                                        "thr_checks",
                                                        "tie_fallbacks", "small_arg_fp64",
                                                        "group_points")}}
    if rank == 0:
        # peaks of this device
        p32, p64 = ctx.measure_peaks()
        # FP64 form on the same HOD vector as the last step, and parity of every term
        last_hod = (args.warmup + args.steps - 1) % len(hods)
        if not args.no_fp64:
            ctx.set_hod(0, hods[last_hod])
            r64 = ctx.eval(specs(0), G.FP64)
            s64 = ctx.stats()
            rel = np.abs(results[-1]["val"] - r64["val"]) / np.abs(r64["val"])
            out["fp64"] = {"value": 1e3 / s64["device_ms"], "unit": "evals/s",
                           "ms_per_step": s64["device_ms"],
                           "mixed_over_fp64": (1e3 / (dev_total * 1e3 / args.steps)) /
                                              (1e3 / s64["device_ms"])}
            out["parity_vs_fp64"] = {
                "max_rel": {"1h": float(rel[0::3].max()), "2h": float(rel[1::3].max()),
                            "3h": float(rel[2::3].max())},
                "median_rel": float(np.median(rel)), "terms_over_1e-4": int((rel > 1e-4).sum()),
                "neval_identical": bool(np.array_equal(results[-1]["neval"], r64["neval"]))}
        # roofline of the dominant rule kernel from a host-driven pass (per-kernel events)
        ctx.set_options(use_graph=0)
        ctx.set_hod(0, hods[last_hod])
        ctx.eval(specs(0), G.MIXED)
        sr = ctx.stats()
        ctx.set_options(use_graph=0 if args.host_loop else 1)
        g = 1  # NNMap 2-halo
        fpp = FLOPS_PER_POINT["nnmap_2h"]
        ms_g = sr["group_ms"][g]
        pts_g = sr["group_points"][g]
        kern = {"kernel": "k_evalmx<NNMap,2h>", "ms": ms_g, "points": pts_g,
                "points_per_s": pts_g / (ms_g * 1e-3) if ms_g else None,
                "share_of_loop": ms_g / max(1e-9, sum(sr["group_ms"]) + sr["reeval_ms"] +
                                            sr["select_ms"]),
                "group_ms": sr["group_ms"], "reeval_ms": sr["reeval_ms"],
                "select_ms": sr["select_ms"]}
        if fpp:
            ach = pts_g * fpp / (ms_g * 1e-3) / 1e12
            out["roofline"] = {"bound": "fp32", "achieved": ach, "peak": p32, "unit": "TFLOP/s",
                               "frac": ach / p32, "traffic": DRAM_BYTES_PER_LAUNCH["nnmap_2h"],
                               "traffic_unit": "bytes per launch (ncu dram read+write, 110-triplet "
                                               "case scaled by duration)",
                               "flops_per_point": fpp,
                               "peak_source": "measured FP32 FMA rate of this device "
                                              "(g3l_measure_peaks, CUDA events); the measured-peaks "
                                              "file holds only HBM and bf16 figures",
                               "pipes_ncu_pct": PIPES_NCU, **kern}
        else:
            out["roofline"] = {"bound": "fp32", "achieved": None, "peak": p32, "unit": "TFLOP/s",
                               "frac": None, "traffic": None, **kern}
        out["peaks_measured"] = {"fp32_tflops": p32, "fp64_tflops": p64}
        # secondary legs: a failure is recorded in the line instead of losing it
        def leg(key, fn):
            try:
                return fn()
            except Exception as e:  # noqa: BLE001
                out[key] = {"error": "%s: %s" % (type(e).__name__, e)}
                return None

        if not args.no_serving:
            r = leg("serving", lambda: serving_leg(G, ctx, trip, hods, args))
            if r is not None:
                out["serving"] = r
        if args.sweep:
            r = leg("sweep", lambda: sweep_leg(G, ctx, trip, hods, args.sweep, args.max_eval,
                                               args.sweep_parity))
            if r is not None:
                out["sweep"] = r
        if not args.no_config2:
            r = leg("nmapmap_twopop", lambda: config2_leg(G, trip, args.max_eval))
            if r is not None:
                out["nmapmap_twopop"] = r
        if not args.no_config0:
            r = leg("config0", lambda: config0_leg(G, T, W_hod_default(), args.max_eval))
            if r is not None:
                out["config0"] = r
        pre = None
        if not args.no_precompute:
            r = leg("precompute", lambda: precompute_leg(G))
            if r is not None:
                pre, out["precompute"] = r
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_sample(T, trip, hods[last_hod], args.max_eval, 11)
            if pre is not None:
                r = leg("cpu_precompute", lambda: precompute_cpu(pre))
                if r is not None:
                    out["cpu_baseline"]["precompute"] = r
        out["config"] = config(len(trip), args.max_eval)
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()
