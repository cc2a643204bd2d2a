"""FP32 error of the mixed path's decision quantities, measured against the FP64 form.

The mixed-precision path evaluates the integrand in FP32 and decides in FP64 from the
FP32 rule sums, treating every point value v as exact to within eps |v| + tau
(g3l_options.unc_eps_rel, unc_tau_abs).  This module measures how large eps must be to
cover the actual FP32 error of the quantities those decisions read, region by region:

- the 7th-degree value (the region's contribution to the integral),
- the error estimate |res7 - res5| (the selection key),
- the fourth differences of each dimension (the split dimension,
  src/hcubature.cpp:512-576 of the reference).

For a quantity Q = sum_p w_p v_p the effective eps is the smallest eps with
|Q32 - Q64| <= sum_p |w_p| (eps |v32_p| + tau); the bound holds for a region when that
eps is at most unc_eps_rel.  The point values come from Context.debug_region in both
precisions (the FP32 integrand is scaled by a per-integral constant, which is divided
out).
"""
import numpy as np

LAMBDA2 = 0.3585685828003180919906451539079374954541
LAMBDA4 = 0.9486832980505137995996680633298155601160
RATIO = (LAMBDA2 * LAMBDA2) / (LAMBDA4 * LAMBDA4)


def rule_weights(dim):
    """Per-point weights (res7, res5) of the dim-dimensional Genz-Malik rule in the
    reference's point order (centre, 4 axis points per dimension, the (+-r4, +-r4) pairs,
    the corners)."""
    n = 1 + 4 * dim + 2 * dim * (dim - 1) + (1 << dim)
    w1 = (12824 - 9120 * dim + 400 * dim * dim) / 19683
    w3 = (1820 - 400 * dim) / 19683
    w5 = 6859 / 19683 / (1 << dim)
    wE1 = (729 - 950 * dim + 50 * dim * dim) / 729
    wE3 = (265 - 100 * dim) / 1458
    w2, w4, wE2, wE4 = 980 / 6561, 200 / 19683, 245 / 486, 25 / 729
    r7 = np.zeros(n)
    r5 = np.zeros(n)
    r7[0], r5[0] = w1, wE1
    for k in range(dim):
        b = 1 + 4 * k
        r7[b:b + 2], r5[b:b + 2] = w2, wE2
        r7[b + 2:b + 4], r5[b + 2:b + 4] = w3, wE3
    k0 = 1 + 4 * dim
    nrr = 2 * dim * (dim - 1)
    r7[k0:k0 + nrr], r5[k0:k0 + nrr] = w4, wE4
    r7[k0 + nrr:] = w5
    return r7, r5


def effective_eps(v32, v64, dim, tau=1e-34, scale=None):
    """Effective eps of one region's value, error estimate and fourth differences.

    v32: FP32 point values (the kernel's scaled units); v64: FP64 point values; scale:
    v64 / v32 for an exact FP32 value (default: the median ratio over the points where
    both are non-zero).  Returns {"val", "err", "diff"} (diff: the largest over the
    dimensions)."""
    v32 = np.asarray(v32, dtype=np.float64)
    v64 = np.asarray(v64, dtype=np.float64)
    if scale is None:
        ok = (v32 != 0) & (v64 != 0)
        scale = float(np.median(v64[ok] / v32[ok])) if ok.any() else 1.0
    d = v32 - v64 / scale
    a = np.abs(v32)
    r7, r5 = rule_weights(dim)

    def eff(w):
        den = np.sum(np.abs(w) * a)
        num = abs(np.sum(w * d)) - tau * np.sum(np.abs(w))
        return max(num, 0.0) / den if den > 0 else 0.0

    diffs = []
    for k in range(dim):
        b = 1 + 4 * k
        D = d[b] + d[b + 1] - 2 * d[0] - RATIO * (d[b + 2] + d[b + 3] - 2 * d[0])
        U = a[b] + a[b + 1] + RATIO * (a[b + 2] + a[b + 3]) + (2 - 2 * RATIO) * a[0]
        num = abs(D) - 4.0 * tau  # tau x (1 + 1 + RATIO (1 + 1) + (2 - 2 RATIO))
        diffs.append(max(num, 0.0) / U if U > 0 else 0.0)
    return {"val": eff(r7), "err": eff(r7 - r5), "diff": max(diffs)}


def measure(ctx, specs, mixed, fp64, results, items=None, regions=24, largest=8,
            significance=(1e-9, 1e-7, 1e-5, 1e-3), seed=0, tau=1e-34):
    """Effective eps over regions of a finished evaluation of `specs` (the context's
    last g3l_eval, with `results` its output), binned by the region's share of its
    integral's error estimate.

    items: indices of specs to sample (default all); per item `regions` random live
    regions and its `largest` regions by error.  mixed, fp64: the precision constants.
    Returns {term: {significance: {"n", "val", "err", "diff"}}} with the largest
    effective eps among the regions whose FP64 error is >= significance x the
    integral's error."""
    rng = np.random.default_rng(seed)
    out = {}
    for idx in (range(len(specs)) if items is None else items):
        sp = specs[idx]
        term, dim = sp[1], sp[1] + 4
        pool = ctx.debug_pool(idx)
        n = pool["n"]
        if n == 0:
            continue
        cen = pool["centers"][:dim * n].reshape(dim, n).T
        lev = pool["levels"][:dim * n].reshape(dim, n).T
        pick = set(rng.choice(n, size=min(n, regions), replace=False).tolist())
        pick |= set(np.argsort(-pool["err"])[:largest].tolist())
        E = abs(float(results["err"][idx]))
        for j in sorted(pick):
            v32, _ = ctx.debug_region(sp, cen[j], lev[j], mixed)
            v64, o64 = ctx.debug_region(sp, cen[j], lev[j], fp64)
            if np.count_nonzero((v32 != 0) & (v64 != 0)) < 3:
                continue
            e = effective_eps(v32, v64, dim, tau)
            share = abs(float(o64[1])) / E if E > 0 else 0.0
            for s in significance:
                if share >= s:
                    b = out.setdefault(term, {}).setdefault(s, {"n": 0, "val": 0.0, "err": 0.0,
                                                                "diff": 0.0})
                    b["n"] += 1
                    for q in ("val", "err", "diff"):
                        b[q] = max(b[q], e[q])
    return out


def main(argv=None):
    """The error model on the benchmark workload (220 triplets x NNMap 1h+2h+3h, rtol 1e-4,
    maxEval 1e6, 64 z x 128 m x 256 k tables): prints one JSON object, per term and
    significance, the number of regions and the largest effective eps."""
    import argparse
    import json

    import g3lhalo_gb300 as G
    from g3lhalo_gb300 import workloads as W
    from g3lhalo_gb300.tables import make_tables
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--hods", type=int, nargs="+", default=[3, 0],
                    help="indices into the 64 seeded fit-sweep HOD vectors")
    ap.add_argument("--stride", type=int, default=4, help="every stride-th integral")
    ap.add_argument("--regions", type=int, default=40, help="random live regions per integral")
    ap.add_argument("--largest", type=int, default=40, help="largest-error regions per integral")
    a = ap.parse_args(argv)
    T = make_tables(Nz=64, Nm=128, Nk=256)
    trip = W.triplets_all()
    hods = W.hod_sweep(64, seed=12345)
    ctx = G.Context(T, device=0)
    opt = ctx.options()
    merged = {}
    for h in a.hods:
        ctx.set_hod(0, hods[h])
        specs = [(G.NNMAP, t, 0, 0, tuple(th), 1e-4, 1_000_000) for th in trip for t in (1, 2, 3)]
        r = ctx.eval(specs, G.MIXED)
        m = measure(ctx, specs, G.MIXED, G.FP64, r, items=range(0, len(specs), a.stride),
                    regions=a.regions, largest=a.largest, seed=h)
        for term, bins in m.items():
            for s, b in bins.items():
                o = merged.setdefault(term, {}).setdefault(s, {"n": 0, "val": 0.0, "err": 0.0,
                                                               "diff": 0.0})
                o["n"] += b["n"]
                for q in ("val", "err", "diff"):
                    o[q] = max(o[q], b[q])
    print(json.dumps({"unc_eps_rel": opt.unc_eps_rel, "hods": a.hods, "stride": a.stride,
                      "effective_eps": {"%dh" % t: {"%g" % s: v for s, v in sorted(b.items())}
                                        for t, b in sorted(merged.items())}}))


if __name__ == "__main__":
    main()
