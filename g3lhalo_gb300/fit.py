"""HOD fitting client on the serving API.

The reference's fitter (src/Fitstuff - not fixed/fitHelpers.cu:194-271, fit_twoPop.cu)
minimises chi^2 = d^T C^-1 d with GSL's Nelder-Mead simplex, where d stacks the
measured-minus-model <N1 N2 M_ap>, <N1 N1 M_ap> and <N2 N2 M_ap> over the triplets and
each model value is NNMap(theta1, theta2, theta3, type1, type2), i.e. the sum of the
three halo terms.  Here the same objective is evaluated through a continuous-batching
server: every vertex of the simplex is submitted at once (each with its own pair of HOD
slots), so the model evaluations of one iteration integrate concurrently on the device.
"""
from __future__ import annotations

import numpy as np

from . import api as A
from .workloads import hod_from_log10

# The two-population parameter vector of the reference (src/Fitstuff - not fixed/
# fitHelpers.h Params): per population f, alpha, log10 Mth, sigma, log10 M', beta.
PARAM_NAMES = ("f1", "f2", "alpha1", "alpha2", "lmth1", "lmth2", "sigma1", "sigma2",
               "lmp1", "lmp2", "beta1", "beta2")


def hods_from_params(p):
    """Parameter vector (PARAM_NAMES order) -> the two HOD slot vectors
    {f, alpha, Mth, sigma, M', beta} of the C ABI."""
    p = np.asarray(p, dtype=np.float64)
    h1 = np.array([p[0], p[2], 10.0 ** p[4], p[6], 10.0 ** p[8], p[10]])
    h2 = np.array([p[1], p[3], 10.0 ** p[5], p[7], 10.0 ** p[9], p[11]])
    return h1, h2


def params_from_log10(lmth, sig, lm1, slope, f=1.0):
    """One population's parameters in PARAM_NAMES form from the sweep's variables."""
    h = hod_from_log10(lmth, sig, lm1, slope, f=f)
    return h[0], h[1], np.log10(h[2]), h[3], np.log10(h[4]), h[5]


class ChiSquared:
    """chi^2 of NNMap model values against data, evaluated on a server.

    thetas: (Nx, 3) aperture radii [rad]; data: (3 * Nx,) the N1N2, N1N1 and N2N2
    blocks; inv_cov: (3 Nx, 3 Nx).  free: indices into PARAM_NAMES that are fitted;
    the others stay at `base`.  lo / hi: bounds of the free parameters (the reference's
    priors); points outside get chi^2 = +inf."""

    def __init__(self, server, ctx, thetas, data, inv_cov, base, free, lo, hi, rtol=1e-4,
                 max_eval=200_000, slot0=64, max_inflight=32):
        self.srv, self.ctx = server, ctx
        self.thetas = np.asarray(thetas, dtype=np.float64)
        self.data = np.asarray(data, dtype=np.float64)
        self.icov = np.asarray(inv_cov, dtype=np.float64)
        self.base = np.asarray(base, dtype=np.float64)
        self.free = list(free)
        self.lo, self.hi = np.asarray(lo, float), np.asarray(hi, float)
        self.rtol, self.max_eval = rtol, max_eval
        self.slots = list(range(slot0, slot0 + 2 * max_inflight))
        self.calls = 0

    def full(self, x):
        p = self.base.copy()
        p[self.free] = x
        return p

    def _specs(self, s1, s2):
        out = []
        for a, b in ((s1, s2), (s1, s1), (s2, s2)):
            for th in self.thetas:
                for t in (1, 2, 3):
                    out.append((A.NNMAP, t, a, b, tuple(th), self.rtol, self.max_eval))
        return out

    def model_many(self, xs):
        """Model vectors for several parameter points, integrated concurrently."""
        xs = [np.asarray(x, float) for x in xs]
        res = [None] * len(xs)
        pending = list(range(len(xs)))
        while pending:
            batch = pending[: len(self.slots) // 2]
            pending = pending[len(batch):]
            tickets = []
            for k, i in enumerate(batch):
                s1, s2 = self.slots[2 * k], self.slots[2 * k + 1]
                h1, h2 = hods_from_params(self.full(xs[i]))
                self.ctx.set_hod(s1, h1)
                self.ctx.set_hod(s2, h2)
                tickets.append((i, self.srv.submit(self._specs(s1, s2))))
            for i, t in tickets:
                r, _ = self.srv.poll(t)
                res[i] = r["result"].reshape(-1, 3).sum(axis=1)  # NNMap = 1h + 2h + 3h
        self.calls += len(xs)
        return res

    def many(self, xs):
        """chi^2 of several points (inf outside the bounds)."""
        out = np.full(len(xs), np.inf)
        inside = [i for i, x in enumerate(xs)
                  if np.all(np.asarray(x) >= self.lo) and np.all(np.asarray(x) <= self.hi)]
        models = self.model_many([xs[i] for i in inside])
        for i, m in zip(inside, models):
            d = self.data - m
            out[i] = float(d @ self.icov @ d)
        return out


def nelder_mead(fmany, x0, step, iters=100, tol=1e-10):
    """Nelder-Mead simplex minimisation (standard coefficients 1, 2, 1/2, 1/2).

    fmany(list of points) -> values: the initial simplex and each shrink are evaluated
    as one batch.  Returns (best point, best value, history of best values)."""
    x0 = np.asarray(x0, float)
    n = len(x0)
    simplex = [x0] + [x0 + np.eye(n)[i] * step[i] for i in range(n)]
    fv = list(fmany(simplex))
    hist = []
    for _ in range(iters):
        order = np.argsort(fv)
        simplex = [simplex[i] for i in order]
        fv = [fv[i] for i in order]
        hist.append(fv[0])
        if abs(fv[-1] - fv[0]) <= tol * (abs(fv[0]) + tol):
            break
        c = np.mean(simplex[:-1], axis=0)
        xr = c + (c - simplex[-1])
        xe = c + 2.0 * (c - simplex[-1])
        xc = c + 0.5 * (simplex[-1] - c)
        fr, fe, fc = fmany([xr, xe, xc])  # the candidates of one step, concurrently
        if fr < fv[0]:
            simplex[-1], fv[-1] = (xe, fe) if fe < fr else (xr, fr)
        elif fr < fv[-2]:
            simplex[-1], fv[-1] = xr, fr
        elif fc < fv[-1]:
            simplex[-1], fv[-1] = xc, fc
        else:  # shrink towards the best vertex
            simplex = [simplex[0]] + [simplex[0] + 0.5 * (x - simplex[0]) for x in simplex[1:]]
            fv = [fv[0]] + list(fmany(simplex[1:]))
    k = int(np.argmin(fv))
    hist.append(fv[k])
    return simplex[k], fv[k], hist
