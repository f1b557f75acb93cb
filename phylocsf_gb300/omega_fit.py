"""Gradient MAP fit of the OmegaModel tree scale and kappa (and optionally omega), beside
the reference's Brent coordinate ascent (kr_map, src/OmegaModel.ml:160-190).

The objective is the one kr_map maximises, F(rho, kappa) = lpr(rho, kappa) +
log p(rho) + log p(kappa) with the half-Cauchy prior on rho (OmegaModel.ml:148-156) and
the Gamma(7, 0.25) prior on kappa - 1 (OmegaModel.ml:157), over rho in [0.001, 10],
kappa in [1, 10]; with fit_omega, omega in [0.001, 10] is a third free parameter
(no prior: its maximum-likelihood estimate given the other two).  Every iteration is
one batched pcsf_omega_grad call for all regions (lpr and d lpr / d {rho, kappa, omega}
from the adjoint pass); the step is a projected quasi-Newton step in log-parameters with
a per-region BFGS estimate of the Hessian and a backtracking line search.
"""
from __future__ import annotations

import math

import numpy as np

RHO_BOUNDS = (1e-3, 10.0)
KAPPA_BOUNDS = (1.0, 10.0)
OMEGA_BOUNDS = (1e-3, 10.0)


def log_prior_rho(x):
    mode, scale = 1.0, 0.5
    z = (x - mode) / scale
    cdf = math.atan((0.0 - mode) / scale) / math.pi + 0.5
    return np.log(1.0 / (math.pi * scale * (1.0 + z * z))) - math.log(1.0 - cdf)


def dlog_prior_rho(x):
    mode, scale = 1.0, 0.5
    z = (x - mode) / scale
    return -2.0 * z / (scale * (1.0 + z * z))


def log_prior_kappa(k):
    y = k - 1.0 + 2.220446049250313e-16
    a, b = 7.0, 0.25
    with np.errstate(divide="ignore"):
        return np.where(y > 0, (a - 1.0) * np.log(np.maximum(y, 1e-300)) - y / b - math.lgamma(a) - a * math.log(b),
                        -np.inf)


def dlog_prior_kappa(k):
    y = np.maximum(k - 1.0 + 2.220446049250313e-16, 1e-300)
    return (7.0 - 1.0) / y - 1.0 / 0.25


def _objective(engine, batch, x, omega, sigma, fit_omega):
    """F and its gradient in log-parameters x = log [rho, kappa(, omega)] for every region."""
    rho, kappa = np.exp(x[:, 0]), np.exp(x[:, 1])
    om = np.exp(x[:, 2]) if fit_omega else omega
    g = engine.omega_grad(batch, kappa, om, rho, sigma, branches=False)
    f = g["lpr"] + log_prior_rho(rho) + log_prior_kappa(kappa)
    # gradient in log-parameters (the bounds are multiplicative ranges)
    cols = [(g["d_rho"] + dlog_prior_rho(rho)) * rho, (g["d_kappa"] + dlog_prior_kappa(kappa)) * kappa]
    if fit_omega:
        cols.append(g["d_omega"] * om)
    return f, np.stack(cols, axis=1), g["status"]


def gradient_map(engine, batch, omega=1.0, sigma: float = 1.0, rho0: float = 1.0, kappa0: float = 2.5,
                 iters: int = 40, gtol: float = 1e-6, fit_omega: bool = False, omega0: float = 1.0):
    """Per-region MAP (rho, kappa), or (rho, kappa, omega) with fit_omega, by batched projected
    BFGS in log-parameters.

    Returns dict rho, kappa, omega, objective, evals (objective evaluations per region), status."""
    n = batch.n_regions
    D = 3 if fit_omega else 2
    bounds = [RHO_BOUNDS, KAPPA_BOUNDS, OMEGA_BOUNDS][:D]
    lo = np.log([b[0] for b in bounds])
    hi = np.log([b[1] for b in bounds])
    start = [rho0, max(kappa0, KAPPA_BOUNDS[0] * (1 + 1e-9)), omega0][:D]
    x = np.tile(np.log(start), (n, 1))
    f, g, st = _objective(engine, batch, x, omega, sigma, fit_omega)
    evals = np.ones(n, np.int64)
    # first step of length ~0.1 in log-parameters along the gradient
    Hinv = np.eye(D)[None, :, :] * (0.1 / np.maximum(np.linalg.norm(g, axis=1), 1e-12))[:, None, None]
    active = np.ones(n, bool)
    for _ in range(iters):
        # projected ascent direction; components pushing out of the box at a bound are dropped
        d = np.einsum("nij,nj->ni", Hinv, g)
        at_lo, at_hi = x <= lo + 1e-12, x >= hi - 1e-12
        d[(at_lo & (d < 0)) | (at_hi & (d > 0))] = 0.0
        pg = g.copy()
        pg[(at_lo & (pg < 0)) | (at_hi & (pg > 0))] = 0.0
        active &= np.abs(pg).max(axis=1) > gtol * np.maximum(1.0, np.abs(f))
        if not active.any():
            break
        step = np.ones(n)
        accepted = np.zeros(n, bool)
        xn, fn, gn = x.copy(), f.copy(), g.copy()
        for _ls in range(12):
            todo = active & ~accepted
            if not todo.any():
                break
            xt = np.clip(x + step[:, None] * d, lo, hi)
            ft, gt, stt = _objective(engine, batch, xt, omega, sigma, fit_omega)
            evals[todo] += 1
            ok = todo & (ft >= f + 1e-4 * np.einsum("ni,ni->n", g, xt - x)) & (stt == 0)
            xn[ok], fn[ok], gn[ok] = xt[ok], ft[ok], gt[ok]
            accepted |= ok
            step[todo & ~ok] *= 0.5
        # BFGS update of the inverse Hessian of -F for the regions that moved
        s = xn - x
        yv = -(gn - g)
        sy = np.einsum("ni,ni->n", s, yv)
        upd = accepted & (sy > 1e-12)
        for r in np.nonzero(upd)[0]:
            rho_ = 1.0 / sy[r]
            I = np.eye(D)
            V = I - rho_ * np.outer(s[r], yv[r])
            Hinv[r] = V @ Hinv[r] @ V.T + rho_ * np.outer(s[r], s[r])
        active &= accepted
        x, f, g = xn, fn, gn
    om = np.exp(x[:, 2]) if fit_omega else np.broadcast_to(np.asarray(omega, np.float64), (n,)).copy()
    return {"rho": np.exp(x[:, 0]), "kappa": np.exp(x[:, 1]), "omega": om, "objective": f, "evals": evals,
            "status": st, "gradient": g}
