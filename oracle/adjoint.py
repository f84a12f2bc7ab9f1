"""Float64 NumPy restatement of the reverse-mode pieces (test infrastructure).

Only ``tests/`` uses this module: it checks ``csrc/mpm_adjoint.cu``, never
stands in for it.  ``return_map_vjp`` is the vector-Jacobian product of the
sand return map + Drucker-Prager stress (engine_stress/mpm_utils.py:87-112,
:45-52, as restated in ``mpm_numpy.return_map_and_stress``) written in the
singular frames -- the same formulation as the CUDA kernel, but with the
principal-space Jacobians taken by central differences in float64 instead
of dual numbers, and LAPACK's SVD instead of the Jacobi SVD.
"""
from __future__ import annotations

import numpy as np

from . import mpm_numpy as NP


def principal(s, mu, lam, alpha):
    """Sand return map in principal space: (regime, g (3), t (3))."""
    e = np.log(np.maximum(np.abs(s), 1e-14))
    tr = e.sum()
    h = e - tr / 3.0
    hn = np.sqrt((h * h).sum())
    dg = hn + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha
    if dg <= 0:
        return 0, s.copy(), 2 * mu * e + lam * tr, 1.0
    if tr > 0:
        return 1, np.ones(3), np.zeros(3), 0.0
    r = dg / hn
    ep = e - h * r
    return 2, np.exp(ep), 2 * mu * ep + lam * ep.sum(), 1.0 - r


def _jac(s, th, eps=1e-7):
    """d(g, t)/d(s, mu, lam, alpha) by central differences (float64)."""
    x0 = np.concatenate([s, th])
    J = np.zeros((6, 6))
    for k in range(6):
        step = eps * max(abs(x0[k]), 1.0)
        xp, xm = x0.copy(), x0.copy()
        xp[k] += step
        xm[k] -= step
        _, gp, tp, _ = principal(xp[:3], *xp[3:])
        _, gm, tm, _ = principal(xm[:3], *xm[3:])
        J[:, k] = (np.concatenate([gp, tp]) - np.concatenate([gm, tm])) / (2 * step)
    return J


def return_map_vjp(F_trial, F_bar, tau_bar, mu, lam, alpha):
    """Per row: adjoint of F_trial (n, 9) and the summed (mu, lam, alpha) adjoints."""
    n = F_trial.shape[0]
    U, s, V = NP.svd_rot(F_trial.reshape(n, 3, 3).astype(np.float64))
    s = np.abs(s)
    out = np.zeros((n, 9))
    thb = np.zeros(3)
    th = np.array([mu, lam, alpha], dtype=np.float64)
    for p in range(n):
        reg, g, t, k = principal(s[p], mu, lam, alpha)
        J = _jac(s[p], th)
        Ab = U[p].T @ F_bar[p].reshape(3, 3) @ V[p]
        Tb = U[p].T @ tau_bar[p].reshape(3, 3) @ U[p]
        Pb = np.zeros((3, 3))
        da, dt_ = np.diag(Ab), np.diag(Tb)
        for m in range(3):
            Pb[m, m] = da @ J[:3, m] + dt_ @ J[3:, m]
        thb += da @ J[:3, 3:] + dt_ @ J[3:, 3:]
        for i in range(3):
            for j in range(3):
                if i == j:
                    continue
                si, sj = s[p, i], s[p, j]
                if abs(si - sj) > 1e-6 * sj:
                    Dg = (g[i] - g[j]) / (si - sj)
                    Dt = (t[i] - t[j]) / (si - sj)
                else:  # the limits of the divided differences
                    L = 1.0 / sj
                    Dg = {0: 1.0, 1: 0.0, 2: g[j] * k * L}[reg]
                    Dt = {0: 2 * mu * L, 1: 0.0, 2: 2 * mu * k * L}[reg]
                avg = (g[i] + g[j]) / (si + sj)
                a, b = 0.5 * (Dg + avg), 0.5 * (Dg - avg)
                Pb[i, j] = a * Ab[i, j] + b * Ab[j, i] + (Tb[i, j] + Tb[j, i]) * Dt * sj / (si + sj)
        out[p] = (U[p] @ Pb @ V[p].T).ravel()
    return out, thb


def return_map_fd(F_trial, F_bar, tau_bar, mu, lam, alpha, h=1e-6):
    """The same products by central differences of the float64 return map
    (directional derivative along each input coordinate)."""
    n = F_trial.shape[0]

    def J(F, m, l, a):
        Fn, tau, _ = NP.return_map_and_stress(F, 2, m, l, a)
        return (Fn * F_bar).sum(axis=1) + (tau * tau_bar).sum(axis=1)

    out = np.zeros((n, 9))
    for q in range(9):
        d = np.zeros_like(F_trial)
        d[:, q] = h
        out[:, q] = (J(F_trial + d, mu, lam, alpha) - J(F_trial - d, mu, lam, alpha)) / (2 * h)
    thb = np.zeros(3)
    for q, base in enumerate((mu, lam, alpha)):
        hh = h * base
        args_p = [mu, lam, alpha]
        args_m = [mu, lam, alpha]
        args_p[q] += hh
        args_m[q] -= hh
        thb[q] = ((J(F_trial, *args_p) - J(F_trial, *args_m)) / (2 * hh)).sum()
    return out, thb
