"""Independent NumPy (float64, LAPACK SVD) restatement of the MPM substep.

Test infrastructure only.  It pins the C oracle (``mpm_oracle.c``): the two
are written separately -- this one vectorised over particles, with
``np.add.at`` scatters and ``np.linalg.svd`` converted to the rotation
convention (U, V proper rotations, det sign on the last singular value) --
and must agree to float64 rounding on small cases.

Follows engine_stress/mpm_utils.py:29-112 (stress, return maps), :318-413 (reduced P2G),
:190-237 (P2G, grid update), :241-306 (G2P) and
engine_stress/mpm_solver_warp.py:156-199 (order), :429-449, :505-523 (BCs).
"""
from __future__ import annotations

import numpy as np


def svd_rot(F: np.ndarray):
    """SVD with U, V in SO(3), |s| descending, sign(det F) on s[:, 2]."""
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    U = U.copy()
    s = s.copy()
    du = np.linalg.det(U) < 0
    U[du, :, 2] *= -1
    s[du, 2] *= -1
    dv = np.linalg.det(V) < 0
    V[dv, :, 2] *= -1
    s[dv, 2] *= -1
    return U, s, V


def _udvt(U, d, V):
    return np.einsum("nij,nj,nkj->nik", U, d, V)


def return_map_and_stress(F_trial, material, mu, lam, alpha, yield_stress=None, hardening=0,
                          xi=0.0):
    """mpm_utils.py:59-112 + :284-306 (two SVDs, as the reference)."""
    n = F_trial.shape[0]
    Ft = F_trial.reshape(n, 3, 3)
    Fn = Ft.copy()
    ys = None if yield_stress is None else np.array(yield_stress, dtype=np.float64, copy=True)
    if material == 2:
        U, sig, V = svd_rot(Ft)
        eps = np.log(np.maximum(np.abs(sig), 1e-14))
        tr = eps.sum(1)
        eh = eps - tr[:, None] / 3
        ehn = np.linalg.norm(eh, axis=1)
        dg = ehn + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha
        plast = dg > 0
        m1 = plast & (tr > 0)
        m2 = plast & (tr <= 0)
        Fn[m1] = np.einsum("nij,nkj->nik", U[m1], V[m1])
        if m2.any():
            H = eps[m2] - eh[m2] * (dg[m2] / ehn[m2])[:, None]
            Fn[m2] = _udvt(U[m2], np.exp(H), V[m2])
    elif material == 1:
        U, sig0, V = svd_rot(Ft)
        sig = np.maximum(sig0, 0.01)
        eps = np.log(sig)
        temp = eps.sum(1) / 3
        tau = 2 * mu * eps + lam * eps.sum(1)[:, None]
        cond = tau - tau.sum(1)[:, None] / 3
        pl = np.linalg.norm(cond, axis=1) > ys
        eh = eps - temp[:, None]
        ehn = np.linalg.norm(eh, axis=1) + 1e-6
        dg = ehn - ys / (2 * mu)
        e2 = eps - (dg / ehn)[:, None] * eh
        Fn[pl] = _udvt(U[pl], np.exp(e2[pl]), V[pl])
        if hardening == 1:
            ys = np.where(pl, ys + 2 * mu * xi * dg, ys)
    U, sig, V = svd_rot(Fn)
    if material == 0:
        J = np.linalg.det(Fn)
        R = np.einsum("nij,nkj->nik", U, V)
        tau = 2 * mu * np.einsum("nij,nkj->nik", Fn - R, Fn) + (lam * J * (J - 1))[:, None, None] * np.eye(3)
    elif material == 1:
        s = np.maximum(sig, 0.01)
        le = np.log(s)
        t = 2 * mu * le + lam * le.sum(1)[:, None]
        tau = _udvt(U, t, V)
    else:
        le = np.log(sig)
        c = (2 * mu * le + lam * le.sum(1)[:, None]) / sig
        tau = np.einsum("nij,nkj->nik", _udvt(U, c, V), Fn)
    return Fn.reshape(n, 9), tau.reshape(n, 9), ys


def _stencil(x, inv_dx):
    gp = x * inv_dx
    base = np.trunc(gp - 0.5).astype(np.int64)
    fx = gp - base
    w = np.stack([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2], axis=-1)
    dw = np.stack([fx - 1.5, -2.0 * (fx - 1.0), fx - 0.5], axis=-1)
    return base, fx, w, dw  # w[p, d, i]


def p2g2p(state: dict, n_grid: int, dx: float, dt: float, material: int, mu: float, lam: float,
          alpha: float, gravity, colliders=(), time: float = 0.0, hardening=0, xi=0.0):
    """One substep on float64 arrays in ``state`` (keys x0,u,v,C,F,stress,mass,vol,yield).

    Returns the grid (m, v_in, v_out) for per-stage comparison; updates state.
    """
    inv_dx = 1.0 / dx
    n = n_grid
    x = state["x0"] + state["u"]
    v, Cm, F, tau = state["v"], state["C"].reshape(-1, 3, 3), state["F"].reshape(-1, 3, 3), state["stress"].reshape(-1, 3, 3)
    mass, vol = state["mass"], state["vol"]
    base, fx, w, dw = _stencil(x, inv_dx)
    gm = np.zeros(n ** 3)
    gp = np.zeros((n ** 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                off = np.array([i, j, k], dtype=np.float64)
                dpos = (off[None] - fx) * dx
                wt = w[:, 0, i] * w[:, 1, j] * w[:, 2, k]
                dwt = np.stack([dw[:, 0, i] * w[:, 1, j] * w[:, 2, k],
                                w[:, 0, i] * dw[:, 1, j] * w[:, 2, k],
                                w[:, 0, i] * w[:, 1, j] * dw[:, 2, k]], axis=1) * inv_dx
                idx = ((base[:, 0] + i) * n + base[:, 1] + j) * n + base[:, 2] + k
                mom = (wt * mass)[:, None] * (v + np.einsum("nij,nj->ni", Cm, dpos))
                force = np.einsum("nij,nj->ni", -vol[:, None, None] * tau, dwt) * dt
                np.add.at(gp, idx, mom + force)
                np.add.at(gm, idx, wt * mass)
    gv = np.zeros_like(gp)
    act = gm > 1e-15
    gv[act] = gp[act] / gm[act, None] + dt * np.asarray(gravity)[None]
    ii = np.arange(n)
    IX, IY, IZ = np.meshgrid(ii, ii, ii, indexing="ij")
    pos = np.stack([IX.ravel(), IY.ravel(), IZ.ravel()], axis=1)
    for col in colliders:
        if not (time >= col["start_time"] and time < col["end_time"]):
            continue
        if col["kind"] == 0:
            off = pos * dx - np.asarray(col["point"])[None]
            gv[(off @ np.asarray(col["normal"])) < 0] = 0
        else:
            for c in range(3):
                lo = (pos[:, c] < 3) & (gv[:, c] < 0)
                hi = (pos[:, c] >= n - 3) & (gv[:, c] > 0)
                gv[lo | hi, c] = 0
    nv = np.zeros((x.shape[0], 3))
    nC = np.zeros((x.shape[0], 3, 3))
    nF = np.zeros((x.shape[0], 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                off = np.array([i, j, k], dtype=np.float64)
                dpos = off[None] - fx
                wt = w[:, 0, i] * w[:, 1, j] * w[:, 2, k]
                dwt = np.stack([dw[:, 0, i] * w[:, 1, j] * w[:, 2, k],
                                w[:, 0, i] * dw[:, 1, j] * w[:, 2, k],
                                w[:, 0, i] * w[:, 1, j] * dw[:, 2, k]], axis=1) * inv_dx
                idx = ((base[:, 0] + i) * n + base[:, 1] + j) * n + base[:, 2] + k
                g = gv[idx]
                nv += g * wt[:, None]
                nC += np.einsum("ni,nj->nij", g, dpos) * (wt * inv_dx * 4.0)[:, None, None]
                nF += np.einsum("ni,nj->nij", g, dwt)
    xn = x + dt * nv
    Ftr = np.einsum("nij,njk->nik", np.eye(3)[None] + nF * dt, F)
    Fn, taun, ys = return_map_and_stress(Ftr.reshape(-1, 9), material, mu, lam, alpha,
                                         state.get("yield"), hardening, xi)
    state["v"] = nv
    state["C"] = nC.reshape(-1, 9)
    state["F"] = Fn
    state["stress"] = taun
    if ys is not None:
        state["yield"] = ys
    state["u"] = xn - state["x0"]
    return gm.reshape(n, n, n), gp.reshape(n, n, n, 3), gv.reshape(n, n, n, 3)


def p2g2p_reduced(state: dict, n_grid: int, dx: float, dt: float, material: int, mu: float, lam: float,
                  gravity, sample, density):
    """The reduced sampled-quadrature substep without colliders, float64
    (mpm_solver_warp.py:214-227; mpm_utils.py:318-335, :353-413).  Sets
    state["F"] = F_disp + I on the marked particles; returns (marks, m, v_in, v_out)."""
    inv_dx = 1.0 / dx
    n = n_grid
    x = state["x0"] + state["u"]
    base, fx, w, dw = _stencil(x, inv_dx)
    mask = np.zeros((n, n, n), np.int32)
    offs = np.arange(-2, 3)
    for p in np.asarray(sample):
        b = base[p]
        ix, iy, iz = (b[d] + offs for d in range(3))
        ix, iy, iz = ix[(ix >= 0) & (ix < n)], iy[(iy >= 0) & (iy < n)], iz[(iz >= 0) & (iz < n)]
        mask[np.ix_(ix, iy, iz)] = 1
    sel = mask[base[:, 0], base[:, 1], base[:, 2]] > 0
    F = state["F"].reshape(-1, 3, 3)
    F[sel] = state["F_disp"].reshape(-1, 3, 3)[sel] + np.eye(3)[None]
    Fs = F[sel]
    U, s, V = svd_rot(Fs)
    if material == 2:
        ls = np.log(s).sum(1, keepdims=True)
        c = (2.0 * mu * np.log(s) + lam * ls) / s
        tau = np.einsum("nij,nkj->nik", _udvt(U, c, V), Fs)
    else:
        J = np.prod(s, axis=1)
        R = np.einsum("nij,nkj->nik", U, V)
        tau = 2.0 * mu * np.einsum("nij,nkj->nik", Fs - R, Fs) + (lam * J * (J - 1.0))[:, None, None] * np.eye(3)
    m = state["mass"][sel]
    tau = -(m / np.asarray(density)[sel])[:, None, None] * tau
    v = state["v"][sel]
    b, fxs, ws, dws = base[sel], fx[sel], w[sel], dw[sel]
    gm = np.zeros(n ** 3)
    gp = np.zeros((n ** 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                wt = ws[:, 0, i] * ws[:, 1, j] * ws[:, 2, k]
                dwt = np.stack([dws[:, 0, i] * ws[:, 1, j] * ws[:, 2, k],
                                ws[:, 0, i] * dws[:, 1, j] * ws[:, 2, k],
                                ws[:, 0, i] * ws[:, 1, j] * dws[:, 2, k]], axis=1) * inv_dx
                idx = ((b[:, 0] + i) * n + b[:, 1] + j) * n + b[:, 2] + k
                np.add.at(gp, idx, (wt * m)[:, None] * v + dt * np.einsum("nij,nj->ni", tau, dwt))
                np.add.at(gm, idx, wt * m)
    gv = np.zeros_like(gp)
    act = (mask.ravel() > 0) & (gm > 1e-10)
    gv[act] = gp[act] / gm[act, None] + dt * np.asarray(gravity)[None]
    return mask, gm.reshape(n, n, n), gp.reshape(n, n, n, 3), gv.reshape(n, n, n, 3)
