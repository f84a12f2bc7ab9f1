"""Float64 NumPy restatement of the surrogate stress stage (test infrastructure).

Only ``tests/`` and ``bench.py``'s CPU legs use this module: it checks
``csrc/mpm_surrogate.cu`` given the same network outputs, never stands in
for it.  The exact quantities it relies on follow the reference's sand path
(sand_return_mapping, engine_stress/mpm_utils.py:87-112, and
kirchoff_stress_drucker_prager, :45-52): the return map keeps the trace of
the Hencky strain and scales its deviator, so the mean stress and the
deviatoric norm follow from the eigenvalues of F F^T alone.
"""
from __future__ import annotations

import numpy as np

ACC_ELASTIC, ACC_PLASTIC, FB_DOMAIN, FB_APEX, FB_STEP, FB_GATE, FB_MATERIAL = range(7)
SYM = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


def left_strain(F: np.ndarray) -> np.ndarray:
    """B = F F^T - I, (n, 3, 3)."""
    F = F.reshape(-1, 3, 3).astype(np.float64)
    return F @ F.transpose(0, 2, 1) - np.eye(3)


def nu_phi(mu: float, lam: float, alpha: float):
    nu = lam / (2.0 * (lam + mu))
    sphi = 3.0 * alpha / (2.0 * np.sqrt(2.0 / 3.0) + alpha)
    return nu, np.degrees(np.arcsin(np.clip(sphi, -1, 1)))


def features(F: np.ndarray, mu: float, lam: float, alpha: float) -> np.ndarray:
    """Network inputs (n, 12)."""
    B = left_strain(F)
    rho = np.sqrt((B * B).sum(axis=(1, 2)))
    nu, phi = nu_phi(mu, lam, alpha)
    x = np.empty((B.shape[0], 12))
    x[:, :9] = (B / np.maximum(rho, 1e-30)[:, None, None]).reshape(-1, 9)
    x[:, 9] = (np.log10(np.maximum(rho, 1e-30)) + 2.5) / 1.5
    x[:, 10] = (nu - 0.3) * 10.0
    x[:, 11] = (phi - 30.0) * 0.1
    return x


def targets(F: np.ndarray, stress: np.ndarray, mu: float) -> np.ndarray:
    """Network targets tau / (mu rho) as [xx, xy, xz, yy, yz, zz], (n, 6)."""
    B = left_strain(F)
    rho = np.sqrt((B * B).sum(axis=(1, 2)))
    t = stress.reshape(-1, 3, 3)
    y = np.stack([t[:, i, j] for i, j in SYM], axis=1)
    return y / (mu * np.maximum(rho, 1e-30))[:, None]


def _sym(v6):
    M = np.empty((3, 3))
    for k, (i, j) in enumerate(SYM):
        M[i, j] = M[j, i] = v6[k]
    return M


def _expm_sym(X):
    w, Q = np.linalg.eigh(X)
    return (Q * np.exp(w)) @ Q.T


def apply(F: np.ndarray, y: np.ndarray, mu: float, lam: float, alpha: float, cfg: dict):
    """Per row: (code, F_out, tau) from F_trial and the network output y.

    Rows that fall back get code only (F_out, tau = NaN): the SVD path that
    handles them is checked by the return-map tests.
    """
    n = F.shape[0]
    B = left_strain(F)
    nu, phi = nu_phi(mu, lam, alpha)
    codes = np.empty(n, np.int32)
    Fo = np.full((n, 9), np.nan)
    tau = np.full((n, 9), np.nan)
    domain_ok = (cfg["nu_min"] <= nu <= cfg["nu_max"]) and (cfg["phi_min"] <= phi <= cfg["phi_max"])
    for i in range(n):
        b = B[i]
        rho = np.sqrt((b * b).sum())
        if not (domain_ok and cfg["rho_min"] <= rho <= cfg["rho_max"]):
            codes[i] = FB_DOMAIN
            continue
        ev = np.linalg.eigvalsh(b)
        if ev.min() <= -0.9:
            codes[i] = FB_DOMAIN
            continue
        e = 0.5 * np.log1p(ev)
        tr = e.sum()
        h = e - tr / 3.0
        hn = np.sqrt((h * h).sum())
        dg = hn + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha
        if dg <= 0:
            code, dn = ACC_ELASTIC, 2 * mu * hn
        elif tr > 0:
            codes[i] = FB_APEX
            continue
        elif dg > cfg["dgamma_max"]:
            codes[i] = FB_STEP
            continue
        else:
            code, dn = ACC_PLASTIC, 2 * mu * (hn - dg)
        pm = (2 * mu + 3 * lam) * tr / 3.0
        T = _sym(y[i] * mu * rho)
        D = T - np.trace(T) / 3.0 * np.eye(3)
        dnorm = np.sqrt((D * D).sum())
        tcn = np.sqrt(3 * pm * pm + dn * dn)
        if not tcn > 0:
            codes[i] = FB_GATE
            continue
        w = dn / tcn
        if not dnorm > 1e-6 * tcn:
            if w > 1e-3:
                codes[i] = FB_GATE
                continue
            N = np.zeros((3, 3))
        else:
            N = D / dnorm
        Tc = pm * np.eye(3) + dn * N
        err = 0.0
        if w > 1e-4:
            Bd = b - np.trace(b) / 3.0 * np.eye(3)
            bn = np.sqrt((Bd * Bd).sum())
            if bn > 0:
                if not (N * Bd).sum() / bn >= 0.5:
                    codes[i] = FB_GATE
                    continue
                C = N @ Bd - Bd @ N
                evd = ev[::-1]  # largest first
                gap = max(min(evd[0] - evd[1], evd[1] - evd[2]) / bn, 0.2)
                err = max(err, w * np.sqrt((C * C).sum()) / bn / gap)
            k36 = 3.0 * np.sqrt(6.0)
            xn = np.clip(k36 * np.linalg.det(N), -1, 1)
            xe = np.clip(k36 * h.prod() / hn ** 3, -1, 1) if hn > 0 else 0.0
            err = max(err, w * abs(np.arccos(xn) - np.arccos(xe)) / 3.0)
        if not err <= cfg["tol"]:
            codes[i] = FB_GATE
            continue
        codes[i] = code
        tau[i] = Tc.ravel()
        Fi = F[i].reshape(3, 3).astype(np.float64)
        Fo[i] = (Fi if code == ACC_ELASTIC else _expm_sym(-dg * N) @ Fi).ravel()
    return codes, Fo, tau
