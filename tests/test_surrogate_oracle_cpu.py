"""The surrogate stage's exact-invariant correction on the CPU.

Fed with the exact normalised stress (what a perfect network would output),
the correction + gate + F update of oracle/surrogate.py must reproduce the
reference's SVD return map (restated in oracle/mpm_numpy.py, LAPACK SVD,
float64) for every particle it accepts, and must refuse apex projections.
This pins the algebra the CUDA stage (csrc/mpm_surrogate.cu) is built on:
trace-preserving Drucker-Prager projection, closed-form strain invariants,
and F = exp(-dgamma N) F_trial for the plastic update."""
import math

import numpy as np

from oracle import mpm_numpy as NP
from oracle import surrogate as SO

CFG = dict(tol=1e-2, rho_min=1e-6, rho_max=2.5, nu_min=0.25, nu_max=0.35, phi_min=20.0,
           phi_max=40.0, dgamma_max=0.25)


def _haar(n, rng):
    q, r = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    q = q * np.sign(np.diagonal(r, axis1=1, axis2=2))[:, None, :]
    q[np.linalg.det(q) < 0, :, 0] *= -1
    return q


def _material(E=2e5, nu=0.3, phi=30.0):
    mu = E / 2 / (1 + nu)
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    s = math.sin(phi / 180 * math.pi)
    return mu, lam, math.sqrt(2 / 3) * 2 * s / (3 - s)


def _trial(n, rng, scale):
    s = rng.uniform(-scale, scale, size=(n, 3))
    F = (_haar(n, rng) * np.exp(s)[:, None, :]) @ _haar(n, rng).transpose(0, 2, 1)
    return F.reshape(n, 9)


def test_exact_outputs_reproduce_the_svd_return_map():
    rng = np.random.default_rng(0)
    mu, lam, alpha = _material()
    F = _trial(4000, rng, 0.08)
    Fn, tau, _ = NP.return_map_and_stress(F, 2, mu, lam, alpha)
    y = SO.targets(F, tau, mu)
    codes, Fo, to = SO.apply(F, y, mu, lam, alpha, CFG)
    acc = (codes == SO.ACC_ELASTIC) | (codes == SO.ACC_PLASTIC)
    assert acc.sum() > 1000 and (codes == SO.ACC_PLASTIC).sum() > 200
    assert not np.any(codes == SO.FB_GATE)
    # the apex rows are refused, and only they (besides too large increments)
    assert set(np.unique(codes[~acc])) <= {SO.FB_APEX, SO.FB_STEP}
    dt = np.linalg.norm(to[acc] - tau[acc], axis=1) / np.linalg.norm(tau[acc], axis=1)
    dF = np.linalg.norm(Fo[acc] - Fn[acc], axis=1)
    assert dt.max() < 1e-9, dt.max()
    assert dF.max() < 1e-10, dF.max()


def test_gate_rejects_wrong_directions_and_magnitudes():
    rng = np.random.default_rng(1)
    mu, lam, alpha = _material(phi=35.0)
    F = _trial(500, rng, 0.05)
    Fn, tau, _ = NP.return_map_and_stress(F, 2, mu, lam, alpha)
    y = SO.targets(F, tau, mu)
    good, _, _ = SO.apply(F, y, mu, lam, alpha, CFG)
    # rotate the predicted stress by 0.1 rad: the deviator is no longer coaxial with F F^T
    R = _haar(1, rng)[0]
    th = 0.1
    K = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 0]])
    Rot = R @ (np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K) @ R.T
    t3 = tau.reshape(-1, 3, 3)
    tr = np.einsum("ij,njk,lk->nil", Rot, t3, Rot)
    y_rot = SO.targets(F, tr.reshape(-1, 9), mu)
    bad, _, _ = SO.apply(F, y_rot, mu, lam, alpha, CFG)
    ok = (good <= SO.ACC_PLASTIC)
    assert np.mean(bad[ok] == SO.FB_GATE) > 0.8
    # a deviator pointing against the strain deviator is refused outright
    t3n = tau.reshape(-1, 3, 3)
    p = np.trace(t3n, axis1=1, axis2=2)[:, None, None] / 3 * np.eye(3)
    flipped = (2 * p - t3n).reshape(-1, 9)
    bad2, _, _ = SO.apply(F, SO.targets(F, flipped, mu), mu, lam, alpha, CFG)
    dev_share = np.linalg.norm((t3n - p).reshape(-1, 9), axis=1) / np.maximum(np.linalg.norm(tau, axis=1), 1e-30)
    sel = ok & (dev_share > 1e-3)
    assert np.all(bad2[sel] == SO.FB_GATE)
    # the magnitudes are taken from the exact invariants: a uniformly scaled
    # prediction gives the same accepted stress
    sc, _, t_sc = SO.apply(F, y * 1.05, mu, lam, alpha, CFG)
    _, _, t_ok = SO.apply(F, y, mu, lam, alpha, CFG)
    assert np.array_equal(sc, good)
    assert np.allclose(t_sc[ok], t_ok[ok], rtol=1e-9, atol=1e-9 * np.abs(tau).max())


def test_domain_limits():
    mu, lam, alpha = _material(nu=0.45)
    F = np.tile(np.eye(3).ravel() * 1.001, (4, 1))
    codes, _, _ = SO.apply(F, np.zeros((4, 6)), mu, lam, alpha, CFG)
    assert np.all(codes == SO.FB_DOMAIN)
    mu, lam, alpha = _material()
    codes, _, _ = SO.apply(np.tile(np.eye(3).ravel(), (2, 1)), np.zeros((2, 6)), mu, lam, alpha, CFG)
    assert np.all(codes == SO.FB_DOMAIN)  # rho = 0 < rho_min
