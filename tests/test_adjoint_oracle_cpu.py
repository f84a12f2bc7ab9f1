"""The return-map adjoint's formulation (singular-frame VJP with closed-form
divided differences, oracle/adjoint.py) against central differences of the
float64 return map of oracle/mpm_numpy.py, on the CPU: elastic, cone and
apex particles, and nearly equal singular values."""
import math

import numpy as np

from oracle import adjoint as AD


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


def _check(F, rng, tol=2e-5):
    mu, lam, alpha = _material()
    n = F.shape[0]
    Fb = rng.standard_normal((n, 9))
    Tb = rng.standard_normal((n, 9)) / mu
    g, th = AD.return_map_vjp(F, Fb, Tb, mu, lam, alpha)
    gf, thf = AD.return_map_fd(F, Fb, Tb, mu, lam, alpha)
    err = np.linalg.norm(g - gf) / np.linalg.norm(gf)
    assert err < tol, err
    scale = np.array([mu, lam, alpha])
    assert np.allclose(th * scale, thf * scale, rtol=1e-4, atol=1e-6 * np.abs(thf * scale).max()), (th, thf)


def _trial(n, rng, s):
    return ((_haar(n, rng) * np.exp(s)[:, None, :]) @ _haar(n, rng).transpose(0, 2, 1)).reshape(n, 9)


def test_vjp_matches_finite_differences_in_every_regime():
    rng = np.random.default_rng(0)
    mu, lam, alpha = _material()
    s = rng.uniform(-0.05, 0.05, size=(300, 3))
    F = _trial(300, rng, s)
    regimes = [AD.principal(np.linalg.svd(f.reshape(3, 3), compute_uv=False), mu, lam, alpha)[0] for f in F]
    assert {0, 1, 2} <= set(regimes)
    _check(F, rng)


def test_vjp_with_nearly_equal_singular_values():
    rng = np.random.default_rng(1)
    base = rng.uniform(-0.02, 0.0, size=(200, 1))
    s = base + rng.uniform(-1e-7, 1e-7, size=(200, 3))  # two or three almost equal
    s[:100, 0] += 0.01  # one separated value, the other two close
    _check(_trial(200, rng, s), rng, tol=1e-4)
