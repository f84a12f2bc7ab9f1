"""Hand-written adjoint (csrc/mpm_adjoint.cu) on the GPU: the return-map
vector-Jacobian product against the float64 oracle (oracle/adjoint.py), and
rollout gradients w.r.t. Young's modulus, friction angle and the initial
velocity against central finite differences of the forward rollout."""
import math

import numpy as np
import pytest
import torch

from oracle import adjoint as AD
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300 import surrogate as SU
from reduced_mpm_stress_training_gb300.adjoint import SandRollout, rollout

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_return_map_vjp_matches_oracle(cuda):
    rng = np.random.default_rng(0)
    n = 3000
    F = SU.synthetic_F(n, rng, max_log=0.05)
    E, nu, phi = 2e5, 0.3, 30.0
    mu, lam = E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)
    s = math.sin(phi / 180 * 3.14159265)
    alpha = math.sqrt(2 / 3) * 2 * s / (3 - s)
    Fb = rng.standard_normal((n, 9)).astype(np.float32)
    Tb = (rng.standard_normal((n, 9)) / mu).astype(np.float32)
    sc = SU.sand_scene(E, nu, phi)
    dF = torch.from_numpy(F).to(cuda)
    dFb = torch.from_numpy(Fb).to(cuda)
    dTb = torch.from_numpy(Tb).to(cuda)
    out = torch.empty_like(dF)
    th = torch.zeros(3, dtype=torch.float64, device=cuda)
    A.check(A.load().mpm_return_map_vjp(A.C.byref(sc), dF.data_ptr(), dFb.data_ptr(), dTb.data_ptr(),
                                        out.data_ptr(), th.data_ptr(), n,
                                        torch.cuda.current_stream().cuda_stream), "vjp")
    g_ref, th_ref = AD.return_map_vjp(F.astype(np.float64), Fb.astype(np.float64), Tb.astype(np.float64),
                                      mu, lam, alpha)
    e = rel(out.cpu().numpy(), g_ref)
    print("F_trial adjoint rel", e, "theta", th.cpu().numpy(), th_ref)
    assert e < 1e-3
    assert rel(th.cpu().numpy() * [mu, lam, alpha], th_ref * [mu, lam, alpha]) < 1e-3


def _prestrained(n, rng, cuda, E=2e5, nu=0.3, phi=30.0, stretches=(0.97, 0.976, 0.982)):
    """F = R diag(stretches) R^T (a compressed start clear of the return map's
    switching points at F = I): (F, returned F, stress of the return map)."""
    R = SU.haar_rotations(n, rng)
    s = np.array(stretches)
    F = torch.from_numpy(((R * s[None, None, :]) @ R.transpose(0, 2, 1)).reshape(n, 9).astype(np.float32)).to(cuda)
    Fo = torch.empty_like(F)
    tau = torch.empty_like(F)
    sc = SU.sand_scene(E, nu, phi)
    A.check(A.load().mpm_return_map(A.C.byref(sc), F.data_ptr(), None, Fo.data_ptr(), tau.data_ptr(), n,
                                    torch.cuda.current_stream().cuda_stream), "return_map")
    return F, Fo, tau


def test_adjoint_matches_central_differences_on_a_deterministic_block(cuda):
    """64 particles, one per cell of one 4x4x4 block of a 32^3 grid: one warp
    owns every P2G contribution and every cell holds one particle, so the
    forward is deterministic and central differences resolve every input's
    adjoint (initial x, v, C, F, stress, E, friction angle) over 6 substeps
    (checkpoints every 2)."""
    rng = np.random.default_rng(4)
    n, dx = 64, 1.0 / 32
    cells = np.stack(np.meshgrid(*(np.arange(12, 16),) * 3, indexing="ij"), -1).reshape(-1, 3)
    x0 = ((cells + 0.75 + rng.uniform(-0.1, 0.1, (n, 3))) * dx).astype(np.float32)
    v0 = rng.normal(0.0, 0.1, (n, 3)).astype(np.float32)
    vol = np.full(n, dx ** 3, np.float32)
    mass = (2200.0 * vol).astype(np.float32)
    sc = S.Scene("block_64", n, 32, 1.0, (0.375, 0.375, 0.375), (0.5, 0.5, 0.5), "sand", 2e5, 0.3, 30.0,
                 2200.0, (0.0, 0.0, -9.8), 1e-4, 6, floor_z=None)
    # sheared past the Drucker-Prager cone (|h| exceeds the yield value by about
    # 0.008): every substep is a plastic step with margin, so the friction
    # angle matters and no particle switches regime
    F0, _, tau0 = _prestrained(n, rng, cuda, stretches=(0.97, 1.0, 1.01))
    C0 = torch.from_numpy(rng.normal(0.0, 1.0, (n, 9)).astype(np.float32)).to(cuda)
    base = {A.FIELD_U: torch.zeros(n, 3, device=cuda), A.FIELD_C: C0, A.FIELD_F: F0, A.FIELD_STRESS: tau0}
    sand = SandRollout(sc, checkpoint_every=2, device=cuda, particles=(x0, v0, vol, mass), initial=base)
    mu = sand.params.mu
    g = torch.Generator(device=cuda).manual_seed(2)
    W = torch.randn(n, A.ADJ_WORDS, generator=g, device=cuda, dtype=torch.float64)
    W[:, A.ADJ_STRESS:A.ADJ_STRESS + 9] /= mu
    W[:, 33:] = 0.0
    fields = [(A.FIELD_U, A.ADJ_X, 3), (A.FIELD_V, A.ADJ_V, 3), (A.FIELD_C, A.ADJ_C, 9),
              (A.FIELD_F, A.ADJ_F, 9), (A.FIELD_STRESS, A.ADJ_STRESS, 9)]
    e = sand.engine

    def J(v, E, phi):
        sand.forward(v, E, phi, keep=False)
        tot = 0.0
        for f, off, c in fields:
            tot += float((e.export(f).reshape(n, c).double() * W[:, off:off + c]).sum())
        return tot

    v0t = torch.from_numpy(v0).to(cuda)
    sand.forward(v0t, sc.E, sc.friction_angle)
    _, Eb, phib = sand.backward(W)
    sb = sand.state_bar.double()
    # steps large enough that the change of J stands well above its float32
    # rounding, small enough to stay in the linear regime
    scale = {A.FIELD_U: 1e-4, A.FIELD_V: 1e-2, A.FIELD_C: 1e-1, A.FIELD_F: 1e-4, A.FIELD_STRESS: mu * 1e-3}
    res = {}
    for f, off, c in fields:
        d = torch.randn(n, c, generator=g, device=cuda, dtype=torch.float64) * scale[f]
        if f == A.FIELD_V:
            fd = (J(v0t.double() + d, sc.E, sc.friction_angle) - J(v0t.double() - d, sc.E, sc.friction_angle)) / 2
        else:
            keep = sand.initial[f].clone()
            sand.initial[f] = (keep.double() + d).float()
            jp = J(v0t, sc.E, sc.friction_angle)
            sand.initial[f] = (keep.double() - d).float()
            jm = J(v0t, sc.E, sc.friction_angle)
            sand.initial[f] = keep
            fd = (jp - jm) / 2
        ad = float((sb[:, off:off + c] * d).sum())
        res[f] = (ad, fd, abs(ad - fd) / abs(fd))
    h = 1e-2
    fdE = (J(v0t, sc.E * (1 + h), sc.friction_angle) - J(v0t, sc.E * (1 - h), sc.friction_angle)) / (2 * h * sc.E)
    fdP = (J(v0t, sc.E, sc.friction_angle * (1 + h)) - J(v0t, sc.E, sc.friction_angle * (1 - h))) / (
        2 * h * sc.friction_angle)
    res["E"] = (Eb, fdE, abs(Eb - fdE) / abs(fdE))
    res["phi"] = (phib, fdP, abs(phib - fdP) / max(abs(fdP), 1e-300))
    print(res)
    for k, (ad, fd, err) in res.items():
        assert err < 5e-3, (k, ad, fd, err)


def _scene(n=8000, steps=50):
    sc = S.small_column(n, 32, seed=11, floor_z=0.15, v0_sigma=0.1)
    sc.substeps = steps
    return sc


def _loss_fn(sand, target):
    def J(v0, E, phi):
        x = sand.positions(sand.forward(v0, E, phi, keep=False))
        return float(((x - target) ** 2).mean())
    return J


@pytest.fixture(scope="module")
def setup(cuda):
    sc = _scene()
    rng = np.random.default_rng(7)
    _, F0, tau0 = _prestrained(sc.n_particles, rng, cuda)
    sand = SandRollout(sc, checkpoint_every=10, device=cuda, initial={A.FIELD_F: F0, A.FIELD_STRESS: tau0})
    target = sand.positions(sand.forward(sand.v0_default, 3e5, 35.0, keep=False)).clone()
    return sc, sand, target


def test_rollout_gradients_match_central_differences(cuda, setup):
    """8000 prestrained sand particles, 50 substeps: P2G's float atomics make
    each forward differ at rounding level and the return map switches regime
    for some particles, so the differences use 1e-2 relative steps and the
    tolerance is 5e-2 (the deterministic block above checks to 3e-3)."""
    sc, sand, target = setup
    v0 = sand.v0_default.clone()
    E, phi = sc.E, sc.friction_angle
    x = sand.positions(sand.forward(v0, E, phi))
    xb = 2.0 * (x - target) / x.numel()
    v0b, Eb, phib = sand.backward(xb)
    J = _loss_fn(sand, target)
    rh = 1e-2
    res = {"E": (Eb, (J(v0, E * (1 + rh), phi) - J(v0, E * (1 - rh), phi)) / (2 * rh * E)),
           "phi": (phib, (J(v0, E, phi * (1 + rh)) - J(v0, E, phi * (1 - rh))) / (2 * rh * phi))}
    g = torch.Generator(device=cuda).manual_seed(0)
    for d in range(4):
        dirn = torch.randn(v0.shape, generator=g, device=cuda)
        dirn /= dirn.norm()
        h = rh * v0.norm().item()
        fd = (J(v0 + h * dirn, E, phi) - J(v0 - h * dirn, E, phi)) / (2 * h)
        res[f"v0_dir{d}"] = (float((v0b.double() * dirn.double()).sum()), fd)
    print({k: (a, f, abs(a - f) / abs(f)) for k, (a, f) in res.items()})
    for name, (ad, fd) in res.items():
        assert abs(ad - fd) <= 5e-2 * abs(fd), (name, ad, fd)


def test_checkpoint_interval_does_not_change_gradients(cuda, setup):
    sc, sand, target = setup
    v0 = sand.v0_default
    grads = []
    for k in (1, 10, 50):
        sand.k = k
        x = sand.positions(sand.forward(v0, sc.E, sc.friction_angle))
        grads.append(sand.backward(2.0 * (x - target) / x.numel()))
    sand.k = 10
    # recomputed trajectories differ at rounding level (P2G atomics)
    for g in grads[1:]:
        assert rel(g[0].cpu().numpy(), grads[0][0].cpu().numpy()) < 5e-3
        assert abs(g[1] - grads[0][1]) <= 5e-3 * abs(grads[0][1])
        assert abs(g[2] - grads[0][2]) <= 5e-3 * abs(grads[0][2])


def test_grid_tape_matches_recompute(cuda, setup):
    """The grid tape (states rebuilt by G2P from the forward's saved grids)
    and whole-substep recompute give the same gradients up to the rounding
    differences of separate forward runs."""
    sc, sand, target = setup
    assert sand.grid_tape
    plain = SandRollout(sc, checkpoint_every=10, device=cuda, initial=sand.initial, grid_tape=False)
    v0 = sand.v0_default
    grads = []
    for r in (sand, plain):
        x = r.positions(r.forward(v0, sc.E, sc.friction_angle))
        grads.append(r.backward(2.0 * (x - target) / x.numel()))
    assert rel(grads[1][0].cpu().numpy(), grads[0][0].cpu().numpy()) < 5e-3
    assert abs(grads[1][1] - grads[0][1]) <= 5e-3 * abs(grads[0][1])
    assert abs(grads[1][2] - grads[0][2]) <= 5e-3 * abs(grads[0][2])


def test_autograd_function(cuda, setup):
    sc, sand, target = setup
    v0 = sand.v0_default.clone().requires_grad_(True)
    E = torch.tensor(sc.E, dtype=torch.float64, requires_grad=True)
    phi = torch.tensor(sc.friction_angle, dtype=torch.float64, requires_grad=True)
    x = rollout(v0, E, phi, sand)
    loss = ((x - target) ** 2).mean()
    loss.backward()
    x2 = sand.positions(sand.forward(v0.detach(), sc.E, sc.friction_angle))
    v0b, Eb, phib = sand.backward(2.0 * (x2 - target) / x2.numel())
    assert rel(v0.grad.cpu().numpy(), v0b.cpu().numpy()) < 5e-3
    assert abs(E.grad.item() - Eb) <= 5e-3 * abs(Eb)
    assert abs(phi.grad.item() - phib) <= 5e-3 * abs(phib)
