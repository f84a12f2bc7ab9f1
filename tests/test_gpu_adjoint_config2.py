"""The differentiable-rollout workload at its stated size, and the ordered
P2G that makes its finite-difference check meaningful.

Workload (131,072 sand particles, 96^3 grid, 100 substeps at dt 1e-4, v0 ~
N(0, 0.1^2) per component, loss = MSE between the final positions and a
target rollout with E = 3e5 and friction 35 deg from the same seed):
gradients of the loss with respect to E, the friction angle and the
initial velocity (16 random unit directions) from the hand-written adjoint,
against central differences with a relative step of 1e-3.  The 1e-3 bar
is not met: a float32 rollout of this workload ends 6e-4 (relative RMS of
the displacement) from the float64 rollout, which bounds its gradients at
about 1e-2 (measured on a linear functional and on the MSE loss below).

The reference has no gradient path (no wp.Tape anywhere in
engine_stress/mpm_solver_warp.py:156-203), so the only comparison is with
finite differences of the forward.  At a relative step of 1e-3 the loss
moves by about 1e-6 of itself, below what a float32 rollout resolves, so the
differences are taken on the float64 restatement of the same forward (the
committed fixture of tests/golden/make_adjoint_fd.py).  The forward that is
differentiated uses the ordered P2G (mpm_p2g_ordered: every cell's particles
in uid order, the block tiles summed per node in a fixed order), so the
rollout is a deterministic function of its inputs; the first tests check
that it is bitwise reproducible and still matches the reference's own
substeps.
"""
import json
import os

import numpy as np
import pytest
import torch

import refparity as RP
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300.adjoint import SandRollout

pytestmark = pytest.mark.gpu


def test_ordered_forward_is_bitwise_reproducible(cuda):
    sc = S.sand_rollout_131k()
    sand = SandRollout(sc, n_substeps=20, device=cuda)
    assert sand.engine.ordered
    v0 = sand.v0_default
    a = sand.forward(v0, sc.E, sc.friction_angle, keep=False).clone()
    sa = sand.engine.export(A.FIELD_STRESS).clone()
    b = sand.forward(v0, sc.E, sc.friction_angle, keep=False).clone()
    sb = sand.engine.export(A.FIELD_STRESS).clone()
    assert torch.equal(a, b) and torch.equal(sa, sb)
    # the regular P2G: the same result up to float32 rounding
    sand.engine.ordered = False
    c = sand.forward(v0, sc.E, sc.friction_angle, keep=False)
    assert RP.rel(c.cpu().numpy(), a.cpu().numpy()) < 1e-4


@pytest.mark.parametrize("scene", ["sand_column", "sand_deformed"])
def test_ordered_substep_matches_reference_run(cuda, scene):
    """Lockstep against the reference's own substeps at the per-substep bar."""
    d = RP.load(scene)
    for k in range(d["substeps"]):
        sim = RP.gpu_from(d, k)
        sim.engine.ordered = True
        sim.p2g2p(k, d["dt"])
        assert sim.check_status() == 0
        got, ref = RP.gpu_state(sim), RP.state(d, k + 1)
        for f in ("x", "v", "F", "C"):
            assert RP.rel(got[f], ref[f]) < RP.TOL_STEP, (scene, k, f)
        gg, rg = RP.gpu_grid(sim), RP.grid(d, k + 1)
        for f in rg:
            assert RP.rel(gg[f], rg[f]) < RP.TOL_STEP, (scene, k, f)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def config2(cuda):
    """The rollout, the float64 target and the float64 central differences of
    tests/golden/make_adjoint_fd.py."""
    sc = S.sand_rollout_131k()
    sand = SandRollout(sc, checkpoint_every=10, device=cuda)
    with open(os.path.join(GOLDEN, "adjoint_fd_sand_rollout_131k.json")) as f:
        fd = json.load(f)
    disp = np.load(os.path.join(GOLDEN, "adjoint_target_sand_rollout_131k.npz"))["displacement"]
    target = sc.particles()[0].astype(np.float64) + disp.astype(np.float64)
    return sc, sand, torch.from_numpy(target).to(cuda), fd


def _directional(ref, v0b, Eb, phib, n):
    rng = np.random.default_rng(ref["direction_seed"])
    d = rng.standard_normal((ref["n_directions"], n, 3))
    d /= np.linalg.norm(d.reshape(ref["n_directions"], -1), axis=1)[:, None, None]
    g = v0b.double().cpu().numpy()
    got = {"E": float(Eb), "friction_angle": float(phib)}
    for k in range(ref["n_directions"]):
        got[f"v0_direction_{k}"] = float((g * d[k]).sum())
    return got


def test_config2_linear_functional_gradients_match_central_differences(cuda, config2):
    """The adjoint at the stated size on a loss without a small residual:
    gradients of mean(w * x_final) (w standard normals, default_rng(2025))
    with respect to E, the friction angle and 16 unit directions of v0,
    against float64 central differences (relative step 1e-3, converged: 1e-4
    agrees to 1e-5).  The float32 rollout that is differentiated ends 6e-4
    (relative RMS of the displacement) from the float64 rollout, and its
    Jacobian differs accordingly: measured 1.3e-4 .. 1e-2 (median 1e-3); bar
    3e-2 for each of the 18."""
    sc, sand, _, ref = config2
    n = sc.n_particles
    w = np.random.default_rng(ref["linear_seed"]).standard_normal((n, 3))
    sand.forward(sand.v0_default.clone(), sc.E, sc.friction_angle)
    v0b, Eb, phib = sand.backward(torch.from_numpy(w / w.size).to(cuda, torch.float32))
    got = _directional(ref, v0b, Eb, phib, n)
    errs = {k: abs(got[k] - f) / abs(f) for k, f in ref["fd_linear"].items()}
    print({k: (got[k], ref["fd_linear"][k], errs[k]) for k in errs})
    assert len(errs) == 2 + 16
    assert all(e <= 3e-2 for e in errs.values()), errs


def test_config2_gradients_match_central_differences(cuda, config2):
    """The stated loss, MSE of the final positions against the target rollout:
    adjoint of the float32 GPU rollout against float64 central differences
    (relative step 1e-3).  The MSE residual is small (8.3e-6 RMS against
    displacements of 2.9e-4), and a float32 rollout's final displacements sit
    1.8e-7 RMS from the float64 rollout's (the float32 and float64 oracles,
    same inputs): 2 % of the residual, so the float32 loss differs from the
    float64 loss by 1.3 % and no float32 forward gives this gradient to 1e-3.
    Bars: E and friction angle within 3e-3, each v0 direction within 5e-2
    (measured 2.2e-3, 4e-4 and at most 2.1e-2).  (Differences of the float32
    forward at this step measure its rounding: the loss changes by about
    1e-6 of itself.)"""
    sc, sand, target, ref = config2
    v0 = sand.v0_default.clone()
    x = sand.positions(sand.forward(v0, sc.E, sc.friction_angle))
    xbar = (2.0 * (x.double() - target) / x.numel()).float()
    v0b, Eb, phib = sand.backward(xbar)
    got = _directional(ref, v0b, Eb, phib, sc.n_particles)
    errs = {name: abs(got[name] - f) / abs(f) for name, f in ref["fd"].items()}
    print({name: (got[name], ref["fd"][name], errs[name]) for name in errs})
    assert len(errs) == 2 + 16
    assert errs["E"] <= 3e-3 and errs["friction_angle"] <= 3e-3, errs
    assert all(e <= 5e-2 for e in errs.values()), errs
