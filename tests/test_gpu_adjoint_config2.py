"""The differentiable-rollout workload at its stated size, and the ordered
P2G that makes its finite-difference check meaningful.

Workload (131,072 sand particles, 96^3 grid, 100 substeps at dt 1e-4, v0 ~
N(0, 0.1^2) per component, loss = MSE between the final positions and a
target rollout with E = 3e5 and friction 35 deg from the same seed):
gradients of the loss with respect to E, the friction angle and the
initial velocity (16 random unit directions) from the hand-written adjoint,
against central differences with a relative step of 1e-3, agreeing to 1e-3.

The reference has no gradient path (no wp.Tape anywhere in
engine_stress/mpm_solver_warp.py:156-203), so the only comparison is with
finite differences of the forward.  Those need a forward that is a
deterministic function of its inputs: the ordered P2G (mpm_p2g_ordered)
takes every cell's particles in uid order and sums the block tiles per node
in a fixed order, and the first tests check that it is bitwise
reproducible and still matches the reference's own substeps.
"""
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


@pytest.fixture(scope="module")
def config2(cuda):
    sc = S.sand_rollout_131k()
    sand = SandRollout(sc, checkpoint_every=10, device=cuda)
    target = sand.positions(sand.forward(sand.v0_default, 3e5, 35.0, keep=False)).clone()
    return sc, sand, target


def test_config2_gradients_match_central_differences(cuda, config2):
    sc, sand, target = config2
    v0 = sand.v0_default.clone()
    E, phi = sc.E, sc.friction_angle

    def J(v, e_, p_):
        x = sand.positions(sand.forward(v, e_, p_, keep=False))
        return float(((x - target) ** 2).mean())

    x = sand.positions(sand.forward(v0, E, phi))
    v0b, Eb, phib = sand.backward(2.0 * (x - target) / x.numel())
    rh = 1e-3
    res = {"E": (Eb, (J(v0, E * (1 + rh), phi) - J(v0, E * (1 - rh), phi)) / (2 * rh * E)),
           "friction_angle": (phib, (J(v0, E, phi * (1 + rh)) - J(v0, E, phi * (1 - rh))) / (2 * rh * phi))}
    g = torch.Generator(device=cuda).manual_seed(0)
    for k in range(16):
        dirn = torch.randn(v0.shape, generator=g, device=cuda)
        dirn /= dirn.norm()
        h = rh * v0.norm().item()
        fd = (J(v0 + h * dirn, E, phi) - J(v0 - h * dirn, E, phi)) / (2 * h)
        res[f"v0_direction_{k}"] = (float((v0b.double() * dirn.double()).sum()), fd)
    errs = {name: abs(a - f) / abs(f) for name, (a, f) in res.items()}
    print({name: (a, f, errs[name]) for name, (a, f) in res.items()})
    assert all(e <= 1e-3 for e in errs.values()), errs
