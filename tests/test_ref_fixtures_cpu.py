"""The oracle pinned to the reference's OWN outputs (no GPU).

The fixtures in ``tests/golden/ref_*.npz`` were produced by running the
reference's unmodified solver (engine_stress/mpm_solver_warp.py:156-203,
mpm_utils.py:190-306) and decoder (CROMnet_secondary.py:203-301) through a
test-only Warp stand-in (``tests/golden/make_ref_fixtures.py``).  Here the
C oracle (float32 and float64) restarts from every recorded state and must
land on the next one:

  x (= x0 + u), v, C, F, grid mass / momentum / velocity:  1e-5 relative L2
  stress: 1e-5, or (near F = I, where float32 rounding dominates) the
          oracle's own error against its float64 twin within 4x the
          reference's (refparity.stress_check)
  metal yield stress (hardening): 1e-5

and run free for all substeps: x, v, F at 1e-5 per substep, C (the
velocity gradient, which picks up the float32 noise of the stress) at the
1e-4 rollout bar.  The float64 oracle's
distance to the reference is printed for every substep: it is the
reference's own float32 error.
"""
import numpy as np
import pytest
import torch

import refparity as RP
from helpers import netdec_torch
from oracle import decoder as OD
from reduced_mpm_stress_training_gb300 import decoder as D

FIELDS = ("x", "v", "C", "F")


@pytest.mark.parametrize("scene", RP.SCENES)
def test_oracle_lockstep_matches_reference_run(scene):
    d = RP.load(scene)
    for k in range(d["substeps"]):
        o32 = RP.oracle_from(d, k, 32)
        o64 = RP.oracle_from(d, k, 64)
        o32.p2g2p(d["dt"])
        o64.p2g2p(d["dt"])
        ref = RP.state(d, k + 1)
        got, got64 = RP.oracle_state(o32), RP.oracle_state(o64)
        errs = {f: RP.rel(got[f], ref[f]) for f in FIELDS}
        g = RP.grid(d, k + 1)
        for f in g:
            errs[f] = RP.rel(getattr(o32, f), g[f])
        if "yield" in ref:
            errs["yield"] = RP.rel(got["yield"], ref["yield"])
        print(scene, k + 1, "oracle32 vs reference", errs,
              "oracle64 vs reference", {f: RP.rel(got64[f], ref[f]) for f in FIELDS + ("stress",)})
        assert all(e < RP.TOL_STEP for e in errs.values()), (k, errs)
        ok, info = RP.stress_check(got["stress"], ref["stress"], got64["stress"])
        assert ok, (k, info)
        assert o32.status.value == 0


@pytest.mark.parametrize("scene", RP.SCENES)
def test_oracle_free_run_matches_reference_run(scene):
    d = RP.load(scene)
    o32 = RP.oracle_from(d, 0, 32)
    for k in range(d["substeps"]):
        o32.p2g2p(d["dt"])
        ref = RP.state(d, k + 1)
        got = RP.oracle_state(o32)
        errs = {f: RP.rel(got[f], ref[f]) for f in ("x", "v", "F")}
        assert all(e < RP.TOL_STEP for e in errs.values()), (k, errs)
        assert RP.rel(got["C"], ref["C"]) < RP.TOL_ROLLOUT, k


def test_fixture_scenes_exercise_every_branch():
    """The fixtures cover what they are meant to: every Drucker-Prager regime
    (elastic, apex, cone) in the deformed sand scene, plastic flow with
    hardening in the metal scene, walls and floor in every scene."""
    from oracle import oracle as O

    d = RP.load("sand_deformed")
    m = O.make_model(d["n_grid"], material="sand", mu=d["mu"], lam=d["lam"], friction_angle=d["friction_angle"])
    # regimes of the first substep's return map, recomputed in float64 from F_trial = F_new with
    # the elastic F unchanged: count the reference's outcomes by comparing F before and after
    Ft = RP.state(d, 0)["F"].reshape(-1, 3, 3).astype(np.float64)
    s = np.linalg.svd(Ft, compute_uv=False)
    eps = np.log(np.abs(s))
    tr = eps.sum(1)
    dev = eps - tr[:, None] / 3
    alpha = m.alpha
    dg = np.linalg.norm(dev, axis=1) + (3 * d["lam"] + 2 * d["mu"]) / (2 * d["mu"]) * tr * alpha
    assert (dg <= 0).sum() > 10 and ((dg > 0) & (tr > 0)).sum() > 10 and ((dg > 0) & (tr <= 0)).sum() > 10
    dm = RP.load("metal_block")
    assert (dm["yield"][-1] > dm["yield"][0] * (1 + 1e-6)).sum() > 50  # hardened particles
    for scene in RP.SCENES:
        d = RP.load(scene)
        ng = d["n_grid"]
        g = RP.grid(d, 1)
        touched = g["grid_m"] > 0
        assert touched[:3].any() and touched[ng - 3:].any() or touched[:, :, ng - 3:].any()
        assert touched[:, : int(d["floor_y"] * ng) + 1].any()  # nodes under the floor plane


@pytest.mark.parametrize("tag", ["elu", "siren"])
def test_decoder_restatements_match_reference_netdec(tag):
    """NetDec as the reference ran it vs the float64 NumPy restatement and the
    PyTorch float32 restatement of the decoder kernels' checker."""
    f = RP.netdec(tag)
    sd, rows, out = f["state_dict"], f["rows"], f["out"].astype(np.float64)
    q32 = netdec_torch(sd, torch.from_numpy(rows), f["label_dim"], f["siren"], f["omega_0"]).numpy()
    assert RP.rel(q32, out) < 1e-6
    blob = D.pack(sd, f["siren"]).numpy()
    hidden = sd["dec0.weight"].shape[0]
    mu_dim = sd["dec0.weight"].shape[1] - f["label_dim"] - 3
    q64 = OD.forward(blob, rows, f["label_dim"], mu_dim, hidden, f["siren"], f["omega_0"])
    assert RP.rel(out, q64) < 1e-5, RP.rel(out, q64)


def test_reference_frame_layout():
    """save_data_at_frame's datasets (mpm_solver_warp.py:339-404) as the
    reference wrote them for the last sand_column state, against a plain
    statement of the layout: x (3, n) = x_initial^T, q (3, n) = u^T,
    time (1, 1), masses (1, n), f_tensor (9, n) = (F - I) row-major ^T,
    stress (6, n) = [xx, xy, xz, yy, yz, zz]^T, v (3, n), mu (1, n) = the
    friction angle, C (9, n) row-major ^T; the OBJ file one 'v x y z c c c'
    line per particle."""
    d = RP.load("sand_column")
    fr = RP.frame()
    k = d["substeps"]
    s = RP.state(d, k)
    n = d["n"]
    assert np.array_equal(fr["x"], d["x0"].T)
    assert np.array_equal(fr["q"], s["u"].T)
    assert fr["time"].shape == (1, 1) and abs(float(fr["time"][0, 0]) - k * d["dt"]) < 1e-12
    assert np.array_equal(fr["masses"], d["mass"].reshape(1, n))
    fd = (s["F"].reshape(n, 3, 3) - np.eye(3, dtype=np.float32)).reshape(n, 9)
    assert np.array_equal(fr["f_tensor"], fd.T)
    st = s["stress"].reshape(n, 3, 3)
    six = np.stack([st[:, 0, 0], st[:, 0, 1], st[:, 0, 2], st[:, 1, 1], st[:, 1, 2], st[:, 2, 2]])
    assert fr["stress"].shape == (6, n) and np.array_equal(fr["stress"], six)
    assert np.array_equal(fr["v"], s["v"].T)
    assert np.array_equal(fr["mu"], np.full((1, n), d["friction_angle"]))
    assert np.array_equal(fr["C"], s["C"].T)
    lines = str(fr["obj_text"]).splitlines()
    assert len(lines) == n
    vals = np.array([[float(t) for t in ln.split()[1:]] for ln in lines])
    assert all(ln.split()[0] == "v" and len(ln.split()) == 7 for ln in lines)
    assert np.abs(vals[:, :3] - s["x"]).max() < 1e-6 and np.all(vals[:, 3:] == 0.0)
