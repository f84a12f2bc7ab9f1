"""Learned stress surrogate on the GPU: features and the gated, corrected
stress against the float64 oracle (oracle/surrogate.py) given the same
network outputs; a network trained by the library's own kernels against the
plain return map; the surrogate substep against the plain substep."""
import numpy as np
import pytest
import torch

from oracle import surrogate as SO
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300 import surrogate as SU

pytestmark = pytest.mark.gpu

MAT = (2e5, 0.3, 30.0)


def _exact(F, E, nu, phi):
    """Plain return map (the SVD path) on the device: (F_out, stress)."""
    lib = A.load()
    F = F.contiguous()
    Fo = torch.empty_like(F)
    tau = torch.empty_like(F)
    sc = SU.sand_scene(E, nu, phi)
    A.check(lib.mpm_return_map(A.C.byref(sc), F.data_ptr(), None, Fo.data_ptr(), tau.data_ptr(),
                               F.shape[0], torch.cuda.current_stream().cuda_stream), "return_map")
    return Fo, tau


def _column(n, material="sand", seed=3):
    """A column standing on the sticky floor (loaded from the first substep)."""
    return S.small_column(n, 48, material=material, seed=seed, floor_z=0.15)


@pytest.fixture(scope="module")
def rollout(cuda):
    return SU.rollout_F_trial(_column(20000), 600, 60, device=cuda)


@pytest.fixture(scope="module")
def trained(cuda, rollout):
    x, y = SU.build_training_set(2_000_000, device=cuda, seed=0, rollout=rollout)
    net = SU.StressMLP(cuda, seed=0)
    # a shorter schedule than the full recipe (60k steps at lr 1e-3) keeps the test fast
    log = SU.train(net, x, y, steps=20000, lr=3e-3, lr_min=1e-5, log_every=4000)
    print("training loss", log)
    return net


def _held_out(cuda, rollout, n=200_000, seed=99):
    rng = np.random.default_rng(seed)
    a = torch.from_numpy(SU.synthetic_F(n // 2, rng, max_log=0.1, log_uniform_scale=True)).to(cuda)
    pick = torch.from_numpy(rng.choice(rollout.shape[0], n - n // 2)).to(cuda)
    return torch.cat([a, rollout[pick]])


def test_features_match_oracle(cuda):
    rng = np.random.default_rng(0)
    F = torch.from_numpy(SU.synthetic_F(5000, rng, log_uniform_scale=True)).to(cuda)
    E, nu, phi = 3e5, 0.28, 33.0
    _, tau = _exact(F, E, nu, phi)
    x, y = SU.label(F, E, nu, phi)
    mu, lam = E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)
    s = np.sin(phi / 180 * 3.14159265)
    alpha = np.sqrt(2 / 3) * 2 * s / (3 - s)
    xr = SO.features(F.cpu().numpy(), mu, lam, alpha)
    yr = SO.targets(F.cpu().numpy(), tau.cpu().numpy(), mu)
    # B = F F^T - I from a rotated float32 F carries ~1e-7 absolute rounding
    # (the rotation cancels): compare where rho >= 1e-4, the gate's domain
    dom = xr[:, 9] >= (np.log10(1e-4) + 2.5) / 1.5
    assert dom.sum() > 3000
    assert np.abs(x.cpu().numpy()[dom] - xr[dom]).max() < 5e-3
    assert np.abs(y.cpu().numpy()[dom] - yr[dom]).max() < 5e-3 * max(1.0, np.abs(yr[dom]).max())


def test_apply_matches_oracle_given_the_network_outputs(cuda, trained, rollout):
    F = _held_out(cuda, rollout, 20000)
    E, nu, phi = MAT
    sur = SU.StressSurrogate(trained)
    Fo, tau, codes = sur.apply(F, E, nu, phi)
    x, _ = SU.label(F, E, nu, phi)
    y = trained.forward(x).cpu().numpy()
    mu, lam = E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)
    s = np.sin(phi / 180 * 3.14159265)
    alpha = np.sqrt(2 / 3) * 2 * s / (3 - s)
    rc, rF, rt = SO.apply(F.cpu().numpy(), y, mu, lam, alpha, SU.DEFAULT_CONFIG)
    c = codes.cpu().numpy()
    agree = np.mean(c == rc)
    assert agree > 0.98, agree
    both = (c <= 1) & (rc <= 1)
    assert both.sum() > 1000
    tn = np.linalg.norm(rt[both], axis=1)
    dt = np.linalg.norm(tau.cpu().numpy()[both] - rt[both], axis=1) / np.maximum(tn, 1e-30)
    assert np.quantile(dt, 0.99) < 1e-3, np.quantile(dt, 0.99)
    dF = np.abs(Fo.cpu().numpy()[both] - rF[both]).max()
    assert dF < 1e-5, dF
    # elastic rows keep F_trial bit for bit
    el = c == SU.A.SUR_ELASTIC
    assert torch.equal(Fo[torch.from_numpy(el).to(cuda)], F[torch.from_numpy(el).to(cuda)])


def test_trained_network_gain(cuda, trained, rollout):
    """Against the plain return map on held-out tuples: the trained surrogate
    (gated, with fallback) meets 1e-2 relative stress error and takes most
    particles off the SVD path; an untrained network takes almost none, and
    the SVD-free linear-elastic stress that the network replaces is far off."""
    F = _held_out(cuda, rollout)
    E, nu, phi = MAT
    Fe, te = _exact(F, E, nu, phi)
    res = {}
    for name, net in (("trained", trained), ("untrained", SU.StressMLP(cuda, seed=1))):
        sur = SU.StressSurrogate(net)
        Fo, tau, codes = sur.apply(F, E, nu, phi)
        eligible = (codes <= 1) | (codes == A.SUR_FB_GATE)
        acc = ((codes <= 1).sum() / eligible.sum()).item()
        err = SU.stress_errors(tau, te)
        res[name] = (acc, err["rel_l2"], err["row_p99"])
    # linear elasticity without the return map: tau = mu B + lam/2 tr(B) I
    mu, lam = E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)
    F3 = F.reshape(-1, 3, 3).double()
    B = F3 @ F3.transpose(1, 2) - torch.eye(3, device=cuda, dtype=torch.float64)
    tl = mu * B + 0.5 * lam * B.diagonal(dim1=1, dim2=2).sum(1)[:, None, None] * torch.eye(3, device=cuda)
    lin = SU.stress_errors(tl.reshape(-1, 9).float(), te)["rel_l2"]
    print({"trained (accepted, rel_l2, row_p99)": res["trained"],
           "untrained": res["untrained"], "linear_elastic_rel_l2": lin})
    acc_t, err_t, _ = res["trained"]
    acc_u, err_u, _ = res["untrained"]
    assert err_t <= 1e-2 and err_u <= 1e-2  # fallback keeps both within tolerance
    assert acc_t > 0.3, acc_t
    assert acc_u < 0.05, acc_u
    assert lin > 10 * err_t


def _pair(cuda, material="sand", n=20000, warm=300):
    sc = _column(n, material=material, seed=5)
    a = S.build_simulator(sc, device=cuda)
    b = S.build_simulator(sc, device=cuda)
    for k in range(warm):
        a.p2g2p(k, sc.dt)
        b.p2g2p(k, sc.dt)
    return sc, a, b


def _field(sim, f):
    return sim.engine.export(f).reshape(sim.n_particles, -1)


def test_surrogate_substep_against_plain(cuda, trained):
    sc, plain, sur_sim = _pair(cuda)
    sur = SU.StressSurrogate(trained)
    sur_sim.set_stress_surrogate(sur)
    plain.p2g2p(0, sc.dt)
    sur_sim.p2g2p(0, sc.dt)
    torch.cuda.synchronize()
    # x and v do not depend on this substep's return map (P2G's float atomics
    # make two runs differ at rounding level only)
    for f in (A.FIELD_X, A.FIELD_V):
        d = SU.stress_errors(_field(sur_sim, f), _field(plain, f))["rel_l2"]
        assert d < 1e-5, (f, d)
    e = SU.stress_errors(_field(sur_sim, A.FIELD_STRESS), _field(plain, A.FIELD_STRESS))
    dF = (_field(sur_sim, A.FIELD_F) - _field(plain, A.FIELD_F)).abs().max().item()
    counts = sur.outcome_counts()
    print("one substep:", e, "max |dF|", dF, counts)
    assert e["rel_l2"] <= 1e-2, e
    assert dF < 1e-4
    accepted = counts["elastic"] + counts["plastic"]
    assert accepted > 0.25 * (accepted + counts["fb_gate"]), counts
    # a short rollout stays close
    for k in range(1, 20):
        plain.p2g2p(k, sc.dt)
        sur_sim.p2g2p(k, sc.dt)
    e20 = SU.stress_errors(_field(sur_sim, A.FIELD_STRESS), _field(plain, A.FIELD_STRESS))
    dx = (_field(sur_sim, A.FIELD_X) - _field(plain, A.FIELD_X)).abs().max().item()
    print("20 substeps:", e20, "max |dx|", dx)
    assert e20["rel_l2"] <= 3e-2 and dx < 1e-4


def test_metal_scene_takes_the_svd_path(cuda, trained):
    sc, plain, sur_sim = _pair(cuda, material="metal", n=8000, warm=40)
    sur = SU.StressSurrogate(trained)
    sur_sim.set_stress_surrogate(sur)
    plain.p2g2p(0, sc.dt)
    sur_sim.p2g2p(0, sc.dt)
    # the same return map on the same F_trial; the states differ only by the
    # rounding-level run-to-run differences of P2G's float atomics
    for f in (A.FIELD_F, A.FIELD_STRESS, A.FIELD_V, A.FIELD_X, A.FIELD_YIELD):
        d = SU.stress_errors(_field(sur_sim, f), _field(plain, f))["rel_l2"]
        assert d < 1e-3, (f, d)
    assert sur.outcome_counts()["fb_material"] == sc.n_particles


def test_surrogate_substeps_replay_in_a_graph(cuda, trained):
    sc, eager, graphed = _pair(cuda, warm=200)
    for sim in (eager, graphed):
        sim.set_stress_surrogate(SU.StressSurrogate(trained))
    g = graphed.engine.graph(4, 0.0, sc.dt)
    g.replay()
    for k in range(4):
        eager.engine.substep_raw(0.0, sc.dt)
    torch.cuda.synchronize()
    for f in (A.FIELD_X, A.FIELD_F, A.FIELD_STRESS):
        d = SU.stress_errors(_field(graphed, f), _field(eager, f))["rel_l2"]
        assert d < 1e-2, (f, d)
