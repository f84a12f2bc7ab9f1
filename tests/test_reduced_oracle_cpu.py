"""CPU checks of the oracle's reduced sampled-quadrature substep
(MPM_Simulator_WARP.p2g2p_reduced, engine_stress/mpm_solver_warp.py:207-227;
kernels engine_stress/mpm_utils.py:318-471): closed-form marks, a stress-free
known answer, the independent NumPy float64 restatement, the float32 build
against the float64 one, the sample gather, and the reference's indexing of
yield_stress by the sample's list position."""
import numpy as np
import pytest

from oracle import mpm_numpy as MN
from oracle import oracle as O
from reduced_mpm_stress_training_gb300 import scenarios as S


@pytest.fixture(scope="module", autouse=True)
def _build_oracle():
    from oracle import build

    build.build()


def _sim(material="sand", n_grid=16, n=512, bits=32, seed=0, fdisp_sigma=0.0, **model_kw):
    sc = S.small_column(n, n_grid, material=material, seed=seed)
    x0, v0, vol, mass = sc.particles()
    m = O.make_model(n_grid, material=material, E=sc.E, nu=sc.nu, friction_angle=sc.friction_angle,
                     gravity=sc.gravity, **model_kw)
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=bits, yield_stress=sc.yield_stress)
    sim.density[:] = sc.density
    rng = np.random.default_rng(seed + 1)
    sim.v[:] = rng.normal(0.0, 0.3, sim.v.shape)
    if fdisp_sigma:
        sim.F_disp[:] = rng.normal(0.0, fdisp_sigma, sim.F_disp.shape)
    return sc, sim


def _base(x, n_grid):
    return np.trunc(x.astype(np.float32) * np.float32(n_grid) - np.float32(0.5)).astype(np.int64)


def test_marks_are_the_clipped_neighbourhood():
    sc, sim = _sim()
    sim.x0[0] = (0.5, 0.5, 0.5)      # base cell (7, 7, 7): marks 5..9 on every axis
    sim.x0[1] = (0.02, 0.5, 0.5)     # base cell (0, 7, 7): x clipped to 0..2
    sim.sample_particle_index_short = np.array([0, 1], np.int32)
    sim.p2g2p_reduced(sc.dt)
    want = np.zeros((16, 16, 16), np.int32)
    want[5:10, 5:10, 5:10] = 1
    want[0:3, 5:10, 5:10] = 1
    assert np.array_equal(sim.neighboring_cells, want)
    assert not sim.neighboring_cells_grid_v.any()
    # experiment_for_C: offsets -2..4, added to what is there
    sim.sample_particle_index_short = np.array([0], np.int32)
    g = sim.experiment_for_C()
    want_v = np.zeros_like(want)
    want_v[5:12, 5:12, 5:12] = 1
    assert np.array_equal(g, want_v)
    sim.sample_particle_index_short = np.array([1], np.int32)
    g = sim.experiment_for_C()
    want_v[0:5, 5:12, 5:12] = 1
    assert np.array_equal(g, want_v)
    assert sim.status.value == 0


@pytest.mark.parametrize("material", ["jelly", "metal", "sand"])
def test_stress_free_known_answer(material):
    """F_disp = 0 gives F = I and zero stress for every material: the grid holds
    the marked particles' mass and momentum, v_out = v_in / m + dt g on marked
    nodes and 0 elsewhere."""
    sc, sim = _sim(material)
    sim.sample_particle_index_short = np.array([3, 100, 250], np.int32)
    sim.p2g2p_reduced(sc.dt)
    assert sim.status.value == 0
    base = _base(sim.x0 + sim.u, 16)
    marked = sim.neighboring_cells[base[:, 0], base[:, 1], base[:, 2]] > 0
    assert 0 < marked.sum() < sim.n
    assert np.allclose(sim.F[marked], np.eye(3, dtype=np.float32).ravel(), atol=0)
    m = sim.mass.astype(np.float64)
    assert np.isclose(sim.grid_m.sum(dtype=np.float64), m[marked].sum(), rtol=1e-5)
    mom = (m[:, None] * sim.v)[marked].sum(0)
    assert np.allclose(sim.grid_v_in.reshape(-1, 3).sum(0, dtype=np.float64), mom, rtol=1e-5, atol=1e-9)
    gm = sim.grid_m.ravel()
    mk = sim.neighboring_cells.ravel() > 0
    act = mk & (gm > np.float32(1e-10))
    gv = sim.grid_v_out.reshape(-1, 3)
    expect = sim.grid_v_in.reshape(-1, 3)[act] / gm[act, None] + np.float32(sc.dt) * np.float32(sc.gravity)
    assert np.allclose(gv[act], expect, rtol=1e-6, atol=1e-7)
    assert not gv[~act].any()
    # nodes with mass outside the marked cells (stencils reach two past them) stay at zero
    assert ((gm > 0) & ~mk).any()


@pytest.mark.parametrize("material", [0, 1, 2])
def test_c_oracle_matches_numpy_restatement(material):
    name = ["jelly", "metal", "sand"][material]
    sc, sim = _sim(name, bits=64, fdisp_sigma=0.05)
    sample = np.array([7, 120, 300, 301], np.int32)
    sim.sample_particle_index_short = sample
    state = dict(x0=sim.x0.copy(), u=sim.u.copy(), v=sim.v.copy(), F=sim.F.copy(), F_disp=sim.F_disp.copy(),
                 mass=sim.mass.copy())
    sim.p2g2p_reduced(sc.dt)
    mask, gm, gp, gv = MN.p2g2p_reduced(state, 16, 1.0 / 16, sc.dt, material, sc.mu, sc.lam, sc.gravity,
                                        sample, sim.density)
    assert np.array_equal(mask, sim.neighboring_cells)
    scale = np.abs(gp).max()
    assert np.abs(sim.grid_v_in - gp).max() <= 1e-12 * scale
    assert np.abs(sim.grid_m - gm).max() <= 1e-12 * np.abs(gm).max()
    assert np.abs(sim.grid_v_out - gv).max() <= 1e-10 * max(np.abs(gv).max(), 1.0)
    assert np.abs(sim.F - state["F"].reshape(-1, 9)).max() == 0


@pytest.mark.parametrize("material", ["jelly", "metal", "sand"])
def test_float32_build_tracks_float64(material):
    out = {}
    for bits in (32, 64):
        sc, sim = _sim(material, bits=bits, fdisp_sigma=0.05)
        sim.sample_particle_index_short = np.array([7, 120, 300, 301], np.int32)
        sim.p2g2p_reduced(sc.dt)
        out[bits] = sim
    a, b = out[32], out[64]
    assert np.array_equal(a.neighboring_cells, b.neighboring_cells)
    for f in ("grid_m", "grid_v_in", "grid_v_out"):
        x, y = getattr(a, f).astype(np.float64), getattr(b, f)
        assert np.abs(x - y).max() <= 2e-5 * np.abs(y).max(), f


def test_g2p_sample_uniform_velocity_known_answer():
    """A uniform grid velocity c: sample particles take v = c, x += dt c and
    keep F (jelly); the other particles are untouched."""
    sc, sim = _sim("jelly", fdisp_sigma=0.02)
    sample = np.array([4, 40, 400], np.int32)
    sim.sample_particle_index_short = sample
    sim.p2g2p_reduced(sc.dt)
    before = {k: getattr(sim, k).copy() for k in ("x", "u", "v", "F", "F_disp")}
    c = np.float32([0.25, -0.5, 1.0])
    sim.grid_v_out[:] = c
    sim.g2p_sample(sc.dt)
    assert sim.status.value == 0
    assert np.allclose(sim.v[sample], c, rtol=1e-6)
    assert np.allclose(sim.x[sample], before["x"][sample] + np.float32(sc.dt) * c, rtol=0, atol=1e-7)
    assert np.allclose(sim.F[sample], before["F"][sample], atol=1e-5)
    assert np.array_equal(sim.u[sample], sim.x[sample] - sim.x0[sample])
    eye = np.eye(3, dtype=np.float32).ravel()
    assert np.array_equal(sim.F_disp[sample], sim.F[sample] - eye)
    rest = np.setdiff1d(np.arange(sim.n), sample)
    for k in before:
        assert np.array_equal(getattr(sim, k)[rest], before[k][rest]), k


def test_g2p_sample_reads_yield_of_the_list_position():
    """mpm_utils.py:464 passes the loop index to von_mises_return_mapping:
    sample s = 0 naming particle 5 updates yield_stress[0], not [5]."""
    sc, sim = _sim("metal", hardening=1, xi=0.5)
    sim.sample_particle_index_short = np.array([5], np.int32)
    sim.p2g2p_reduced(sc.dt)
    ng = 16
    ii = np.arange(ng, dtype=np.float32) / ng
    gy = np.broadcast_to(ii[None, :, None], (ng, ng, ng))
    sim.grid_v_out[..., 0] = 300.0 * gy   # strong shear: plastic in one substep
    y0 = sim.yield_.copy()
    sim.g2p_sample(sc.dt)
    assert sim.yield_[0] > y0[0]
    assert sim.yield_[5] == y0[5]
    assert np.array_equal(sim.yield_[1:], y0[1:])


def test_bad_sample_index_is_flagged():
    sc, sim = _sim()
    sim.sample_particle_index_short = np.array([-1, sim.n], np.int32)
    sim.p2g2p_reduced(sc.dt)
    assert sim.status.value & O.ST_BAD_INPUT
    assert not sim.neighboring_cells.any() and not sim.grid_m.any()


def test_parallel_reduced_p2g_matches_serial():
    out = []
    for nt in (1, 4):
        sc, sim = _sim("sand", fdisp_sigma=0.05, bits=64)
        sim.sample_particle_index_short = np.array([7, 120, 300, 301], np.int32)
        sim.p2g2p_reduced(sc.dt, nthreads_p2g=nt)
        out.append(sim)
    a, b = out
    assert np.array_equal(a.neighboring_cells, b.neighboring_cells)
    for f in ("grid_m", "grid_v_in", "grid_v_out"):
        assert np.abs(getattr(a, f) - getattr(b, f)).max() <= 1e-12 * np.abs(getattr(a, f)).max(), f


@pytest.mark.parametrize("bits", [32, 64])
def test_reduced_p2g_golden(bits):
    """The closed-form fixture tests/golden/kat_reduced_p2g.json (one particle, diagonal
    F_disp) against the oracle's p2g_sample_all for jelly, metal and sand."""
    import json
    import os

    cases = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat_reduced_p2g.json")))
    tol = 1e-12 if bits == 64 else 2e-6
    for g in cases:
        m = O.make_model(g["n_grid"], g["grid_lim"], material=g["material"], E=g["E"], nu=g["nu"])
        sim = O.OracleSim(m, np.array([g["x"]]), np.array([g["mass"]]), np.array([g["mass"] / g["density"]]),
                          np.array([g["v"]]), bits=bits)
        sim.F_disp[0] = g["F_disp"]
        sim.density[:] = g["density"]
        sim.sample_particle_index_short = np.array([0], np.int32)
        sim.p2g2p_reduced(g["dt"])
        assert sim.status.value == 0
        scale = max(np.abs(nd["momentum"]).max() for nd in g["nodes"])
        for nd in g["nodes"]:
            i, j, k = nd["index"]
            assert abs(sim.grid_m[i, j, k] - nd["mass"]) <= tol * g["mass"], g["material"]
            assert np.abs(sim.grid_v_in[i, j, k] - nd["momentum"]).max() <= tol * scale * 10, g["material"]
        assert abs(sim.grid_m.sum() - g["mass"]) <= tol * g["mass"]
