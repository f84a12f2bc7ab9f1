"""CPU checks of the oracle itself (no GPU): closed-form known answers
(tests/golden), an independent NumPy/LAPACK float64 restatement, and
analytic invariants of the substep.  These pin the oracle before it is used
to check the GPU path."""
import json
import os

import numpy as np
import pytest

from oracle import mpm_numpy as MN
from oracle import oracle as O
from reduced_mpm_stress_training_gb300 import scenarios as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _build_oracle():
    from oracle import build

    build.build()


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("bits,tol", [(32, 3e-6), (64, 1e-13)])
def test_svd_identities(bits, tol):
    rng = np.random.default_rng(0)
    A = np.concatenate([rng.normal(size=(2000, 3, 3)),
                        np.eye(3)[None] + 1e-3 * rng.normal(size=(2000, 3, 3)),
                        np.tile(np.eye(3), (4, 1, 1)), np.diag([2.0, 1.0, -0.5])[None]])
    U, s, V = (x.astype(np.float64) for x in O.svd3(A, bits))
    R = np.einsum("nij,nj,nkj->nik", U, s, V)
    scale = np.linalg.norm(A, axis=(1, 2))
    assert np.max(np.linalg.norm(R - A, axis=(1, 2)) / scale) < tol * 10
    assert np.abs(np.einsum("nji,njk->nik", U, U) - np.eye(3)).max() < tol
    assert np.abs(np.einsum("nji,njk->nik", V, V) - np.eye(3)).max() < tol
    assert np.abs(np.linalg.det(U) - 1).max() < tol and np.abs(np.linalg.det(V) - 1).max() < tol
    assert np.all(np.abs(s[:, 0]) >= np.abs(s[:, 1]) * (1 - tol))
    assert np.all(np.abs(s[:, 1]) >= np.abs(s[:, 2]) * (1 - tol))
    sref = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(np.abs(s) - sref) / sref[:, :1]) < tol * 10
    det = np.linalg.det(A)
    assert np.all(np.sign(s[:, 2]) == np.sign(det))


def _kat_model(c, bits):
    return O.make_model(8, material=c["material"], E=c["E"], nu=c["nu"],
                        friction_angle=c["friction_angle"])


@pytest.mark.parametrize("bits", [32, 64])
def test_return_map_golden(bits):
    cases = json.load(open(os.path.join(GOLDEN, "kat_return_map.json")))
    for c in cases:
        m = _kat_model(c, bits)
        Fo, tau, _ = O.return_map(m, np.array([c["F_trial"]]), yield_stress=c["yield_stress"],
                                  bits=bits)
        tF = 1e-12 if bits == 64 else 2e-6
        mu = c["E"] / 2 / (1 + c["nu"])
        tT = 1e-9 if bits == 64 else 2e-6
        assert np.max(np.abs(Fo[0] - c["F"])) < tF, c
        assert np.max(np.abs(tau[0] - c["stress"])) < tT * mu, (c, tau[0])


@pytest.mark.parametrize("bits", [32, 64])
def test_p2g_single_particle_golden(bits):
    g = json.load(open(os.path.join(GOLDEN, "kat_p2g.json")))
    m = O.make_model(g["n_grid"], g["grid_lim"], material="jelly", E=1e3, nu=0.3)
    sim = O.OracleSim(m, np.array([g["x"]]), np.array([g["mass"]]), np.array([g["vol"]]),
                      np.array([g["v"]]), bits=bits)
    sim.C[0] = g["C"]
    sim.stress[0] = g["stress"]
    sim.stage_p2g(g["dt"])
    tol = 1e-12 if bits == 64 else 1e-6
    for nd in g["nodes"]:
        i, j, k = nd["index"]
        assert abs(sim.grid_m[i, j, k] - nd["mass"]) <= tol * g["mass"]
        mom = sim.grid_v_in[i, j, k]
        scale = g["mass"] * 1.0
        assert np.max(np.abs(mom - nd["momentum"])) <= tol * scale * 10
    assert abs(sim.grid_m.sum() - g["mass"]) < tol * g["mass"]


def test_c_oracle_matches_numpy_restatement():
    """C float64 oracle vs the independent NumPy/LAPACK restatement, 10 substeps."""
    sc = S.small_column(2048, 32)
    x0, v0, vol, mass = sc.particles()
    rng = np.random.default_rng(5)
    v0 = (0.2 * rng.normal(size=v0.shape)).astype(np.float32)
    m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity)
    cols = [O.surface_collider((0, 0, 0.15), (0, 0, 1)), O.bounding_box()]
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=64, colliders=cols)
    st = dict(x0=x0.astype(np.float64), u=np.zeros((2048, 3)), v=v0.astype(np.float64),
              C=np.zeros((2048, 9)), F=np.tile(np.eye(3).reshape(1, 9), (2048, 1)),
              stress=np.zeros((2048, 9)), mass=mass.astype(np.float64), vol=vol.astype(np.float64))
    cold = [dict(kind=0, point=(0, 0, 0.15), normal=(0, 0, 1.0), start_time=0, end_time=999),
            dict(kind=1, start_time=0, end_time=999)]
    for step in range(10):
        sim.stage_p2g(sc.dt)
        sim.stage_grid(sc.dt)
        gm, gp, gv = MN.p2g2p(st, sc.n_grid, 1 / sc.n_grid, sc.dt, 2, m.mu, m.lam, m.alpha,
                              sc.gravity, cold, time=step * sc.dt)
        assert rel(sim.grid_m, gm) < 1e-12
        assert rel(sim.grid_v_in, gp) < 1e-11
        assert rel(sim.grid_v_out, gv) < 1e-11
        sim.stage_g2p(sc.dt)
    for f in ("u", "v", "C", "F", "stress"):
        assert rel(getattr(sim, f), st[f]) < 1e-9, f


def test_free_fall_closed_form():
    """No stress, no colliders: v_k = k dt g and u_k = dt^2 g k(k+1)/2 exactly (f64)."""
    sc = S.small_column(512, 32, material="sand")
    x0, v0, vol, mass = sc.particles()
    g = (0.0, 0.0, -9.8)
    m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu, gravity=g)
    sim = O.OracleSim(m, x0, mass, vol, np.zeros_like(v0), bits=64)
    dt = 1e-4
    for k in range(1, 21):
        sim.p2g2p(dt)
        assert np.allclose(sim.v[:, 2], -9.8 * dt * k, rtol=1e-11, atol=0)
        assert np.allclose(sim.u[:, 2], -9.8 * dt * dt * k * (k + 1) / 2, rtol=1e-8, atol=1e-15)
        assert np.abs(sim.C).max() < 1e-10
        assert np.abs(sim.F - np.eye(3).reshape(1, 9)).max() < 1e-12


def test_rigid_translation():
    sc = S.small_column(512, 32, material="jelly")
    x0, v0, vol, mass = sc.particles()
    m = O.make_model(sc.n_grid, material="jelly", E=sc.E, nu=sc.nu)
    vel = np.tile(np.array([[0.3, -0.1, 0.2]]), (512, 1))
    # u tolerance: float32 rounding of x = x0 + u (ulp(0.5) = 6e-8) per step
    for bits, tol, tol_u in ((64, 1e-12, 1e-14), (32, 1e-5, 1e-6)):
        sim = O.OracleSim(m, x0, mass, vol, vel, bits=bits)
        for _ in range(10):
            sim.p2g2p(1e-4)
        assert np.max(np.abs(sim.v - vel)) < tol
        assert np.max(np.abs(sim.u - 10 * 1e-4 * vel)) < tol_u


def test_mass_conservation_and_fp_spread():
    """Sum of grid mass = sum of particle mass; and the float32 oracle stays
    within 1e-4 of the float64 rerun over 20 sand substeps on u and F."""
    sc = S.small_column(4096, 32)
    s32 = None
    for bits in (32, 64):
        x0, v0, vol, mass = sc.particles()
        m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu,
                         friction_angle=sc.friction_angle, gravity=sc.gravity)
        cols = [O.surface_collider((0, 0, 0.15), (0, 0, 1)), O.bounding_box()]
        sim = O.OracleSim(m, x0, mass, vol, v0, bits=bits, colliders=cols)
        sim.stage_p2g(sc.dt)
        assert abs(sim.grid_m.astype(np.float64).sum() / mass.astype(np.float64).sum() - 1) < 1e-5
        sim.stage_grid(sc.dt)
        sim.stage_g2p(sc.dt)
        for _ in range(19):
            sim.p2g2p(sc.dt)
        if bits == 32:
            s32 = sim
    assert rel(s32.F, sim.F) < 1e-4
    # positions: float32 rounding of x = x0 + u (ulp(0.5) = 6e-8 per substep)
    assert rel(s32.x0 + s32.u, sim.x0 + sim.u) < 1e-6
    assert np.max(np.abs(s32.u - sim.u)) < 20 * 1.2e-7


def test_parallel_p2g_matches_serial():
    sc = S.small_column(4096, 32)
    x0, v0, vol, mass = sc.particles()
    m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu, gravity=sc.gravity)
    a = O.OracleSim(m, x0, mass, vol, v0, bits=64)
    b = O.OracleSim(m, x0, mass, vol, v0, bits=64)
    for _ in range(3):
        a.p2g2p(sc.dt, nthreads_p2g=1)
        b.p2g2p(sc.dt, nthreads_p2g=4)
    assert rel(a.u, b.u) < 1e-12 and rel(a.F, b.F) < 1e-12


def test_unknown_material_raises():
    with pytest.raises(TypeError):
        O.material_code("water")


def test_out_of_domain_is_flagged_and_frozen():
    sc = S.small_column(64, 16)
    x0, v0, vol, mass = sc.particles()
    x0[3] = (0.99, 0.5, 0.5)
    m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu, gravity=sc.gravity)
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=32)
    sim.p2g2p(sc.dt)
    assert sim.status.value & O.ST_OUT_OF_DOMAIN
    assert np.all(sim.u[3] == 0) and np.all(sim.F[3] == np.eye(3, dtype=np.float32).ravel())


def _collide(col, n=16, time=1e-4, dt=1e-4):
    """The oracle's collider kernel on a zero velocity grid (float32 build)."""
    import ctypes as C
    m = O.make_model(n, 1.0, material="sand", E=2e5, nu=0.3)
    gv = np.zeros(n ** 3 * 3, dtype=np.float32)
    O.lib(32).orc32_collide_extended(C.byref(m), C.byref(col), C.c_double(time), C.c_float(dt),
                                     gv.ctypes.data_as(C.c_void_p))
    idx = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    return gv.reshape(-1, 3), idx.astype(np.float32) * np.float32(1.0 / n)


def test_oracle_extended_colliders_known_answers():
    """Region and velocity of each extended collider kernel on a 16^3 grid
    (engine_stress/mpm_solver_warp.py:527-720), and the host-side motion."""
    f = np.float32
    # sphere: |x - c| < r takes the velocity
    col = O.sphere_leader((0.5, 0.5, 0.5), 0.2, (1.0, -2.0, 0.5))
    v, x = _collide(col)
    inside = np.sqrt(((x - f(0.5)) ** 2).sum(1)) < f(0.2)
    assert inside.sum() > 0 and np.all(v[inside] == np.float32([1.0, -2.0, 0.5])) and np.all(v[~inside] == 0)
    # cube: every axis within the half-width
    col = O.velocity_cube((0.4, 0.5, 0.6), 0.13, (0.0, 0.0, 3.0))
    v, x = _collide(col)
    inside = np.all(np.abs(x - f([0.4, 0.5, 0.6])) < f(0.13), axis=1)
    assert inside.sum() == 4 * 5 * 4 and np.all(v[inside, 2] == 3.0) and np.all(v[~inside] == 0)
    # plane: the slab |(x - p).n| <= threshold
    col = O.velocity_plane((0.5, 0.5, 0.5), (0.0, 0.0, 1.0), (0.0, 1.0, 0.0), 0.07)
    v, x = _collide(col)
    inside = np.abs(x[:, 2] - f(0.5)) <= f(0.07)
    assert inside.sum() == 3 * 256 and np.all(v[inside, 1] == 1.0) and np.all(v[~inside] == 0)
    # disk about x: rigid rotation v = v_scale n x r with r = (0, y, z) - p
    col = O.rotating_disk((0.5, 0.5, 0.5), (1.0, 0.0, 0.0), 0.3, 0.07, 4.0)
    v, x = _collide(col)
    r = x - f(0.5)
    inside = (np.abs(r[:, 0]) < f(0.07)) & (np.sqrt(r[:, 1] ** 2 + r[:, 2] ** 2) < f(0.3))
    r[:, 0] = 0
    expect = 4.0 * np.cross(np.array([1.0, 0.0, 0.0]), r)
    assert inside.sum() > 0 and np.allclose(v[inside], expect[inside], atol=1e-5)
    assert np.all(v[~inside] == 0)
    # the moving kinds advance by dt v while active, in float
    col = O.sphere_leader((0.5, 0.5, 0.5), 0.2, (1.0, -2.0, 0.5), start_time=0.0, end_time=1e-3)
    O.advance_collider(col, 0.0, 1e-4)
    assert tuple(col.point) == tuple(float(f(a + 1e-4 * b)) for a, b in zip((0.5, 0.5, 0.5), (1.0, -2.0, 0.5)))
    O.advance_collider(col, 2e-3, 1e-4)  # outside its window: stays
    assert tuple(col.point) == tuple(float(f(a + 1e-4 * b)) for a, b in zip((0.5, 0.5, 0.5), (1.0, -2.0, 0.5)))
    with pytest.raises(ValueError):
        O.rotating_disk((0.5, 0.5, 0.5), (0.05, 1.0, 0.0), 0.3, 0.07, 4.0)


def test_injected_faults_set_status_bits():
    """Failure detection on the host: a NaN position freezes its particle and sets
    the out-of-domain bit, a NaN deformation gradient sets the non-finite bit, an
    exploding velocity sets the CFL bit -- status words, never a trap or a hang."""
    sc = S.small_column(256, 16)
    m = O.make_model(sc.n_grid, material="sand", E=sc.E, nu=sc.nu, gravity=sc.gravity)
    x0, v0, vol, mass = sc.particles()
    x_nan = x0.copy()
    x_nan[5] = np.nan
    sim = O.OracleSim(m, x_nan, mass, vol, v0, bits=32)
    sim.p2g2p(sc.dt)
    assert sim.status.value & O.ST_OUT_OF_DOMAIN
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=32)
    sim.F[7] = np.nan
    sim.p2g2p(sc.dt)
    assert sim.status.value & O.ST_NONFINITE
    v_fast = v0.copy()
    v_fast[3] = (0.0, 0.0, 1e4)   # far beyond dx / dt
    sim = O.OracleSim(m, x0, mass, vol, v_fast, bits=32)
    sim.p2g2p(sc.dt)
    assert sim.status.value & O.ST_CFL
