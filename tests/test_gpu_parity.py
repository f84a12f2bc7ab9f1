"""GPU-vs-oracle parity of every stage of the substep, called through the
C ABI (libmpm_gb300.so) on seeded inputs.

Tolerances (relative L2 over all particles / nodes):
  per substep: 1e-5 on grid mass / momentum / velocity and particle x, v, F
  200-substep sand rollout: 1e-4 on x and F
  stress and C: within the float32 noise floor measured by the oracle itself
  (GPU vs float32 oracle no further than 3x float32 oracle vs float64 rerun),
  or 1e-5 relative when that is looser -- near F = I both are dominated by
  float32 rounding of the SVD, in the reference as here.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300.engine import MPMStatusError, SceneParams

from helpers import compare, gpu_sim, gpu_state, oracle_sim, rel, within_fp32_floor

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5
TOL_ROLLOUT = 1e-4


def _rand_F(n, rng, kind):
    if kind == "near_identity":
        return (np.eye(3)[None] + 0.02 * rng.normal(size=(n, 3, 3))).astype(np.float32)
    if kind == "compressed":
        # rotations times diag(exp(s)), s in [-0.3, 0.05]: exercises all DP branches
        q = rng.normal(size=(n, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        w, x, y, z = q.T
        R = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                      2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                      2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1).reshape(n, 3, 3)
        s = rng.uniform(-0.3, 0.05, size=(n, 3))
        q2 = rng.normal(size=(n, 4))
        q2 /= np.linalg.norm(q2, axis=1, keepdims=True)
        w, x, y, z = q2.T
        R2 = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                       2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                       2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1).reshape(n, 3, 3)
        return np.einsum("nij,nj,nkj->nik", R, np.exp(s), R2).astype(np.float32)
    return rng.normal(size=(n, 3, 3)).astype(np.float32)


@pytest.mark.parametrize("kind", ["random", "near_identity", "compressed"])
def test_svd3_matches_oracle(cuda, kind):
    rng = np.random.default_rng(1)
    n = 20000
    Fh = _rand_F(n, rng, kind).reshape(n, 9)
    lib = A.load()
    F = torch.from_numpy(Fh).to(cuda)
    U = torch.empty_like(F)
    V = torch.empty_like(F)
    s = torch.empty((n, 3), device=cuda)
    A.check(lib.mpm_svd3(F.data_ptr(), U.data_ptr(), s.data_ptr(), V.data_ptr(), n, 0), "svd")
    torch.cuda.synchronize()
    Ug, sg, Vg = (t.cpu().numpy().astype(np.float64) for t in (U, s, V))
    Ug, Vg = Ug.reshape(n, 3, 3), Vg.reshape(n, 3, 3)
    Uo, so, Vo = O.svd3(Fh, 32)
    # reconstruction, orthogonality, convention
    R = np.einsum("nij,nj,nkj->nik", Ug, sg, Vg)
    scale = np.linalg.norm(Fh.reshape(n, 3, 3), axis=(1, 2))
    assert np.max(np.linalg.norm(R - Fh.reshape(n, 3, 3), axis=(1, 2)) / scale) < 2e-5
    assert np.abs(np.einsum("nji,njk->nik", Ug, Ug) - np.eye(3)).max() < 2e-6
    assert np.abs(np.linalg.det(Ug) - 1).max() < 2e-6 and np.abs(np.linalg.det(Vg) - 1).max() < 2e-6
    assert np.all(np.sign(sg[:, 2]) == np.sign(np.linalg.det(Fh.reshape(n, 3, 3))))
    # singular values agree with the oracle's float32 SVD
    assert np.max(np.abs(sg - so) / np.abs(so[:, :1])) < 1e-5


def _scene_struct(material, mu, lam, friction=30.0, hardening=0, xi=0.0):
    sp = SceneParams(n_particles=0, n_grid=8, material=material, mu=mu, lam=lam,
                     friction_angle=friction, hardening=hardening, xi=xi)
    return sp.to_struct(0)


@pytest.mark.parametrize("material,kind", [(A.SAND, "near_identity"), (A.SAND, "compressed"),
                                           (A.METAL, "near_identity"), (A.METAL, "compressed"),
                                           (A.JELLY, "near_identity")])
def test_return_map_matches_oracle(cuda, material, kind):
    rng = np.random.default_rng(2)
    n = 20000
    Ft = _rand_F(n, rng, kind).reshape(n, 9)
    E, nu = (2e5, 0.3) if material != A.METAL else (1e7, 0.3)
    mu, lam = E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)
    ys = 1e5
    sc = _scene_struct(material, mu, lam, hardening=1 if material == A.METAL else 0, xi=0.5)
    lib = A.load()
    Fd = torch.from_numpy(Ft).to(cuda)
    Fo = torch.empty_like(Fd)
    tau = torch.empty_like(Fd)
    y = torch.full((n,), ys, device=cuda)
    A.check(lib.mpm_return_map(C.byref(sc), Fd.data_ptr(), y.data_ptr(), Fo.data_ptr(),
                               tau.data_ptr(), n, 0), "return_map")
    torch.cuda.synchronize()
    mat = {A.SAND: "sand", A.METAL: "metal", A.JELLY: "jelly"}[material]
    m = O.make_model(8, material=mat, mu=mu, lam=lam, friction_angle=30.0,
                     hardening=1 if material == A.METAL else 0, xi=0.5)
    Fr, tr, yr = O.return_map(m, Ft, yield_stress=ys, bits=32)
    F64, t64, y64 = O.return_map(m, Ft, yield_stress=ys, bits=64)
    assert rel(Fo.cpu().numpy(), Fr) < TOL_STEP
    ok, info = within_fp32_floor(tau.cpu().numpy(), tr, t64)
    assert ok, info
    if material == A.METAL:
        assert rel(y.cpu().numpy(), yr) < TOL_STEP


def _perturbed_pair(sc, seed=3):
    """GPU sim + oracle with non-trivial v, C and stress so every P2G term is exercised."""
    rng = np.random.default_rng(seed)
    x0, v0, vol, mass = sc.particles()
    n = sc.n_particles
    v0 = (0.1 * rng.normal(size=(n, 3))).astype(np.float32)
    Cm = (0.5 * rng.normal(size=(n, 9))).astype(np.float32)
    tau = (1e3 * rng.normal(size=(n, 9))).astype(np.float32)
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    sim.load_C_from_tensor(torch.from_numpy(Cm))
    sim.load_uvstress_from_tensor(torch.zeros(n, 3), torch.from_numpy(v0), torch.from_numpy(tau))
    ref = oracle_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    ref64 = oracle_sim(sc, bits=64, x0=x0, v0=v0, vol=vol, mass=mass)
    for r in (ref, ref64):
        r.C[:] = Cm
        r.stress[:] = tau
    return sim, ref, ref64


def test_p2g_grid_matches_oracle(cuda):
    sc = S.small_column(8192, 32)
    sim, ref, ref64 = _perturbed_pair(sc)
    e = sim._engine
    e.stage("sort")
    e.stage("p2g", dt=sc.dt)
    gm, gvin, _ = e.export_grid(0)
    torch.cuda.synchronize()
    ref.stage_p2g(sc.dt)
    assert rel(gm.cpu().numpy(), ref.grid_m) < TOL_STEP
    assert rel(gvin.cpu().numpy(), ref.grid_v_in) < TOL_STEP
    # mass conservation (partition of unity)
    assert abs(float(gm.double().sum()) / float(ref.mass.astype(np.float64).sum()) - 1) < 1e-5
    e.stage("grid", time=0.0, dt=sc.dt)
    _, _, gvout = e.export_grid(0)
    torch.cuda.synchronize()
    ref.stage_grid(sc.dt)
    assert rel(gvout.cpu().numpy(), ref.grid_v_out) < TOL_STEP
    e.stage("g2p", dt=sc.dt)
    torch.cuda.synchronize()
    ref.stage_g2p(sc.dt)
    ref64.stage_p2g(sc.dt)
    ref64.stage_grid(sc.dt)
    ref64.stage_g2p(sc.dt)
    errs = compare(sim, ref, fields=("x", "v", "F"))
    assert all(v < TOL_STEP for v in errs.values()), errs
    g = gpu_state(sim)
    for f in ("C", "stress"):
        ok, info = within_fp32_floor(g[f], getattr(ref, f), getattr(ref64, f))
        assert ok, (f, info)


def _step_tol(ref, ref64, fields):
    """1e-5, or 3x the oracle's own float32-vs-float64 spread where that is larger
    (free-fall phases: stress is SVD rounding noise that feeds back into v)."""
    out = {}
    for f in fields:
        a = (ref.x0 + ref.u) if f == "x" else getattr(ref, f)
        b = (ref64.x0 + ref64.u) if f == "x" else getattr(ref64, f)
        out[f] = max(TOL_STEP, 3.0 * rel(a, b))
    return out


@pytest.mark.parametrize("material", ["sand", "metal", "jelly"])
def test_substeps_match_oracle(cuda, material):
    sc = S.small_column(8192, 32, material=material)
    sim = gpu_sim(sc)
    ref = oracle_sim(sc)
    ref64 = oracle_sim(sc, bits=64)
    for k in range(10):
        sim.p2g2p(k, sc.dt)
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
        errs = compare(sim, ref, fields=("x", "v", "F"))
        tol = _step_tol(ref, ref64, errs)
        assert all(errs[f] < tol[f] for f in errs), (k, errs, tol)
    assert sim.check_status() == 0
    if material == "metal":
        assert rel(sim._engine.export(A.FIELD_YIELD).cpu().numpy(), ref.yield_) < TOL_STEP


def test_sand_column_32k_rollout(cuda):
    """The 32,768-particle 64^3 sand column, 200 substeps at dt 1e-4."""
    sc = S.sand_column_32k()
    sim = gpu_sim(sc)
    ref = oracle_sim(sc)
    ref64 = oracle_sim(sc, bits=64)
    for k in range(sc.substeps):
        sim.p2g2p(k, sc.dt)
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
    assert sim.check_status() == 0
    errs = compare(sim, ref)
    errs64 = compare(sim, ref64)
    spread = {f: rel(getattr(ref, f), getattr(ref64, f)) for f in ("v", "C", "F", "stress")}
    print("gpu vs oracle32", errs, "gpu vs oracle64", errs64, "oracle32 vs oracle64", spread)
    # v of the falling column carries the float32 rounding of the stress near F = I: the
    # float32 oracle itself ends about 9e-5 from the float64 rerun, so against it v has the
    # per-substep policy's bar (1e-4, or 3x that floor); against the float64 rerun every
    # field must be within 1e-4
    assert errs["x"] < TOL_ROLLOUT and errs["F"] < TOL_ROLLOUT
    assert errs["v"] < max(TOL_ROLLOUT, 3.0 * spread["v"]), (errs, spread)
    assert all(errs64[f] < TOL_ROLLOUT for f in ("x", "v", "F")), errs64
    g = gpu_state(sim)
    for f in ("stress",):
        ok, info = within_fp32_floor(g[f], getattr(ref, f), getattr(ref64, f), rtol=TOL_ROLLOUT)
        assert ok, (f, info)
    g = sim.mpm_state.particle_x.cpu().numpy()
    assert rel(g, ref.x0 + ref.u) < TOL_ROLLOUT


def test_metal_block_32k_rollout(cuda):
    """A von Mises metal block (E = 1e7, yield stress 1e5, rho 2700, v0 =
    (0, 0, -1), hardening with xi = 0.1) of 32,768 particles on the 64^3
    grid, dropped on the sticky floor: 200 substeps at dt 1e-4 against the
    oracle, x, v and F within the 1e-4 rollout bar, the hardened yield
    stresses within 1e-5 (engine_stress/mpm_utils.py:59-84, :36-43)."""
    sc = S.Scene("metal_block_32k", 32768, 64, 1.0, (0.4, 0.4, 0.05), (0.6, 0.6, 0.65), "metal", 1e7, 0.3,
                 30.0, 2700.0, (0.0, 0.0, -9.8), 1e-4, 200, yield_stress=1e5, hardening=1, xi=0.1,
                 v0=(0.0, 0.0, -1.0), seed=3)
    sim = gpu_sim(sc)
    ref = oracle_sim(sc)
    ref64 = oracle_sim(sc, bits=64)
    for k in range(sc.substeps):
        sim.p2g2p(k, sc.dt)
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
    assert sim.check_status() == 0
    errs = compare(sim, ref, fields=("x", "v", "F"))
    errs64 = compare(sim, ref64, fields=("x", "v", "F"))
    spread = {f: rel(getattr(ref, f), getattr(ref64, f)) for f in ("v", "F")}
    print("gpu vs oracle32", errs, "gpu vs oracle64", errs64, "oracle32 vs oracle64", spread)
    assert all(e < TOL_ROLLOUT for e in errs.values()), errs
    g = gpu_state(sim)
    assert rel(g["yield_"].ravel(), ref.yield_) < TOL_STEP
    assert (g["yield_"].ravel() > sc.yield_stress * (1 + 1e-6)).sum() > 100  # the impact hardened the block


def test_out_of_domain_particle_is_flagged_not_fatal(cuda):
    sc = S.small_column(1024, 32)
    x0, v0, vol, mass = sc.particles()
    x0[5] = (0.99, 0.5, 0.5)  # base index 31 > n-3: stencil leaves the 32^3 grid
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    sim.p2g2p(0, sc.dt)
    with pytest.raises(MPMStatusError) as ei:
        sim.check_status()
    assert ei.value.bits & A.ST_OUT_OF_DOMAIN
    # the particle is frozen, the rest advanced normally
    sim.on_error = "ignore"
    ref = oracle_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    ref64 = oracle_sim(sc, bits=64, x0=x0, v0=v0, vol=vol, mass=mass)
    ref.p2g2p(sc.dt)
    ref64.p2g2p(sc.dt)
    errs = compare(sim, ref, fields=("x", "v", "F"))
    tol = _step_tol(ref, ref64, errs)
    assert all(errs[f] < tol[f] for f in errs), (errs, tol)


def test_cfl_violation_flagged(cuda):
    sc = S.small_column(1024, 32)
    x0, v0, vol, mass = sc.particles()
    v0[:] = (0.0, 0.0, -400.0)  # dx/dt = (1/32)/1e-4 = 312.5
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    sim.p2g2p(0, sc.dt)
    with pytest.raises(MPMStatusError) as ei:
        sim.check_status()
    assert ei.value.bits & A.ST_CFL


@pytest.mark.parametrize("n", [0, 1, 33])
def test_tiny_particle_counts(cuda, n):
    sc = S.small_column(max(n, 1), 16)
    x0, v0, vol, mass = sc.particles()
    x0, v0, vol, mass = x0[:n], v0[:n], vol[:n], mass[:n]
    sc.n_particles = n
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    for k in range(3):
        sim.p2g2p(k, sc.dt)
    assert sim.check_status() == 0
    if n:
        ref = oracle_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
        ref64 = oracle_sim(sc, bits=64, x0=x0, v0=v0, vol=vol, mass=mass)
        for _ in range(3):
            ref.p2g2p(sc.dt)
            ref64.p2g2p(sc.dt)
        errs = compare(sim, ref, fields=("x", "v", "F"))
        tol = _step_tol(ref, ref64, errs)
        assert all(errs[f] < tol[f] for f in errs), (errs, tol)


@pytest.mark.parametrize("chunk", [32, 64, 128, 256])
def test_chunk_size_does_not_change_results(cuda, chunk):
    sc = S.small_column(4096, 32)
    sim = gpu_sim(sc, chunk_size=chunk)
    ref = oracle_sim(sc)
    ref64 = oracle_sim(sc, bits=64)
    for k in range(6):
        sim.p2g2p(k, sc.dt)
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
    errs = compare(sim, ref, fields=("x", "v", "F"))
    tol = _step_tol(ref, ref64, errs)
    assert all(errs[f] < tol[f] for f in errs), (errs, tol)


def _dev_norm_and_trace(tau):
    """Per particle: Frobenius norm of the deviator and the trace of (n, 9) matrices."""
    t = tau.reshape(-1, 3, 3).astype(np.float64)
    t = 0.5 * (t + t.transpose(0, 2, 1))
    tr = np.trace(t, axis1=1, axis2=2)
    dev = t - tr[:, None, None] / 3.0 * np.eye(3)
    return np.sqrt((dev * dev).sum(axis=(1, 2))), tr


@pytest.mark.parametrize("name", ["sand_column_1m", "metal_block_1m"])
def test_full_size_workload(cuda, name):
    """The 1,048,576-particle, 128^3 workloads at full size and full length.

    20 substeps in lockstep with the float32 oracle at the per-substep
    tolerance, then the rest of the 1,000 substeps on the GPU alone, checked
    through properties that hold at any size: no status bits, finite state,
    every particle inside the domain, the returned stress inside the yield
    surface of its material (Drucker-Prager: |dev tau| + alpha tr tau <= 0;
    von Mises: |dev 2 mu log(sigma)| <= yield stress), and the grid mass of a
    fresh P2G equal to the particles' total mass (partition of unity)."""
    sc = getattr(S, name)()
    sim = gpu_sim(sc)
    ref = oracle_sim(sc)
    ref64 = oracle_sim(sc, bits=64)
    lockstep = 20
    for k in range(lockstep):
        sim.p2g2p(k, sc.dt)
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
        errs = compare(sim, ref, fields=("x", "v", "F"))
        tol = _step_tol(ref, ref64, errs)
        assert all(errs[f] < tol[f] for f in errs), (k, errs, tol)
    g = gpu_state(sim)
    ok, info = within_fp32_floor(g["stress"], ref.stress, ref64.stress)
    assert ok, info
    del ref, ref64

    for k in range(lockstep, sc.substeps):
        sim.p2g2p(k, sc.dt)
    assert sim.check_status() == 0
    g = gpu_state(sim)
    for f in ("x", "v", "F", "stress"):
        assert np.isfinite(g[f]).all(), f
    assert (g["x"] > 0).all() and (g["x"] < sc.grid_lim).all()
    assert np.abs(g["u"]).max() > 1e-3  # the material moved
    mu = sc.E / (2 * (1 + sc.nu))
    if sc.material == "sand":
        alpha = float(np.sqrt(2.0 / 3.0) * 2 * np.sin(np.radians(sc.friction_angle))
                      / (3 - np.sin(np.radians(sc.friction_angle))))
        dn, tr = _dev_norm_and_trace(g["stress"])
        scale = np.sqrt(dn * dn + tr * tr / 3.0)
        assert scale.max() > 1e3  # gravity loaded the column
        assert (dn + alpha * tr <= 1e-4 * scale + 1.0).all(), float((dn + alpha * tr - 1e-4 * scale).max())
    else:
        sig = np.linalg.svd(g["F"].reshape(-1, 3, 3).astype(np.float64), compute_uv=False)
        eps = np.log(np.maximum(sig, 0.01))
        dev = eps - eps.mean(axis=1, keepdims=True)
        vm = 2 * mu * np.sqrt((dev * dev).sum(axis=1))
        ys = g["yield_"].ravel().astype(np.float64)
        assert vm.max() > 0.5 * sc.yield_stress  # the impact yielded the block
        assert (vm <= ys * (1 + 1e-3)).all(), float((vm / ys).max())
    e = sim._engine
    e.stage("sort")
    e.stage("p2g", dt=sc.dt)
    gm, _, _ = e.export_grid(0)
    mass = sc.particles()[3].astype(np.float64).sum()
    assert abs(float(gm.double().sum()) / mass - 1) < 1e-5


def test_fused_uvstress_transfers_match_per_field(cuda):
    """mpm_load_uvstress / mpm_export_uvFstress (one pass each, host or device
    buffers) against the per-field mpm_load / mpm_export, on a state whose
    sorted order differs from the user order; the C words sharing record
    quads with v and stress stay untouched."""
    sc = S.small_column(4096, 32)
    sim = gpu_sim(sc)
    for k in range(3):
        sim.p2g2p(k, sc.dt)
    e = sim._engine
    n = sc.n_particles
    rng = np.random.default_rng(5)
    u = torch.from_numpy(1e-3 * rng.normal(size=(n, 3)).astype(np.float32))
    v = torch.from_numpy(rng.normal(size=(n, 3)).astype(np.float32))
    tau = torch.from_numpy(1e3 * rng.normal(size=(n, 3, 3)).astype(np.float32))
    C0 = e.export(A.FIELD_C).clone()
    e.load_uvstress(*(t.reshape(-1).contiguous().pin_memory() for t in (u, v, tau)))
    per = [e.export(f) for f in (A.FIELD_U, A.FIELD_V, A.FIELD_F_DISP, A.FIELD_STRESS)]
    assert torch.equal(per[0].cpu(), u.reshape(-1))
    assert torch.equal(per[1].cpu(), v.reshape(-1))
    assert torch.equal(per[3].cpu(), tau.reshape(-1))
    assert torch.equal(e.export(A.FIELD_C), C0)
    host = tuple(torch.empty(n * c, dtype=torch.float32).pin_memory() for c in (3, 3, 9, 9))
    e.export_uvFstress(host)
    for a, b in zip(host, per):
        assert torch.equal(a, b.cpu())
    for a, b in zip(e.export_uvFstress(), per):
        assert torch.equal(a, b)
    for t in host:
        t.zero_()
    e.export_uvFstress(host, wait=False)  # copies only enqueued
    e.sync_transfers()
    for a, b in zip(host, per):
        assert torch.equal(a, b.cpu())
    e.load_uvstress(2 * u.to(cuda), 2 * v.to(cuda), 2 * tau.to(cuda))
    uu, vv, _, ss = e.export_uvFstress()
    assert torch.equal(uu.cpu(), 2 * u.reshape(-1)) and torch.equal(vv.cpu(), 2 * v.reshape(-1))
    assert torch.equal(ss.cpu(), 2 * tau.reshape(-1))
    # the simulator's reference-named methods go through the same calls
    su, sv, sfd, sst = sim.export_uvFstress_from_warp()
    assert torch.equal(su.reshape(-1), uu) and torch.equal(sst.reshape(-1), ss)


def test_particle_leaving_the_domain_is_carried_over(cuda):
    """A particle that flies out of the grid is frozen there (skipped by P2G
    and G2P, flagged out-of-domain) and its record is carried over by every
    later substep's re-sort, while the others keep matching the oracle."""
    sc = S.small_column(1024, 32)
    x0, v0, vol, mass = sc.particles()
    x0[5] = (0.94, 0.5, 0.5)   # stencil base 29 = n - 3: the last valid cell
    v0[5] = (5.0, 0.0, 0.0)    # leaves after ~26 substeps (dx / dt = 312.5 m/s)
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    sim.on_error = "ignore"
    ref = oracle_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    ref64 = oracle_sim(sc, bits=64, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    bits = 0
    for k in range(40):
        sim.p2g2p(k, sc.dt)
        bits |= sim._engine.status()
        sim._engine.clear_status()
        ref.p2g2p(sc.dt)
        ref64.p2g2p(sc.dt)
    assert bits & A.ST_OUT_OF_DOMAIN
    assert not bits & A.ST_INTERNAL, bits
    errs = compare(sim, ref, fields=("x", "v", "F"))
    tol = _step_tol(ref, ref64, errs)
    assert all(errs[f] < tol[f] for f in errs), (errs, tol)
    g = gpu_state(sim)
    assert g["x"][5, 0] * 32 - 0.5 >= 30  # outside, where it stopped
    assert abs(g["x"][5, 0] - float((ref.x0 + ref.u)[5, 0])) < 1e-6


def test_tilted_timed_colliders_match_oracle(cuda):
    """A tilted slip plane (normal not along an axis, friction given) that is
    active only for substeps 3-7, plus the bounding box from substep 2 on:
    every node below the plane is zeroed while it is active (the reference
    zeroes for all surface types, engine_stress/mpm_solver_warp.py:449), and
    the windows switch on the same substeps as the oracle's."""
    sc = S.small_column(8192, 32)
    dt = sc.dt
    x0, v0, vol, mass = sc.particles()
    plane = dict(point=(0.5, 0.5, 0.32), normal=(0.3, -0.2, 1.0), surface="slip", friction=0.1,
                 start_time=2.5 * dt, end_time=6.5 * dt)
    box = dict(start_time=1.5 * dt, end_time=999.0)
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    sim.add_surface_collider(**plane)
    sim.add_bounding_box(**box)
    m = O.make_model(sc.n_grid, sc.grid_lim, material=sc.material, E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity)
    cols = [O.surface_collider(**plane), O.bounding_box(**box)]
    ref = O.OracleSim(m, x0, mass, vol, v0, bits=32, colliders=cols)
    ref64 = O.OracleSim(m, x0, mass, vol, v0, bits=64, colliders=cols)
    moved = []
    for k in range(10):
        sim.p2g2p(k, dt)
        ref.p2g2p(dt)
        ref64.p2g2p(dt)
        errs = compare(sim, ref, fields=("x", "v", "F"))
        tol = _step_tol(ref, ref64, errs)
        assert all(errs[f] < tol[f] for f in errs), (k, errs, tol)
        moved.append(float(np.abs(gpu_state(sim)["v"]).max()))
    assert sim.check_status() == 0
    assert max(moved) > 0.0


# the reference's other grid boundary conditions (mpm_solver_warp.py:527-720):
# (simulator method, oracle factory, keyword arguments); windows end between
# substeps so the reset rules run too
_EXTENDED_COLLIDERS = {
    "velocity_plane": ("set_velocity_on_infinite_plane", "velocity_plane",
                       dict(point=(0.5, 0.5, 0.3), normal=(0.2, 0.1, 1.0), velocity=(0.0, 0.1, 0.4),
                            threshold=0.03, start_time=0.0, end_time=6.5e-4, reset=1)),
    "circle_column": ("set_column_moving_as_circle", "circle_column",
                      dict(R=0.1, radius=0.08, height=0.5, v_scale=0.5, start_time=0.0, end_time=999.0)),
    "rotating_disk": ("set_rotation_on_disk", "rotating_disk",
                      dict(point=(0.5, 0.5, 0.45), normal=(1.0, 0.15, 0.1), radius=0.12, width=0.05,
                           v_scale=5.0, start_time=1.5e-4, end_time=6.5e-4, reset=1)),
    "velocity_cube": ("set_velocity_on_cube", "velocity_cube",
                      dict(point=(0.5, 0.5, 0.4), width=0.06, velocity=(0.3, 0.0, 0.2), start_time=0.0,
                           end_time=6.5e-4, reset=1)),
    "sphere_leader": ("add_sphere_leader", "sphere_leader",
                      dict(center=(0.45, 0.5, 0.5), radius=0.07, velocity=(0.5, 0.0, -0.3), start_time=0.0,
                           end_time=999.0)),
}


@pytest.mark.parametrize("name", sorted(_EXTENDED_COLLIDERS))
def test_extended_colliders_match_oracle(cuda, name):
    """Each of the reference's other colliders, moving ones included, over 10
    substeps against the oracle; halfway through a bounding box is added,
    which re-uploads the scene table and must keep the moving collider where
    the device advanced it."""
    method, factory, kw = _EXTENDED_COLLIDERS[name]
    sc = S.small_column(8192, 32)
    dt = sc.dt
    x0, v0, vol, mass = sc.particles()
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass, colliders=False)
    getattr(sim, method)(**kw)
    m = O.make_model(sc.n_grid, sc.grid_lim, material=sc.material, E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity)
    refs = [O.OracleSim(m, x0, mass, vol, v0, bits=b, colliders=[getattr(O, factory)(**kw)]) for b in (32, 64)]
    for k in range(10):
        if k == 5:
            sim.add_bounding_box()
            for r in refs:
                r.colliders.append(O.bounding_box())
        sim.p2g2p(k, dt)
        for r in refs:
            r.p2g2p(dt)
        errs = compare(sim, refs[0], fields=("x", "v", "F"))
        tol = _step_tol(refs[0], refs[1], errs)
        assert all(errs[f] < tol[f] for f in errs), (name, k, errs, tol)
    assert sim.check_status() == 0
    col = sim._params.colliders[0]
    sim._engine.update_scenes()  # reads the device-side point back
    ref_col = refs[0].colliders[0]
    assert np.allclose(col.point, tuple(ref_col.point), rtol=0, atol=1e-6), (col.point, tuple(ref_col.point))


def test_disk_with_small_normal_x_is_refused(cuda):
    sc = S.small_column(64, 16)
    sim = gpu_sim(sc)
    with pytest.raises(ValueError):
        sim.set_rotation_on_disk((0.5, 0.5, 0.5), (0.05, 1.0, 0.0), 0.1, 0.05, 1.0)


def test_moving_collider_advances_inside_a_graph(cuda):
    """A moving collider (sphere leader, open window) stepped eagerly and by
    replaying a captured 4-substep graph: same particles, same final point."""
    sc = S.small_column(8192, 32)
    dt = sc.dt
    kw = dict(center=(0.45, 0.5, 0.5), radius=0.07, velocity=(0.5, 0.0, -0.3))
    sims = []
    for _ in range(2):
        sim = gpu_sim(sc, colliders=False)
        sim.add_sphere_leader(**kw)
        sim.p2g2p(0, dt)
        sims.append(sim)
    eager, graphed = sims
    for k in range(1, 9):
        eager.p2g2p(k, dt)
    g = graphed._engine.graph(4, float(graphed.time), dt)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    a, b = gpu_state(eager), gpu_state(graphed)
    for f in ("x", "v", "F"):
        assert rel(b[f], a[f]) < 1e-5, (f, rel(b[f], a[f]))
    for sim in sims:
        sim._engine.update_scenes()
    assert np.allclose(graphed._params.colliders[0].point, eager._params.colliders[0].point, rtol=0, atol=1e-7)
    moved = np.array(eager._params.colliders[0].point) - np.array(kw["center"])
    assert np.allclose(moved, 9 * dt * np.array(kw["velocity"]), atol=1e-6)


def test_large_scene_properties(cuda):
    """32M particles on a 256^3 grid (about 13 GB of state and workspace):
    the 64-bit record offsets and the sort's block tables at scale.  Three
    substeps, then size-independent checks: no status bits, finite state,
    grid mass equal to particle mass, and the particles that fall freely
    (above the column's load path, first substeps) at 3 g dt."""
    sc = S.Scene("sand_column_32m", 32 * 1024 * 1024, 256, 1.0, (0.35, 0.35, 0.05), (0.65, 0.65, 0.85),
                 "sand", 2e5, 0.3, 30.0, 2200.0, (0.0, 0.0, -9.8), 2.5e-5, 3, seed=5)
    sim = gpu_sim(sc)
    for k in range(sc.substeps):
        sim.p2g2p(k, sc.dt)
    assert sim.check_status() == 0
    e = sim._engine
    u = e.export(A.FIELD_U).view(-1, 3)
    assert bool(torch.isfinite(u).all()) and bool(torch.isfinite(e.export(A.FIELD_STRESS)).all())
    # the top of the column is still in free fall: v_z = 3 g dt after three substeps
    top = e.export(A.FIELD_X).view(-1, 3)[:, 2] > 0.8
    vz = e.export(A.FIELD_V).view(-1, 3)[top, 2].double()
    expect = -9.8 * sc.dt * 3.0
    assert int(top.sum()) > 100000 and abs(float(vz.median()) / expect - 1.0) < 1e-4, (float(vz.median()), expect)
    e.stage("sort")
    e.stage("p2g", dt=sc.dt)
    gm, _, _ = e.export_grid(0)
    mass = float(sc.density * sc.box_volume)
    assert abs(float(gm.double().sum()) / mass - 1.0) < 1e-4
