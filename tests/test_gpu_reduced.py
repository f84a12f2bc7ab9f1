"""GPU-vs-oracle parity of the reduced sampled-quadrature substep
(MPM_Simulator_WARP.p2g2p_reduced, engine_stress/mpm_solver_warp.py:207-227;
kernels engine_stress/mpm_utils.py:318-471), called through the C ABI.

Each case runs a few plain substeps first (so v, F and u are not trivial),
copies the GPU state into the oracle, then runs the reduced stage on both.

Tolerances:
  mark arrays, and F = F_disp + I of the marked particles: bit-exact
  grid_m: 1e-5 relative L2 (float32 atomic order)
  grid_v_in, grid_v_out and the sample gather (u, v, F, F_disp, yield):
  1e-5 relative L2, or within the float32 noise floor the oracle measures
  on itself (GPU vs float32 oracle no further than 3x float32 oracle vs its
  float64 rerun): the force term carries the stress of an SVD of F near I,
  whose float32 rounding is a large relative error of a small stress, in
  the reference as here
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300.engine import MPMStatusError

from helpers import compare, gpu_sim, gpu_state, oracle_sim, rel, within_fp32_floor

pytestmark = pytest.mark.gpu

TOL = 1e-5
EYE = np.eye(3, dtype=np.float32).reshape(1, 9)


def _pair(material="sand", n=8192, n_grid=32, steps=3, seed=0, n_samples=64, plane=False, **kw):
    sc = S.small_column(n, n_grid, material=material, seed=seed, **kw)
    sim = gpu_sim(sc)
    sim.set_parameters(density=sc.density)
    refs = [oracle_sim(sc), oracle_sim(sc, bits=64)]
    for r in refs:
        r.density[:] = sc.density
    if plane:  # a moving collider that writes nodes with and without mass
        sim.set_velocity_on_infinite_plane((0.0, 0.0, 0.5), (0.0, 0.0, 1.0), (0.5, 0.0, 0.0), 0.05)
        for r in refs:
            r.colliders.append(O.velocity_plane((0.0, 0.0, 0.5), (0.0, 0.0, 1.0), (0.5, 0.0, 0.0), 0.05))
    for k in range(steps):
        sim.p2g2p(k, sc.dt)
        for r in refs:
            r.p2g2p(sc.dt)
    sim.check_status()
    # both oracles continue from the GPU's state, so the reduced stage is compared alone
    g = gpu_state(sim)
    rng = np.random.default_rng(seed + 7)
    sample = rng.choice(n, n_samples, replace=False).astype(np.int32)
    sim.load_sample_particle_index_from_tensor(torch.from_numpy(sample))
    for r in refs:
        r.u[:] = g["u"]
        r.v[:] = g["v"]
        r.F[:] = g["F"]
        r.C[:] = g["C"]
        r.stress[:] = g["stress"]
        r.F_disp[:] = g["F"] - EYE
        r.yield_[:] = g["yield_"].ravel()
        r.sample_particle_index_short = sample
    ref, ref64 = refs
    ref.twin = ref64
    return sc, sim, ref


def _reduced(sim, ref, dt, step=0):
    sim.p2g2p_reduced(step, dt)
    ref.p2g2p_reduced(dt)
    ref.twin.p2g2p_reduced(dt)


def _close(gpu, o32, o64, what):
    ok, info = within_fp32_floor(gpu, o32, o64, rtol=TOL)
    assert ok, (what, info)


def _grids(sim):
    st = sim.mpm_state
    return {k: getattr(st, k).cpu().numpy() for k in
            ("grid_m", "grid_v_in", "grid_v_out", "neighboring_cells", "neighboring_cells_grid_v")}


def _check_grid(sim, ref):
    g = _grids(sim)
    assert np.array_equal(g["neighboring_cells"], ref.neighboring_cells)
    assert g["neighboring_cells"].any()
    assert rel(g["grid_m"], ref.grid_m) <= TOL
    for f in ("grid_v_in", "grid_v_out"):
        _close(g[f], getattr(ref, f), getattr(ref.twin, f), f)
    # no mass and no velocity outside the marked cells' stencils: same zero pattern of mass
    assert np.array_equal(g["grid_m"] > 0, ref.grid_m > 0)


@pytest.mark.parametrize("material", ["sand", "metal", "jelly"])
def test_p2g2p_reduced_matches_oracle(cuda, material):
    sc, sim, ref = _pair(material)
    _reduced(sim, ref, sc.dt)
    sim.check_status()
    assert ref.status.value == 0
    _check_grid(sim, ref)
    # marked particles took F = F_disp + I, bit for bit; the others kept F
    gF = gpu_state(sim)["F"]
    assert np.array_equal(gF, ref.F)
    assert sim.time == pytest.approx(ref.time)


def test_colliders_sweep_every_node_of_the_dense_grid(cuda):
    sc, sim, ref = _pair("sand", plane=True)
    _reduced(sim, ref, sc.dt)
    sim.check_status()
    _check_grid(sim, ref)
    gv = sim.mpm_state.grid_v_out.cpu().numpy()
    # the plane's slab (iz = 15, 16, 17) moves at 0.5 m/s whether or not a node holds mass
    slab = gv[..., 0] == np.float32(0.5)
    assert slab.sum() == 3 * 32 * 32 and slab[:, :, 15:18].all()
    assert np.array_equal(slab, ref.grid_v_out[..., 0] == np.float32(0.5))
    # the moving plane advanced on the device, as the oracle's host update does
    _reduced(sim, ref, sc.dt, 1)
    sim.check_status()
    _check_grid(sim, ref)


@pytest.mark.parametrize("material,kw", [("sand", {}), ("jelly", {}),
                                         ("metal", dict(hardening=1, xi=0.5, yield_stress=10.0, v0_sigma=0.5))])
def test_g2p_sample_matches_oracle(cuda, material, kw):
    sc, sim, ref = _pair(material, **kw)
    _reduced(sim, ref, sc.dt)
    y_before = gpu_state(sim)["yield_"].ravel()
    sim.g2p_sample(sc.dt)
    ref.g2p_sample(sc.dt)
    ref.twin.g2p_sample(sc.dt)
    sim.check_status()
    assert ref.status.value == 0
    g = gpu_state(sim)
    idx = ref.sample_particle_index_short
    r64 = ref.twin
    _close(g["v"][idx], ref.v[idx], r64.v[idx], "v")
    _close(g["x"][idx], (ref.x0 + ref.u)[idx], (r64.x0 + r64.u)[idx], "x")
    _close(g["F"][idx], ref.F[idx], r64.F[idx], "F")
    fd = sim.mpm_state.particle_F_disp.cpu().numpy().reshape(-1, 9)
    _close(fd[idx], ref.F_disp[idx], r64.F_disp[idx], "F_disp")
    assert np.array_equal(fd[idx], g["F"][idx] - EYE)
    rest = np.setdiff1d(np.arange(sim.n_particles), idx)
    assert np.array_equal(g["u"][rest], ref.u[rest])
    _close(g["yield_"].ravel(), ref.yield_, r64.yield_, "yield")
    if material == "metal":  # only yield words of list positions s < n_samples move (:464)
        changed = np.nonzero(g["yield_"].ravel() != y_before)[0]
        assert changed.size > 0 and changed.max() < idx.size
    # the sample points moved: the next plain substep re-sorts and still matches
    sim.p2g2p(0, sc.dt)
    ref.p2g2p(sc.dt)
    r64.p2g2p(sc.dt)
    sim.check_status()
    g = gpu_state(sim)
    _close(g["x"], ref.x0 + ref.u, r64.x0 + r64.u, "x after a plain substep")
    for f in ("v", "F"):
        _close(g[f], getattr(ref, f), getattr(r64, f), f + " after a plain substep")


def test_experiment_for_C_marks(cuda):
    sc, sim, ref = _pair("sand")
    _reduced(sim, ref, sc.dt)
    got = sim.experiment_for_C().cpu().numpy()
    want = ref.experiment_for_C()
    assert np.array_equal(got, want) and got.sum() > ref.neighboring_cells.sum()
    # marks add up across calls until the next p2g2p_reduced clears them
    other = np.array([1, 2, 3], np.int32)
    sim.load_sample_particle_index_from_tensor(torch.from_numpy(other))
    ref.sample_particle_index_short = other
    assert np.array_equal(sim.experiment_for_C().cpu().numpy(), ref.experiment_for_C())


def test_loaded_F_disp_feeds_the_reduced_p2g(cuda):
    """load_uvF_from_tensor sets F_disp only; p2g_sample_all reads it (:364)."""
    sc, sim, ref = _pair("jelly", steps=1)
    n = sim.n_particles
    rng = np.random.default_rng(3)
    u = gpu_state(sim)["u"].astype(np.float32)
    v = rng.normal(0, 0.2, (n, 3)).astype(np.float32)
    fd = (0.03 * rng.normal(size=(n, 9))).astype(np.float32)
    sim.load_uvF_from_tensor(torch.from_numpy(u), torch.from_numpy(v), torch.from_numpy(fd))
    for r in (ref, ref.twin):
        r.u[:], r.v[:], r.F_disp[:] = u, v, fd
    _reduced(sim, ref, sc.dt)
    sim.check_status()
    _check_grid(sim, ref)
    assert np.array_equal(gpu_state(sim)["F"], ref.F)


def test_empty_sample_list(cuda):
    sc, sim, ref = _pair("sand")
    sim.load_sample_particle_index_from_tensor(torch.empty(0, dtype=torch.int32))
    ref.sample_particle_index_short = ref.twin.sample_particle_index_short = np.empty(0, np.int32)
    _reduced(sim, ref, sc.dt)
    sim.check_status()
    g = _grids(sim)
    assert not g["neighboring_cells"].any() and not g["grid_m"].any() and not g["grid_v_out"].any()
    assert not ref.grid_v_out.any()


def test_bad_sample_index_raises(cuda):
    sc, sim, ref = _pair("sand")
    sim.load_sample_particle_index_from_tensor(torch.tensor([0, sim.n_particles], dtype=torch.int32))
    sim.p2g2p_reduced(0, sc.dt)
    with pytest.raises(MPMStatusError):
        sim.check_status()


def test_abi_checks(cuda):
    """A dense grid of the wrong size is refused on the device (status bit, no
    write); a multi-scene plan is refused on the host."""
    sc, sim, ref = _pair("sand")
    eng = sim.engine
    rg = sim._reduced_grid()
    rg.f_disp = sim._f_disp_state()
    g = rg.struct(eng)
    g.n_grid = sc.n_grid - 1
    lib = A.load()
    assert lib.mpm_p2g2p_reduced(C.byref(eng.buf), C.byref(g), 0.0, sc.dt, eng.stream) == 0
    torch.cuda.synchronize()
    assert eng.status() & A.ST_BAD_INPUT
    assert not rg.grid_v_out.any() and not rg.neighboring_cells.any()
    eng.clear_status()
    from reduced_mpm_stress_training_gb300.batched import BatchedMPM

    b = BatchedMPM([S.small_column(1024, 16), S.small_column(2048, 16)], chunk_size=128)
    assert lib.mpm_p2g2p_reduced(C.byref(b.engine.buf), C.byref(g), 0.0, sc.dt, eng.stream) == A.MPM_ERR_ARG
    with pytest.raises(ValueError):
        b.engine.p2g2p_reduced(rg, 0.0, sc.dt)


@pytest.mark.slow
def test_full_size_properties(cuda):
    """1,048,576 sand particles on a 128^3 grid with 4096 samples: the grid
    holds exactly the marked particles' mass, velocity is nonzero only on
    marked nodes, and the mark count matches the sample neighbourhoods."""
    sc = S.sand_column_1m()
    sim = gpu_sim(sc)
    sim.set_parameters(density=sc.density)
    for k in range(2):
        sim.p2g2p(k, sc.dt)
    n = sc.n_particles
    rng = np.random.default_rng(11)
    sample = torch.from_numpy(rng.choice(n, 4096, replace=False).astype(np.int32))
    sim.load_sample_particle_index_from_tensor(sample)
    sim.p2g2p_reduced(0, sc.dt)
    sim.check_status()
    e = sim.engine
    x = e.export(A.FIELD_X).reshape(n, 3)
    base = torch.trunc(x * np.float32(sc.n_grid) - 0.5).long()
    st = sim.mpm_state
    mask = st.neighboring_cells
    marked = mask[base[:, 0], base[:, 1], base[:, 2]] > 0
    mass = e.export(A.FIELD_MASS)
    assert 0 < int(marked.sum()) < n
    assert float(st.grid_m.double().sum()) == pytest.approx(float(mass[marked].double().sum()), rel=1e-5)
    moving = (st.grid_v_out != 0).any(-1)
    assert not bool((moving & (mask == 0)).any())
    # every sample's 5^3 neighbourhood is marked (the column is far from the walls)
    sb = base[sample.long().to(base.device)]
    for d in (-2, 2):
        assert bool((mask[sb[:, 0] + d, sb[:, 1] + d, sb[:, 2] + d] == 1).all())
