"""Frame files on the GPU path (engine_stress/mpm_solver_warp.py:129-153,
268-404): save_data_at_frame's arrays from mpm_export_frame bit-match the
per-field exports in the frame's transposed layout; load_from_sampling and
load_uvFstress_from_h5 restore what was written."""
import numpy as np
import pytest
import torch

from reduced_mpm_stress_training_gb300 import MPM_Simulator_WARP
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import frames as FR
from reduced_mpm_stress_training_gb300 import scenarios as S

from helpers import gpu_sim, gpu_state

pytestmark = pytest.mark.gpu

EYE = np.eye(3, dtype=np.float32).reshape(1, 9)


def test_save_data_at_frame_matches_the_state(cuda, tmp_path):
    sc = S.small_column(4096, 32)
    sim = gpu_sim(sc)
    for k in range(3):
        sim.p2g2p(k, sc.dt)
    sim.check_status()
    d = str(tmp_path / "seq")
    sim.save_data_at_frame(d, 3, save_visual_F=True)
    path = FR.frame_filename(d, 3)
    got = FR.read_frame(path)
    assert list(got) == ["x", "q", "time", "masses", "f_tensor", "stress", "v", "mu", "C"]
    g = gpu_state(sim)
    n = sim.n_particles
    e = sim.engine
    x0 = e.export(A.FIELD_X_INITIAL).reshape(n, 3).cpu().numpy()
    mass = e.export(A.FIELD_MASS).cpu().numpy()
    assert np.array_equal(got["x"], x0.T) and np.array_equal(got["q"], g["u"].T)
    assert np.array_equal(got["masses"], mass.reshape(1, n))
    assert np.array_equal(got["f_tensor"], (g["F"] - EYE).T)
    assert np.array_equal(got["stress"], g["stress"][:, list(FR.STRESS_COMPONENTS)].T)
    assert np.array_equal(got["v"], g["v"].T) and np.array_equal(got["C"], g["C"].T)
    assert got["time"].shape == (1, 1) and got["time"][0, 0] == sim.time
    assert np.array_equal(got["mu"], np.full((1, n), sc.friction_angle))
    assert got["x"].dtype == np.float32 and got["time"].dtype == np.float64
    lines = open(path[: path.rindex(".")] + ".obj").read().splitlines()
    x = g["x"]
    assert len(lines) == n
    assert lines[7] == "v " + " ".join(str(c) for c in x[7]) + " 0.0 0.0 0.0"
    vis = open(d + "/visualF_f_0000000003.obj").read().splitlines()
    assert len(vis) == n and vis[0].startswith("v " + str(x0[0][0]) + " ") and vis[0].endswith(" 0 0")
    # a fresh simulator takes u, v and the stress back from the frame
    other = gpu_sim(sc)
    other.load_uvFstress_from_h5(path)
    h = gpu_state(other)
    assert np.array_equal(h["u"], g["u"]) and np.array_equal(h["v"], g["v"])
    assert np.array_equal(h["stress"].reshape(n, 3, 3),
                          FR.stress_from_components(g["stress"][:, list(FR.STRESS_COMPONENTS)]))


def test_load_from_sampling(cuda, tmp_path):
    rng = np.random.default_rng(0)
    n = 3000
    x = rng.uniform([0.4, 0.4, 0.1], [0.6, 0.6, 0.5], (n, 3)).astype(np.float32)
    vol = np.full(n, 0.008 * 0.4 / n, np.float32)
    rho = np.full(n, 2200.0, np.float32)
    f = (0.01 * rng.normal(size=(n, 3, 3))).astype(np.float32)
    path = str(tmp_path / "sampling.npz")
    FR.write_frame(path, {"x": x.T, "q": np.zeros((3, n), np.float32), "masses": (rho * vol).reshape(1, n),
                          "particle_volume": vol.reshape(1, n), "particle_density": rho.reshape(1, n),
                          "f_tensor": f})
    sim = MPM_Simulator_WARP(10, n_grid=16, device=cuda)
    sim.load_from_sampling(path, n_grid=32)
    assert sim.n_particles == n and sim.mpm_model.n_grid == 32
    st = sim.mpm_state
    assert np.array_equal(st.particle_x_initial.cpu().numpy(), x)
    assert np.array_equal(st.particle_mass.cpu().numpy(), rho * vol)
    assert np.array_equal(st.particle_vol.cpu().numpy(), vol)
    assert np.array_equal(st.particle_density.cpu().numpy(), rho)
    assert np.array_equal(st.particle_F_disp.cpu().numpy(), f)
    assert np.array_equal(st.particle_F.cpu().numpy().reshape(n, 9), np.tile(EYE, (n, 1)))
    assert not st.particle_v.cpu().numpy().any()
    sim.set_parameters(material="sand", E=2e5, nu=0.3, gravity=(0.0, 0.0, -9.8))
    sim.p2g2p(0, 1e-4)
    sim.check_status()
    with pytest.raises(FileNotFoundError):
        sim.load_from_sampling("/no/such/file.npz")
