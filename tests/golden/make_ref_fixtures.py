"""Generate golden fixtures by running the reference's OWN code.

The reference's solver (engine_stress/mpm_solver_warp.py, mpm_utils.py,
warp_utils.py) is imported unmodified from the reference checkout and run
on the CPU through the test-only Warp stand-in in ``tests/refshim`` (Warp is
not installed and cannot be).  Its decoder NetDec
(offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301) is
imported the same way with a ``pytorch_lightning`` stand-in.

Fixtures written here (NumPy .npz, float32 as the reference computes):

  ref_mpm_<scene>.npz   the initial state and the state after every substep
                        of ``MPM_Simulator_WARP.p2g2p`` (u, v, F, C, stress,
                        yield stress; grid_m, grid_v_in, grid_v_out), for
                        sand from F = I (the generate_sand.py set-up), sand
                        from a deformed state (every Drucker-Prager branch),
                        von Mises metal with hardening, and jelly
  ref_frame_sand.npz    the datasets ``save_data_at_frame`` wrote for the
                        last state of ``sand_column`` (+ its OBJ text)
  ref_netdec.npz        NetDec's state dict, input rows and forward output,
                        ELU and SIREN

The set-up follows the reference's own driver (generate_training_data/
generate_sand.py:15-32): ``load_from_sampling`` of a sampling file (here
written by the ``h5py`` stand-in), ``set_parameters``, a sticky surface
collider under the column and ``add_bounding_box``, then ``p2g2p`` per
substep.  Velocities, C, stress and F are then set through the reference's
loaders (``load_uvF_from_tensor``, ``load_C_from_tensor``,
``load_uvstress_from_tensor``) and, for F, its ``mpm_state.particle_F``
array (the reference has no F loader).  Gravity is the reference's own
-y direction (mpm_utils.py:236), the floor's normal +y.

``random.seed(datetime)`` in NetDec.init_weights (CROMnet_secondary.py:256)
is rejected by Python >= 3.11; the module's ``random`` is given a seed()
that accepts it (the initial weights are replaced by seeded ones anyway).

Run (needs the reference checkout; a few minutes, one core):
    python tests/golden/make_ref_fixtures.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import contextlib
import io
import os
import random
import sys
import tempfile

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(os.path.dirname(HERE), "refshim")
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

# Each scene: particles in a box, material, initial fields.  Grid 16^3 on the
# unit cube, dt 1e-4, g 9.8 along -y; sticky floor plane y = 0.25 and the
# bounding box (3-node walls).  The boxes reach into the wall layers x < 3
# and z >= 13 so the slip walls act.
SCENES = {
    "sand_column": dict(n=1024, material="sand", E=2e5, nu=0.3, phi=30.0, density=2200.0,
                        v_sigma=0.3, v_mean=(0.0, 0.0, 0.0), F_kind=None, C_sigma=0.0,
                        tau_sigma=0.0, substeps=10, seed=11),
    "sand_deformed": dict(n=512, material="sand", E=2e5, nu=0.3, phi=30.0, density=2200.0,
                          v_sigma=0.2, v_mean=(0.0, -0.5, 0.0), F_kind="dp_branches", C_sigma=2.0,
                          tau_sigma=2e3, substeps=8, seed=12),
    "metal_block": dict(n=512, material="metal", E=1e7, nu=0.3, phi=30.0, density=2700.0,
                        v_sigma=0.2, v_mean=(0.0, -1.0, 0.0), F_kind="near_identity", C_sigma=1.0,
                        tau_sigma=1e4, substeps=8, seed=13, yield_stress=1e5, hardening=1, xi=0.5),
    "jelly_block": dict(n=512, material="jelly", E=2e5, nu=0.3, phi=30.0, density=1000.0,
                        v_sigma=0.3, v_mean=(0.0, 0.0, 0.0), F_kind="near_identity", C_sigma=1.0,
                        tau_sigma=1e3, substeps=8, seed=14),
}
N_GRID = 16
GRID_LIM = 1.0
DT = 1e-4
G = 9.8
FLOOR_Y = 0.25
BOX_LO = (0.16, 0.25, 0.30)
BOX_HI = (0.62, 0.65, 0.84)


def _rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                     2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                     2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1).reshape(n, 3, 3)


def initial_F(kind, rng, n):
    if kind is None:
        return np.tile(np.eye(3, dtype=np.float32), (n, 1, 1))
    if kind == "near_identity":
        return (np.eye(3)[None] + 0.02 * rng.normal(size=(n, 3, 3))).astype(np.float32)
    # R1 diag(exp(s)) R2^T with s in [-0.3, 0.1]: compression (cone), expansion
    # (apex) and elastic states all occur
    s = rng.uniform(-0.3, 0.1, size=(n, 3))
    return np.einsum("nij,nj,nkj->nik", _rotations(rng, n), np.exp(s), _rotations(rng, n)).astype(np.float32)


def write_sampling(path, x0, mass, vol, density):
    """The sampling file load_from_sampling reads (mpm_solver_warp.py:135-137)."""
    import h5py  # the stand-in

    n = x0.shape[0]
    f = h5py.File(path, "w")
    f.create_dataset("x", data=x0.T.astype(np.float32))
    f.create_dataset("q", data=np.zeros((3, n), np.float32))
    f.create_dataset("masses", data=mass.reshape(1, n).astype(np.float32))
    f.create_dataset("particle_volume", data=vol.reshape(1, n).astype(np.float32))
    f.create_dataset("particle_density", data=np.full((1, n), density, np.float32))
    f.create_dataset("f_tensor", data=np.zeros((n, 3, 3), np.float32))
    f.close()


def snapshot(sim, with_grid: bool) -> dict:
    st, md = sim.mpm_state, sim.mpm_model
    out = {
        "u": st.particle_u.numpy().copy(), "v": st.particle_v.numpy().copy(),
        "F": st.particle_F.numpy().reshape(-1, 9).copy(), "C": st.particle_C.numpy().reshape(-1, 9).copy(),
        "stress": st.particle_stress.numpy().reshape(-1, 9).copy(),
        "yield": md.yield_stress.numpy().copy(),
    }
    if with_grid:
        out["grid_m"] = st.grid_m.numpy().copy()
        out["grid_v_in"] = st.grid_v_in.numpy().copy()
        out["grid_v_out"] = st.grid_v_out.numpy().copy()
    return out


def run_scene(R, name, cfg, workdir):
    rng = np.random.default_rng(cfg["seed"])
    n = cfg["n"]
    lo, hi = np.array(BOX_LO), np.array(BOX_HI)
    x0 = (lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)
    box_vol = float(np.prod(hi - lo))
    vol = np.full(n, box_vol / n, np.float32)
    mass = (np.float32(cfg["density"]) * vol).astype(np.float32)
    v0 = (np.asarray(cfg["v_mean"]) + cfg["v_sigma"] * rng.normal(size=(n, 3))).astype(np.float32)
    F0 = initial_F(cfg["F_kind"], rng, n)
    C0 = (cfg["C_sigma"] * rng.normal(size=(n, 9))).astype(np.float32)
    tau0 = (cfg["tau_sigma"] * rng.normal(size=(n, 9))).astype(np.float32)
    E, nu = cfg["E"], cfg["nu"]
    mu = E / 2.0 / (1.0 + nu)
    lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)

    sampling = os.path.join(workdir, f"sampling_{name}.h5")
    write_sampling(sampling, x0, mass, vol, cfg["density"])
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        sim = R.MPM_Simulator_WARP(10)
        sim.load_from_sampling("/" + os.path.basename(sampling), n_grid=N_GRID, grid_lim=GRID_LIM)
        kw = dict(material=cfg["material"], mu=mu, lam=lam, friction_angle=cfg["phi"], g=G,
                  density=cfg["density"])
        if cfg["material"] == "metal":
            kw.update(yield_stress=cfg["yield_stress"], hardening=cfg["hardening"], xi=cfg["xi"])
        sim.set_parameters(**kw)
        sim.add_surface_collider((0.0, FLOOR_Y, 0.0), (0.0, 1.0, 0.0), "sticky")
        sim.add_bounding_box()
        u0 = torch.zeros(n, 3)
        sim.load_uvF_from_tensor(u0, torch.from_numpy(v0), torch.from_numpy(F0.reshape(n, 9)) - torch.eye(3).reshape(1, 9))
        sim.load_C_from_tensor(torch.from_numpy(C0))
        sim.load_uvstress_from_tensor(u0, torch.from_numpy(v0), torch.from_numpy(tau0))
        if cfg["F_kind"] is not None:
            sim.mpm_state.particle_F = R.wp.from_numpy(F0, dtype=R.wp.mat33)
        # mass as set_parameters(density=...) computed it (mpm_solver_warp.py:121-124)
        mass = sim.mpm_state.particle_mass.numpy().copy()
        vol = sim.mpm_state.particle_vol.numpy().copy()
        states = [snapshot(sim, with_grid=False)]
        for k in range(cfg["substeps"]):
            with contextlib.redirect_stdout(io.StringIO()):
                sim.p2g2p(k, DT)
            states.append(snapshot(sim, with_grid=True))
            print(f"  {name}: substep {k + 1}/{cfg['substeps']}", flush=True)
        frame = None
        if name == "sand_column":
            fdir = os.path.join(workdir, "frames")
            with contextlib.redirect_stdout(io.StringIO()):
                sim.save_data_at_frame(fdir, 7)
            import h5py

            h = h5py.File(os.path.join(fdir, "h5_f_" + "7".zfill(10) + ".h5"), "r")
            frame = {k: np.asarray(h[k]) for k in h.keys()}
            with open(os.path.join(fdir, "h5_f_" + "7".zfill(10) + ".obj")) as f:
                frame["obj_text"] = np.array(f.read())
    finally:
        os.chdir(cwd)

    out = dict(n_grid=N_GRID, grid_lim=GRID_LIM, dt=DT, g=G, floor_y=FLOOR_Y,
               material=cfg["material"], E=E, nu=nu, mu=mu, lam=lam, friction_angle=cfg["phi"],
               density=cfg["density"], yield_stress=cfg.get("yield_stress", 0.0),
               hardening=cfg.get("hardening", 0), xi=cfg.get("xi", 0.0), substeps=cfg["substeps"],
               x0=x0, vol=vol, mass=mass)
    for key in ("u", "v", "F", "C", "stress"):
        out[key] = np.stack([s[key] for s in states])
    if cfg["material"] == "metal":
        out["yield"] = np.stack([s["yield"] for s in states])
    for key in ("grid_m", "grid_v_in", "grid_v_out"):
        out[key] = np.stack([s[key] for s in states[1:]])
    return out, frame


def make_netdec(ref_root):
    """NetDec forward on seeded rows, ELU (standardised X) and SIREN (clipped X)."""
    d = os.path.join(ref_root, "offline_training_xhat_and_stress_and_mu")
    if SHIM not in sys.path:
        sys.path.insert(0, SHIM)
    sys.path.insert(0, d)
    import CROMnet_secondary as CS

    class _TolerantRandom:
        def __getattr__(self, k):
            return getattr(random, k)

        @staticmethod
        def seed(a=None, *args):
            return random.seed(str(a) if a is not None else None)

    CS.random = _TolerantRandom()
    out = {}
    for tag, siren, omega in (("elu", False, 30.0), ("siren", True, 30.0)):
        fmt = {"i_dim": 3, "o_dim": 6, "mu_dim": 1}
        label = 6
        with contextlib.redirect_stdout(io.StringIO()):
            net = CS.NetDec(fmt, label, 10, siren, omega)
        # seeded weights on the scales of NetDec.init_weights (:259-266): SIREN
        # U(+-sqrt(6/in)/omega_0) with dec0 U(+-1/in); ELU Xavier-like; biases U(+-1/sqrt(in))
        g = torch.Generator().manual_seed(21 if siren else 20)
        with torch.no_grad():
            for lname in ("dec0", "dec1", "dec2", "dec3", "dec4", "enc"):
                layer = getattr(net, lname)
                fan_in = layer.in_features
                if siren:
                    a = 1.0 / fan_in if lname == "dec0" else np.sqrt(6.0 / fan_in) / omega
                else:
                    a = np.sqrt(6.0 / (fan_in + layer.out_features))
                layer.weight.copy_((torch.rand(layer.weight.shape, generator=g) * 2 - 1) * a)
                layer.bias.copy_((torch.rand(layer.bias.shape, generator=g) * 2 - 1) / np.sqrt(fan_in))
        pre = {"min_x": np.array([0.1, 0.2, 0.05]), "max_x": np.array([0.7, 0.8, 0.9]),
               "mean_x": np.array([0.4, 0.45, 0.5]), "std_x": np.array([0.12, 0.1, 0.2]),
               "mean_q": np.array([-100.0, 5.0, -3.0, -120.0, 2.0, -300.0]),
               "std_q": np.array([800.0, 150.0, 120.0, 900.0, 140.0, 2500.0])}
        net.prepare.set_params(pre)
        net.invStandardizeQ.set_params(pre)
        rows = torch.cat([torch.randn(256, label, generator=g),
                          0.1 + 0.8 * torch.rand(256, 3, generator=g),
                          20.0 + 20.0 * torch.rand(256, 1, generator=g) / 40.0], 1)
        with torch.no_grad():
            y = net(rows)
        sd = {k: v.detach().numpy() for k, v in net.state_dict().items()}
        for k, v in sd.items():
            out[f"{tag}/{k}"] = v
        out[f"{tag}/rows"] = rows.numpy()
        out[f"{tag}/out"] = y.numpy()
        out[f"{tag}/omega_0"] = np.float64(omega)
        out[f"{tag}/label_dim"] = np.int64(label)
    sys.path.remove(d)
    return out


def main():
    sys.path.insert(0, SHIM)
    sys.path.insert(0, os.path.join(REF, "engine_stress"))
    import mpm_solver_warp as R

    with tempfile.TemporaryDirectory() as work:
        for name, cfg in SCENES.items():
            print(name, flush=True)
            data, frame = run_scene(R, name, cfg, work)
            np.savez_compressed(os.path.join(HERE, f"ref_mpm_{name}.npz"), **data)
            if frame is not None:
                np.savez_compressed(os.path.join(HERE, "ref_frame_sand.npz"), **frame)
    np.savez_compressed(os.path.join(HERE, "ref_netdec.npz"), **make_netdec(REF))
    print("written to", HERE)


if __name__ == "__main__":
    main()
