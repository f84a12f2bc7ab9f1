"""Shared builders for the parity tests: a GPU simulator and its oracle twin
started from the same seeded scene."""
from __future__ import annotations

import numpy as np
import torch

from oracle import oracle as O
from reduced_mpm_stress_training_gb300 import MPM_Simulator_WARP
from reduced_mpm_stress_training_gb300 import scenarios as S


def rel(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def gpu_sim(sc: S.Scene, device="cuda:0", chunk_size=128, x0=None, v0=None,
            vol=None, mass=None, colliders=True):
    if x0 is None:
        x0, v0, vol, mass = sc.particles()
    sim = MPM_Simulator_WARP(sc.n_particles, n_grid=sc.n_grid, grid_lim=sc.grid_lim,
                             device=device, chunk_size=chunk_size)
    sim.set_parameters(material=sc.material, E=sc.E, nu=sc.nu,
                       friction_angle=sc.friction_angle, gravity=sc.gravity,
                       hardening=sc.hardening, xi=sc.xi)
    if sc.material == "metal":
        sim.set_parameters(yield_stress=sc.yield_stress)
    sim.load_x_initial_from_tensor(torch.from_numpy(x0))
    sim.load_vol_from_tensor(torch.from_numpy(vol))
    sim.load_mass_from_tensor(torch.from_numpy(mass))
    sim.load_v_from_tensor(torch.from_numpy(v0))
    if colliders:
        for kind, kw in sc.colliders():
            if kind == "surface":
                sim.add_surface_collider(**kw)
            else:
                sim.add_bounding_box(**kw)
    return sim


def oracle_sim(sc: S.Scene, bits=32, x0=None, v0=None, vol=None, mass=None, colliders=True):
    if x0 is None:
        x0, v0, vol, mass = sc.particles()
    m = O.make_model(sc.n_grid, sc.grid_lim, material=sc.material, E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity,
                     hardening=sc.hardening, xi=sc.xi)
    cols = []
    if colliders:
        for kind, kw in sc.colliders():
            cols.append(O.surface_collider(**kw) if kind == "surface" else O.bounding_box(**kw))
    return O.OracleSim(m, x0, mass, vol, v0, bits=bits, colliders=cols,
                       yield_stress=sc.yield_stress if sc.material == "metal" else None)


def gpu_state(sim) -> dict:
    n = sim.n_particles
    e = sim._engine
    from reduced_mpm_stress_training_gb300 import _capi as A

    out = {}
    for name, f in (("u", A.FIELD_U), ("v", A.FIELD_V), ("C", A.FIELD_C), ("F", A.FIELD_F),
                    ("stress", A.FIELD_STRESS), ("x", A.FIELD_X), ("yield_", A.FIELD_YIELD)):
        out[name] = e.export(f).cpu().numpy().reshape(n, -1)
    return out


def compare(sim, ref, fields=("x", "v", "C", "F", "stress")) -> dict:
    """Relative L2 errors GPU vs oracle; "x" is x0 + u on both sides (u alone is
    small early on, so its relative error is dominated by float32 rounding of x)."""
    g = gpu_state(sim)
    out = {}
    for f in fields:
        r = (ref.x0 + ref.u) if f == "x" else getattr(ref, f)
        out[f] = rel(g[f], r.reshape(sim.n_particles, -1))
    return out


def within_fp32_floor(gpu, o32, o64, rtol=1e-5, k=3.0):
    """True when the GPU result is as close to the float32 oracle as the float32
    oracle is to the float64 rerun (times k), or within rtol relative; or when
    the GPU result is itself within k times the float32 oracle's own error of
    the float64 rerun (it is then as accurate as a float32 run can be).  Used
    for stress, C and v: near F = I they are dominated by float32 rounding of
    the SVD (singular values carry ~1e-7 noise), the same in the reference."""
    g, a, b = (np.asarray(x, np.float64).ravel() for x in (gpu, o32, o64))
    floor = np.linalg.norm(a - b)
    d32 = np.linalg.norm(g - a)
    d64 = np.linalg.norm(g - b)
    scale = max(np.linalg.norm(b), 1e-30)
    lim = max(rtol * scale, k * floor)
    ok = (d64 <= lim) or ((d32 <= lim) and (d64 <= lim + floor))
    return bool(ok), dict(gpu_vs_o32=d32 / scale, gpu_vs_o64=d64 / scale, o32_vs_o64=floor / scale)


def netdec_torch(sd: dict, rows, label_dim: int, siren: bool, omega_0: float):
    """PyTorch float32 restatement of NetDec.forward
    (offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301, 447-525):
    the float32 reference the decoder kernels are compared with."""
    import torch.nn.functional as Fn

    sd = {k[len("decoder."):] if k.startswith("decoder.") else k: torch.as_tensor(v, dtype=torch.float32)
          for k, v in sd.items()}
    x = torch.as_tensor(rows, dtype=torch.float32).clone()
    xs = x[:, label_dim:label_dim + 3]
    if siren:
        lo, hi = sd["prepare.min_x_torch"], sd["prepare.max_x_torch"]
        x[:, label_dim:label_dim + 3] = 2 * (xs - lo) / (hi - lo) - 1
    else:
        x[:, label_dim:label_dim + 3] = (xs - sd["prepare.mean_x_torch"]) / sd["prepare.std_x_torch"]

    def act(z):
        return torch.sin(omega_0 * z) if siren else Fn.elu(z)

    h = x
    for name in ("dec0", "dec1", "dec2", "dec3", "dec4"):
        h = act(Fn.linear(h, sd[f"{name}.weight"], sd[f"{name}.bias"]))
    q = Fn.linear(h, sd["enc.weight"], sd["enc.bias"])
    return sd["invStandardizeQ.mean_q_torch"] + q * sd["invStandardizeQ.std_q_torch"]
