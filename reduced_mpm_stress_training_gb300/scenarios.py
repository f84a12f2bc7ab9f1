"""Seeded synthetic scenes for the sand-column / metal-block workloads.

No dataset is involved: the reference's initial-sampling h5 files are not
part of its snapshot, so each scene is rebuilt from its description --
uniform-random particle positions in an axis-aligned box (seeded
``numpy.random.Generator``), particle volume = box volume / N,
mass = density * volume, F = I, C = 0, stress = 0, the reference's sticky
surface collider as a floor under the column (normal +z) and its
slip-wall bounding box (engine_stress/mpm_solver_warp.py:407, :499).

Scenes (sizes as named):
  sand_column_32k      32,768 sand particles, 64^3 grid, dt 1e-4, 200 substeps
  sand_column_1m       1,048,576 sand particles, 128^3 grid, dt 5e-5, 1000 substeps
  metal_block_1m       same column, von Mises metal E=1e7, yield 1e5, rho 2700, v0=(0,0,-1)
  sand_rollout_131k    131,072 sand particles, 96^3 grid, dt 1e-4, 100 substeps, v0 ~ N(0, 0.1^2)
  batch_64             64 scenes, N log-uniform [1e4, 2e5], grid 48/64/96, 25 % metal
                       (metal E log-uniform [1e5, 1e6] like the sand, yield [5e4, 5e5])
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Scene:
    name: str
    n_particles: int
    n_grid: int
    grid_lim: float
    box_lo: tuple
    box_hi: tuple
    material: str
    E: float
    nu: float
    friction_angle: float
    density: float
    gravity: tuple
    dt: float
    substeps: int
    yield_stress: float = 0.0
    hardening: int = 0
    xi: float = 0.0
    v0: tuple = (0.0, 0.0, 0.0)
    v0_sigma: float = 0.0
    floor_z: float | None = 0.05
    seed: int = 0

    @property
    def mu(self) -> float:
        """engine_stress/mpm_solver_warp.py:41"""
        return self.E / 2.0 / (1.0 + self.nu)

    @property
    def lam(self) -> float:
        """engine_stress/mpm_solver_warp.py:42"""
        return self.E * self.nu / (1.0 + self.nu) / (1.0 - 2.0 * self.nu)

    @property
    def box_volume(self) -> float:
        return float(np.prod(np.subtract(self.box_hi, self.box_lo)))

    def particles(self):
        """Seeded initial particles: (x0 (N,3), v0 (N,3), vol (N,), mass (N,)) as float32."""
        rng = np.random.default_rng(self.seed)
        lo = np.asarray(self.box_lo, np.float64)
        hi = np.asarray(self.box_hi, np.float64)
        x0 = (lo + (hi - lo) * rng.random((self.n_particles, 3))).astype(np.float32)
        v = np.broadcast_to(np.asarray(self.v0, np.float32), (self.n_particles, 3)).copy()
        if self.v0_sigma > 0:
            v = v + rng.normal(0.0, self.v0_sigma, (self.n_particles, 3)).astype(np.float32)
        vol = np.full(self.n_particles, self.box_volume / self.n_particles, np.float32)
        mass = (np.float32(self.density) * vol).astype(np.float32)
        return x0, v.astype(np.float32), vol, mass

    def colliders(self):
        """(kind, kwargs) in registration order: floor (sticky surface) then box."""
        out = []
        if self.floor_z is not None:
            out.append(("surface", dict(point=(0.0, 0.0, self.floor_z), normal=(0.0, 0.0, 1.0),
                                        surface="sticky", friction=0.0)))
        out.append(("box", {}))
        return out


def scene_to_dict(sc: Scene) -> dict:
    """A scene as plain JSON-ready values (tuples become lists)."""
    return {k: (list(v) if isinstance(v, tuple) else v) for k, v in dataclasses.asdict(sc).items()}


def scene_from_dict(d: dict) -> Scene:
    """The inverse of scene_to_dict; unknown keys raise TypeError."""
    kw = dict(d)
    for k in ("box_lo", "box_hi", "gravity", "v0"):
        if k in kw and kw[k] is not None:
            kw[k] = tuple(float(x) for x in kw[k])
    return Scene(**kw)


def save_scenes(path: str, scenes) -> None:
    """One scene or a list of scenes to a JSON file."""
    import json

    data = [scene_to_dict(s) for s in scenes] if isinstance(scenes, (list, tuple)) else scene_to_dict(scenes)
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def load_scenes(path: str):
    """A scene (or list of scenes) from a JSON file written by save_scenes."""
    import json

    with open(path) as f:
        data = json.load(f)
    return [scene_from_dict(d) for d in data] if isinstance(data, list) else scene_from_dict(data)


def sand_column_32k(seed: int = 0) -> Scene:
    return Scene("sand_column_32k", 32768, 64, 1.0, (0.4, 0.4, 0.05), (0.6, 0.6, 0.65), "sand",
                 2e5, 0.3, 30.0, 2200.0, (0.0, 0.0, -9.8), 1e-4, 200, seed=seed)


def sand_column_1m(seed: int = 0) -> Scene:
    return Scene("sand_column_1m", 1048576, 128, 1.0, (0.35, 0.35, 0.05), (0.65, 0.65, 0.85),
                 "sand", 2e5, 0.3, 30.0, 2200.0, (0.0, 0.0, -9.8), 5e-5, 1000, seed=seed)


def metal_block_1m(seed: int = 0) -> Scene:
    return Scene("metal_block_1m", 1048576, 128, 1.0, (0.35, 0.35, 0.05), (0.65, 0.65, 0.85),
                 "metal", 1e7, 0.3, 30.0, 2700.0, (0.0, 0.0, -9.8), 5e-5, 1000,
                 yield_stress=1e5, v0=(0.0, 0.0, -1.0), seed=seed)


def sand_rollout_131k(seed: int = 0, E: float = 2e5, friction_angle: float = 30.0) -> Scene:
    return Scene("sand_rollout_131k", 131072, 96, 1.0, (0.35, 0.35, 0.05), (0.65, 0.65, 0.85),
                 "sand", E, 0.3, friction_angle, 2200.0, (0.0, 0.0, -9.8), 1e-4, 100,
                 v0_sigma=0.1, seed=seed)


def small_column(n_particles: int = 4096, n_grid: int = 32, material: str = "sand",
                 seed: int = 0, **kw) -> Scene:
    """A scaled-down sand column for fast parity checks."""
    base = dict(E=2e5, nu=0.3, friction_angle=30.0, density=2200.0, gravity=(0.0, 0.0, -9.8),
                dt=1e-4, substeps=20)
    if material == "metal":
        base.update(E=1e7, density=2700.0, yield_stress=1e5, v0=(0.0, 0.0, -1.0))
    base.update(kw)
    return Scene(f"small_{material}_{n_particles}", n_particles, n_grid, 1.0, (0.35, 0.35, 0.15),
                 (0.65, 0.65, 0.75), material, seed=seed, **base)


def batch_64(seed: int = 0, n_scenes: int = 64) -> list[Scene]:
    """64 independent scenes: N log-uniform in [1e4, 2e5], grid 48/64/96, 25 % metal."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(1e4), math.log(2e5)))))
        ng = int(rng.choice([48, 64, 96]))
        metal = rng.random() < 0.25
        if metal:
            # the workload fixes the metal's yield stress range, not its E: it takes the
            # sand's E range, which keeps dt 1e-4 inside the elastic-wave CFL bound on a
            # 96^3 grid (E = 1e7 at 2700 kg/m^3 does not, and goes non-finite)
            E = float(math.exp(rng.uniform(math.log(1e5), math.log(1e6))))
            sc = Scene(f"batch_{s}_metal", n, ng, 1.0, (0.35, 0.35, 0.1), (0.65, 0.65, 0.7),
                       "metal", E, 0.3, 30.0, 2700.0, (0.0, 0.0, -9.8), 1e-4, 500,
                       yield_stress=float(math.exp(rng.uniform(math.log(5e4), math.log(5e5)))),
                       seed=seed * 1000 + s)
        else:
            sc = Scene(f"batch_{s}_sand", n, ng, 1.0, (0.35, 0.35, 0.1), (0.65, 0.65, 0.7),
                       "sand", float(math.exp(rng.uniform(math.log(1e5), math.log(1e6)))), 0.3,
                       float(rng.uniform(20.0, 40.0)), 2200.0, (0.0, 0.0, -9.8), 1e-4, 500,
                       seed=seed * 1000 + s)
        scenes.append(sc)
    return scenes


SCENES = {
    "sand_column_32k": sand_column_32k,
    "sand_column_1m": sand_column_1m,
    "metal_block_1m": metal_block_1m,
    "sand_rollout_131k": sand_rollout_131k,
}


def build_simulator(sc: Scene, device="cuda:0", chunk_size: int = 128):
    """An MPM_Simulator_WARP loaded with the scene (particles, material, colliders)."""
    import torch

    from .solver import MPM_Simulator_WARP

    x0, v0, vol, mass = sc.particles()
    sim = MPM_Simulator_WARP(sc.n_particles, n_grid=sc.n_grid, grid_lim=sc.grid_lim, device=device,
                             chunk_size=chunk_size)
    sim.set_parameters(material=sc.material, E=sc.E, nu=sc.nu, friction_angle=sc.friction_angle,
                       gravity=sc.gravity, hardening=sc.hardening, xi=sc.xi)
    if sc.material == "metal":
        sim.set_parameters(yield_stress=sc.yield_stress)
    sim.load_x_initial_from_tensor(torch.from_numpy(x0))
    sim.load_vol_from_tensor(torch.from_numpy(vol))
    sim.load_mass_from_tensor(torch.from_numpy(mass))
    sim.load_v_from_tensor(torch.from_numpy(v0))
    for kind, kw in sc.colliders():
        if kind == "surface":
            sim.add_surface_collider(**kw)
        else:
            sim.add_bounding_box(**kw)
    return sim


def run(name: str, substeps: int, device="cuda:0") -> dict:
    """Build a named scene and take `substeps` plain substeps on the device
    (the driver the ncu summaries profile); returns the wall time per substep
    and the status word."""
    import time

    import torch

    sc = SCENES[name]()
    sim = build_simulator(sc, device=device)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    for k in range(substeps):
        sim.p2g2p(k, sc.dt)
    torch.cuda.synchronize(device)
    return {"scene": name, "substeps": substeps, "ms_per_substep": 1e3 * (time.perf_counter() - t0) / max(substeps, 1),
            "status": int(sim.check_status())}


if __name__ == "__main__":
    import sys

    print(run(sys.argv[1] if len(sys.argv) > 1 else "sand_column_1m", int(sys.argv[2]) if len(sys.argv) > 2 else 12))
