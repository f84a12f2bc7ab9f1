"""Many independent scenes advanced together: one launch per stage for all.

The reference simulates one scene per ``MPM_Simulator_WARP`` object
(engine_stress/mpm_solver_warp.py:24-87); running many small scenes that way
leaves the GPU mostly idle.  ``BatchedMPM`` concatenates the scenes' particles
and grids in one ``MPMEngine``: every stage (sort, P2G, grid update, G2P) is a
single persistent launch whose work list spans all scenes (each chunk and
grid block knows its scene), and a substep window is replayed from one CUDA
graph.  Scenes may mix sand and metal, particle counts and grid sizes; they
share dt.

``autotune`` picks the G2P chunk size (particles per CTA) for a workload by
timing the candidates, and caches the choice per device and workload shape.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

import numpy as np
import torch

from . import _capi as A
from .engine import Collider, MPMEngine, SceneParams, lame_from_E_nu, material_code
from .scenarios import Scene


def scene_params(sc: Scene) -> SceneParams:
    mu, lam = lame_from_E_nu(sc.E, sc.nu)
    cols = []
    for kind, kw in sc.colliders():
        cols.append(Collider.surface(**kw) if kind == "surface" else Collider.bounding_box(**kw))
    return SceneParams(n_particles=sc.n_particles, n_grid=sc.n_grid, grid_lim=sc.grid_lim,
                       material=material_code(sc.material), mu=mu, lam=lam,
                       friction_angle=sc.friction_angle, hardening=sc.hardening, xi=sc.xi,
                       gravity=sc.gravity, colliders=cols)


class BatchedMPM:
    """All scenes in one engine; particle arrays are the scenes' concatenation."""

    def __init__(self, scenes: list[Scene], device="cuda:0", chunk_size: int | str = "auto"):
        self.scenes = list(scenes)
        self.device = torch.device(device)
        if chunk_size == "auto":
            chunk_size = autotune(self.scenes, device=self.device)
        self.chunk_size = int(chunk_size)
        self.engine = MPMEngine([scene_params(s) for s in self.scenes], device=self.device,
                                chunk_size=self.chunk_size)
        self.offsets = np.cumsum([0] + [s.n_particles for s in self.scenes])
        x0, v0, vol, mass, ys = [], [], [], [], []
        for s in self.scenes:
            a, b, c, d = s.particles()
            x0.append(a); v0.append(b); vol.append(c); mass.append(d)
            ys.append(np.full(s.n_particles, s.yield_stress, np.float32))
        e = self.engine
        e.load(A.FIELD_X_INITIAL, torch.from_numpy(np.concatenate(x0)))
        e.load(A.FIELD_V, torch.from_numpy(np.concatenate(v0)))
        e.load(A.FIELD_VOL, torch.from_numpy(np.concatenate(vol)))
        e.load(A.FIELD_MASS, torch.from_numpy(np.concatenate(mass)))
        e.load(A.FIELD_YIELD, torch.from_numpy(np.concatenate(ys)))
        self.time = 0.0

    @property
    def n_particles(self) -> int:
        return int(self.offsets[-1])

    def step(self, dt: float) -> None:
        self.engine.substep(self.time, dt)
        self.time += dt

    def graph(self, n: int, dt: float):
        """n substeps (even) captured in one CUDA graph; replay() advances all scenes."""
        return self.engine.graph(n, self.time, dt)

    def export(self, field: int, scene: int) -> torch.Tensor:
        """One scene's slice of a field, reference layout."""
        comps = A.FIELD_COMPONENTS[field]
        full = self.engine.export(field).reshape(self.n_particles, comps)
        return full[self.offsets[scene]:self.offsets[scene + 1]]


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
CANDIDATES = (64, 128, 256)


def _cache_path() -> str:
    base = os.environ.get("MPM_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                                           "mpm_gb300"))
    return os.path.join(base, "autotune.json")


def workload_key(scenes: list[Scene], device) -> str:
    name = torch.cuda.get_device_name(device)
    shape = [(s.n_particles, s.n_grid, s.material) for s in scenes]
    h = hashlib.sha1(json.dumps(shape).encode()).hexdigest()[:16]
    return f"{name}|{len(scenes)}|{sum(s.n_particles for s in scenes)}|{h}"


def time_chunk_size(scenes: list[Scene], chunk: int, device, steps: int = 8) -> float:
    """Seconds per substep of the batch at this chunk size (CUDA events, graph replay)."""
    b = BatchedMPM(scenes, device=device, chunk_size=chunk)
    dt = scenes[0].dt
    for _ in range(2):
        b.step(dt)
    g = b.graph(2, dt)
    g.replay()
    torch.cuda.synchronize(device)
    st = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps // 2):
        g.replay()
    e1.record(st)
    torch.cuda.synchronize(device)
    return e0.elapsed_time(e1) / 1e3 / (2 * (steps // 2))


def autotune(scenes: list[Scene], device="cuda:0", candidates=CANDIDATES, use_cache=True) -> int:
    """Fastest G2P chunk size for this workload on this device (cached)."""
    device = torch.device(device)
    key = workload_key(scenes, device)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return int(cache[key]["chunk_size"])
    times = {c: time_chunk_size(scenes, c, device) for c in candidates}
    best = min(times, key=times.get)
    if use_cache:
        cache[key] = {"chunk_size": best, "seconds_per_substep": times,
                      "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            json.dump(cache, open(path, "w"), indent=1)
        except OSError:
            pass
    return best
