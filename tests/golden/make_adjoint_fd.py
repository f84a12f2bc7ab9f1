"""Generate adjoint_fd_sand_rollout_131k.json: central finite differences of the
differentiable-rollout loss, taken on the float64 C oracle.

Workload (the differentiable rollout): 131,072 sand particles, 96^3 grid,
100 substeps at dt 1e-4, v0 ~ N(0, 0.1^2) per component (the scene's seed),
E = 2e5, friction angle 30 deg; target = the final positions of the same
rollout with E = 3e5 and friction angle 35 deg; loss J = mean over the
(n, 3) entries of (x_final - target)^2.  Differences with a relative step of
1e-3: for E, for the friction angle, and along 16 unit directions of the
initial velocity (numpy default_rng(2024) normals, normalised over all
3n entries, step 1e-3 |v0|).  The target is stored as its displacement from
the initial positions in float32 (adjoint_target_sand_rollout_131k.npz,
``displacement``), and the loss uses exactly that rounded target,
x0 + displacement in float64.  The same rollouts also give the differences
of a linear functional of the final positions, mean(w * x_final) with w
standard normals (default_rng(2025), (n, 3)), whose gradient does not pass
through the small MSE residual.

The finite differences of a float32 forward at this step are dominated by
its rounding (the loss moves by about 1e-6 of itself), so the check runs
against the same forward restated in float64 (engine_stress/mpm_utils.py,
engine_stress/mpm_solver_warp.py:156-203, through oracle/mpm_oracle.c built
with ORC_F64): both estimate the derivative of the same exact-arithmetic
rollout.  The GPU adjoint is evaluated on exactly this loss.

Run:  python tests/golden/make_adjoint_fd.py   (about 8 minutes on 8 cores)
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from reduced_mpm_stress_training_gb300 import scenarios as S  # noqa: E402

OUT_JSON = os.path.join(HERE, "adjoint_fd_sand_rollout_131k.json")
OUT_TARGET = os.path.join(HERE, "adjoint_target_sand_rollout_131k.npz")
REL_STEP = 1e-3
N_DIRECTIONS = 16
DIRECTION_SEED = 2024
LINEAR_SEED = 2025


def linear_weights(n: int) -> np.ndarray:
    """w of the linear functional mean(w * x_final): standard normals, (n, 3)."""
    return np.random.default_rng(LINEAR_SEED).standard_normal((n, 3))


def directions(n: int) -> np.ndarray:
    rng = np.random.default_rng(DIRECTION_SEED)
    d = rng.standard_normal((N_DIRECTIONS, n, 3))
    return d / np.linalg.norm(d.reshape(N_DIRECTIONS, -1), axis=1)[:, None, None]


def rollout(sc, v0, E, phi, threads):
    x0, _, vol, mass = sc.particles()
    m = O.make_model(sc.n_grid, sc.grid_lim, material="sand", E=E, nu=sc.nu,
                     friction_angle=phi, gravity=sc.gravity)
    cols = [O.surface_collider(**kw) if kind == "surface" else O.bounding_box(**kw)
            for kind, kw in sc.colliders()]
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=64, colliders=cols)
    for _ in range(sc.substeps):
        sim.p2g2p(sc.dt, nthreads_p2g=threads)
    assert sim.status.value == 0, sim.status.value
    return sim.x0 + sim.u


def main() -> None:
    threads = O.max_threads()
    sc = S.sand_rollout_131k()
    _, v0, _, _ = sc.particles()
    v0 = v0.astype(np.float64)
    E, phi = float(sc.E), float(sc.friction_angle)
    t0 = time.time()
    x0 = sc.particles()[0].astype(np.float64)
    disp = (rollout(sc, v0, 3e5, 35.0, threads) - x0).astype(np.float32)
    target = x0 + disp.astype(np.float64)

    w = linear_weights(sc.n_particles)

    def J(v, e_, p_):
        # both losses from one rollout: the MSE and the linear functional
        x = rollout(sc, v, e_, p_, threads)
        return np.array([np.mean((x - target) ** 2), np.mean(w * x)])

    rh = REL_STEP
    fd = {
        "E": (J(v0, E * (1 + rh), phi) - J(v0, E * (1 - rh), phi)) / (2 * rh * E),
        "friction_angle": (J(v0, E, phi * (1 + rh)) - J(v0, E, phi * (1 - rh))) / (2 * rh * phi),
    }
    h = rh * float(np.linalg.norm(v0))
    for k, d in enumerate(directions(sc.n_particles)):
        fd[f"v0_direction_{k}"] = (J(v0 + h * d, E, phi) - J(v0 - h * d, E, phi)) / (2 * h)
        print(k, fd[f"v0_direction_{k}"].tolist(), f"{time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(OUT_TARGET, displacement=disp)
    base = J(v0, E, phi)
    with open(OUT_JSON, "w") as f:
        json.dump({"workload": "sand_rollout_131k: 131072 sand particles, 96^3 grid, 100 substeps, "
                               "dt 1e-4, E 2e5, friction 30 deg; target E 3e5, friction 35 deg",
                   "forward": "float64 C oracle (orc64_p2g2p)", "relative_step": rh,
                   "direction_seed": DIRECTION_SEED, "n_directions": N_DIRECTIONS,
                   "linear_seed": LINEAR_SEED,
                   "loss_at_base": float(base[0]), "linear_at_base": float(base[1]),
                   "fd": {k: float(v[0]) for k, v in fd.items()},
                   "fd_linear": {k: float(v[1]) for k, v in fd.items()}}, f, indent=1)
    print("wrote", OUT_JSON, f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
