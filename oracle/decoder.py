"""NumPy restatement of the reference's stress decoder NetDec (test infrastructure only).

Only ``tests/`` use this module; it is the checker of the decoder kernels.

Follows offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:
  :217-227  dec0 (in -> hidden), dec1..dec4 (hidden -> hidden), enc (hidden -> 6)
  :236-249  layer order: Prepare, [Linear, Activation] x 5, Linear, invStandardizeQ
  :487-525  Prepare: the position columns clipped to [-1, 1] (SIREN) or standardised
  :447-463  Activation: sin(omega_0 x) (SIREN) or ELU (alpha 1)
  :465-477  invStandardizeQ: mean_q + q * std_q
and reads the packed parameter layout of the decoder ABI (include/mpm_gb300.h,
MpmStressDecoder): dec0 weight and bias, the four hidden weights, their four
biases, enc weight and bias, the six Prepare numbers, mean_q, std_q.
"""
from __future__ import annotations

import numpy as np


def unpack(blob: np.ndarray, label_dim: int, mu_dim: int, hidden: int) -> dict:
    b = np.asarray(blob, np.float64).ravel()
    n_in = label_dim + 3 + mu_dim
    h = hidden
    o = 0

    def take(k, shape):
        nonlocal o
        a = b[o:o + k].reshape(shape)
        o += k
        return a

    p = {"w0": take(h * n_in, (h, n_in)), "b0": take(h, (h,))}
    p["wh"] = [take(h * h, (h, h)) for _ in range(4)]
    p["bh"] = [take(h, (h,)) for _ in range(4)]
    p["we"] = take(6 * h, (6, h))
    p["be"] = take(6, (6,))
    p["prep"] = take(6, (6,))
    p["qm"] = take(6, (6,))
    p["qs"] = take(6, (6,))
    assert o == b.size, (o, b.size)
    return p


def forward(blob, rows, label_dim: int, mu_dim: int, hidden: int, siren: bool, omega_0: float,
            dtype=np.float64) -> np.ndarray:
    """NetDec.forward (:288-291) on rows (n, label_dim + 3 + mu_dim) -> (n, 6)."""
    p = {k: (np.asarray(v, dtype) if not isinstance(v, list) else [np.asarray(a, dtype) for a in v])
         for k, v in unpack(blob, label_dim, mu_dim, hidden).items()}
    x = np.asarray(rows, dtype).copy()
    xs = x[:, label_dim:label_dim + 3]
    lo, hi = p["prep"][:3], p["prep"][3:]
    if siren:
        x[:, label_dim:label_dim + 3] = dtype(2) * (xs - lo) / (hi - lo) - dtype(1)
    else:
        x[:, label_dim:label_dim + 3] = (xs - lo) / hi

    def act(z):
        if siren:
            return np.sin(dtype(omega_0) * z)
        return np.where(z > 0, z, np.expm1(np.minimum(z, 0)))

    h = act(x @ p["w0"].T + p["b0"])
    for w, bb in zip(p["wh"], p["bh"]):
        h = act(h @ w.T + bb)
    q = h @ p["we"].T + p["be"]
    return p["qm"] + q * p["qs"]


def symmetric_stress(q: np.ndarray) -> np.ndarray:
    """[xx, xy, xz, yy, yz, zz] (mpm_solver_warp.py:383) -> row-major 3x3 (n, 9)."""
    q = np.asarray(q)
    return np.stack([q[:, 0], q[:, 1], q[:, 2], q[:, 1], q[:, 3], q[:, 4], q[:, 2], q[:, 4], q[:, 5]], axis=1)
