"""NumPy restatement of the stress-surrogate network kernels (test infrastructure).

Only ``tests/`` and ``bench.py``'s CPU legs use this module: it is the checker
of ``csrc/mpm_mlp.cu``, never the thing measured.  The network has no
counterpart in the reference (its nearest relative is the stress decoder
``CROMnet_secondary.NetDec``, CROMnet_secondary.py:203-301, whose output is
the 6-component stress ``[xx, xy, xz, yy, yz, zz]`` of
engine_stress/mpm_solver_warp.py:383); this file restates the kernels'
arithmetic, with their bfloat16 rounding points, in float64/float32 NumPy:

  forward   Z_l = H_{l-1} W_l^T + b_l (fp32 accumulate of bf16 operands),
            H_l = bf16(silu(Z_l)), saved pre-activation bf16(Z_l),
            y = H_3 W_4^T + b_4, dY = bf16(grad_scale * (y - target))
  backward  dZ_3 = bf16((dY W_4) * silu'(bf16 Z_3)), dZ_2, dZ_1 likewise,
            dW_l = dZ_l^T bf16(silu(bf16 Z_{l-1})) (dW_1 = dZ_1^T bf16(x)),
            db_l = sum_rows dZ_l
  adam      PyTorch's Adam (no weight decay) on fp32 master parameters.

Parameter layout (flat fp32, weights then biases; padded shapes):
W1 [128][16] (inputs 12..15 zero), W2 [128][128], W3 [128][128],
W4 [16][128] (outputs 6..15 zero), b1 b2 b3 [128], b4 [16].
"""
from __future__ import annotations

import numpy as np

IN, K1, H, OUT, N4 = 12, 16, 128, 6, 16
SHAPES = [(H, K1), (H, H), (H, H), (N4, H)]
W_SIZES = [a * b for a, b in SHAPES]
W_COUNT = sum(W_SIZES)
B_SIZES = [H, H, H, N4]
B_COUNT = sum(B_SIZES)
P_COUNT = W_COUNT + B_COUNT


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def silu(z):
    """z sigmoid(z), sigmoid written as (1 + tanh(z/2)) / 2 as the kernels do
    (they evaluate tanh with the hardware approximation)."""
    return z * (0.5 + 0.5 * np.tanh(0.5 * z))


def silu_grad(z):
    s = 0.5 + 0.5 * np.tanh(0.5 * z)
    return s * (1.0 + z * (1.0 - s))


def unpack(p: np.ndarray):
    """Flat parameters -> ([W1..W4], [b1..b4]) views."""
    ws, bs, o = [], [], 0
    for (a, b) in SHAPES:
        ws.append(p[o:o + a * b].reshape(a, b))
        o += a * b
    for n in B_SIZES:
        bs.append(p[o:o + n])
        o += n
    return ws, bs


def init_params(seed: int = 0) -> np.ndarray:
    """torch.nn.Linear-style uniform init, padded entries zero."""
    rng = np.random.default_rng(seed)
    p = np.zeros(P_COUNT, np.float32)
    ws, bs = unpack(p)
    fan_in = [IN, H, H, H]
    for l in range(4):
        bound = 1.0 / np.sqrt(fan_in[l])
        w = rng.uniform(-bound, bound, size=SHAPES[l]).astype(np.float32)
        b = rng.uniform(-bound, bound, size=B_SIZES[l]).astype(np.float32)
        if l == 0:
            w[:, IN:] = 0.0
        if l == 3:
            w[OUT:, :] = 0.0
            b[OUT:] = 0.0
        ws[l][...] = w
        bs[l][...] = b
    return p


def forward(p: np.ndarray, x: np.ndarray, target=None, grad_scale: float = 0.0):
    """Returns (y [n,6], cache); with a target also dY and the summed squared error."""
    ws, bs = unpack(p.astype(np.float32))
    wb = [bf16(w).astype(np.float64) for w in ws]
    n = x.shape[0]
    xin = np.zeros((n, K1), np.float32)
    xin[:, :IN] = x
    h = bf16(xin).astype(np.float64)
    zs = []
    for l in range(3):
        z = (h @ wb[l].T + bs[l]).astype(np.float32)
        zs.append(bf16(z))
        h = bf16(silu(z.astype(np.float64)).astype(np.float32)).astype(np.float64)
    y = (h @ wb[3].T + bs[3]).astype(np.float32)
    cache = {"x": bf16(xin), "z": zs}
    out = {"y": y[:, :OUT], "cache": cache}
    if target is not None:
        r = y[:, :OUT].astype(np.float64) - target
        d = np.zeros((n, N4), np.float32)
        d[:, :OUT] = (grad_scale * r).astype(np.float32)
        cache["dy"] = bf16(d)
        out["loss_sum"] = float((r * r).sum())
    return out


def backward(p: np.ndarray, cache: dict) -> np.ndarray:
    """Flat fp32 gradient of the loss whose dY the forward produced."""
    ws, _ = unpack(p.astype(np.float32))
    wb = [bf16(w).astype(np.float64) for w in ws]
    z = [zz.astype(np.float64) for zz in cache["z"]]
    hs = [cache["x"].astype(np.float64)] + [bf16(silu(zz).astype(np.float32)).astype(np.float64)
                                            for zz in z]
    g = np.zeros(P_COUNT, np.float64)
    gw, gb = unpack(g)
    dz = cache["dy"].astype(np.float64)
    for l in (3, 2, 1, 0):
        gw[l][...] = dz.T @ hs[l]
        gb[l][...] = dz.sum(axis=0)
        if l > 0:
            dh = dz @ wb[l]
            dz = bf16((dh * silu_grad(z[l - 1])).astype(np.float32)).astype(np.float64)
    return g.astype(np.float32)


def adam(p, m, v, g, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update in place (torch.optim.Adam semantics); padded entries stay zero."""
    m[...] = b1 * m + (1 - b1) * g
    v[...] = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    p[...] = p - lr * mh / (np.sqrt(vh) + eps)
    ws, bs = unpack(p)
    ws[0][:, IN:] = 0.0
    ws[3][OUT:, :] = 0.0
    bs[3][OUT:] = 0.0
