"""The network oracle (oracle/mlp.py) against PyTorch fp32 autograd on the CPU.

The oracle rounds weights, inputs and activations to bfloat16 where the
kernels do; PyTorch here runs the same network with bf16-rounded weights in
fp32.  The two agree to the bf16 rounding of the activations, which pins
the oracle's forward, backward and Adam arithmetic before it checks the
kernels."""
import numpy as np
import torch

from oracle import mlp as M


def _torch_net(p):
    ws, bs = M.unpack(p)
    tw = [torch.tensor(M.bf16(w), dtype=torch.float64, requires_grad=True) for w in ws]
    tb = [torch.tensor(b, dtype=torch.float64, requires_grad=True) for b in bs]
    return tw, tb


def _torch_forward(tw, tb, x):
    h = torch.zeros(x.shape[0], M.K1, dtype=torch.float64)
    h[:, :M.IN] = torch.tensor(M.bf16(x), dtype=torch.float64)
    for l in range(3):
        z = h @ tw[l].T + tb[l]
        h = z * torch.sigmoid(z)
    return (h @ tw[3].T + tb[3])[:, :M.OUT]


def test_bf16_rounding_matches_torch():
    a = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 10
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(M.bf16(a), ref)


def test_forward_and_gradient_match_fp32_autograd():
    rng = np.random.default_rng(1)
    p = M.init_params(3)
    x = rng.standard_normal((257, M.IN)).astype(np.float32)
    t = rng.standard_normal((257, M.OUT)).astype(np.float32) * 0.3
    n = x.shape[0]
    gs = 2.0 / (n * M.OUT)
    o = M.forward(p, x, t, gs)
    g = M.backward(p, o["cache"])
    tw, tb = _torch_net(p)
    y = _torch_forward(tw, tb, x)
    loss = ((y - torch.tensor(t, dtype=torch.float64)) ** 2).sum() * (gs / 2)
    loss.backward()
    yr = y.detach().numpy()
    assert np.linalg.norm(o["y"] - yr) / np.linalg.norm(yr) < 1e-2
    ref = np.concatenate([w.grad.numpy().ravel() for w in tw] + [b.grad.numpy() for b in tb])
    # padded rows/columns of W1/W4 and b4 carry no gradient in the kernels' loss
    ws, bs = M.unpack(ref.copy())
    ws[0][:, M.IN:] = 0
    ws[3][M.OUT:, :] = 0
    bs[3][M.OUT:] = 0
    flat = np.concatenate([w.ravel() for w in ws] + list(bs))
    gw, gb = M.unpack(g)
    for l in range(4):
        rw, rb = M.unpack(flat)
        e = np.linalg.norm(gw[l] - rw[l]) / np.linalg.norm(rw[l])
        assert e < 3e-2, (l, e)
        e = np.linalg.norm(gb[l] - rb[l]) / max(np.linalg.norm(rb[l]), 1e-30)
        assert e < 3e-2, (l, e)


def test_adam_matches_torch():
    rng = np.random.default_rng(2)
    p = M.init_params(0)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    tp = torch.nn.Parameter(torch.tensor(p.copy()))
    opt = torch.optim.Adam([tp], lr=1e-3)
    for step in range(1, 4):
        g = rng.standard_normal(p.shape).astype(np.float32)
        ws, bs = M.unpack(g)
        ws[0][:, M.IN:] = 0
        ws[3][M.OUT:, :] = 0
        bs[3][M.OUT:] = 0
        M.adam(p, m, v, g, step)
        tp.grad = torch.tensor(g)
        opt.step()
    assert np.allclose(p, tp.detach().numpy(), rtol=1e-5, atol=1e-7)
