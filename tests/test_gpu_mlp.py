"""Network kernels (csrc/mpm_mlp.cu) against the NumPy oracle (oracle/mlp.py):
forward outputs, loss, parameter gradients and the Adam update, on ragged
batch sizes; then a short training run that must lower the loss."""
import numpy as np
import pytest
import torch

from oracle import mlp as M
from reduced_mpm_stress_training_gb300.surrogate import StressMLP

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, M.IN)).astype(np.float32)
    t = (np.tanh(x[:, :M.OUT] * 0.7 + x[:, M.OUT:M.OUT * 2] * 0.3)).astype(np.float32)
    return x, t


@pytest.mark.parametrize("n", [1, 17, 1000, 4099])
def test_forward_matches_oracle(cuda, n):
    x, _ = _data(n, n)
    net = StressMLP(cuda, seed=5)
    y = net.forward(torch.from_numpy(x).to(cuda)).cpu().numpy()
    ref = M.forward(net.master.cpu().numpy(), x)["y"]
    # same bf16 rounding points; differences come from fp32 summation order
    assert rel(y, ref) < 2e-3, rel(y, ref)


@pytest.mark.parametrize("n", [33, 2048, 5000])
def test_loss_and_gradient_match_oracle(cuda, n):
    x, t = _data(n, 100 + n)
    net = StressMLP(cuda, seed=7)
    loss = net.loss_and_grad(torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)).item()
    p = net.master.cpu().numpy()
    o = M.forward(p, x, t, 2.0 / (n * M.OUT))
    g_ref = M.backward(p, o["cache"])
    assert abs(loss - o["loss_sum"] / (n * M.OUT)) <= 1e-3 * abs(loss) + 1e-7
    g = net.grad.cpu().numpy()
    gw, gb = M.unpack(g)
    rw, rb = M.unpack(g_ref)
    for l in range(4):
        assert rel(gw[l], rw[l]) < 1e-2, ("W", l, rel(gw[l], rw[l]))
        assert rel(gb[l], rb[l]) < 1e-2, ("b", l, rel(gb[l], rb[l]))
    # padded entries get no gradient
    assert np.all(gw[0][:, M.IN:] == 0) and np.all(gw[3][M.OUT:, :] == 0) and np.all(gb[3][M.OUT:] == 0)


def test_adam_step_matches_oracle(cuda):
    x, t = _data(3000, 9)
    net = StressMLP(cuda, seed=11)
    p = net.master.cpu().numpy().copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for step in (1, 2, 3):
        net.loss_and_grad(torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda))
        g = net.grad.cpu().numpy()
        net.adam(lr=1e-3)
        M.adam(p, m, v, g, step)
        assert np.allclose(net.master.cpu().numpy(), p, rtol=1e-5, atol=1e-7)
    # the bf16 blob follows the master copy
    blob = net.params.cpu()
    w = blob[:M.W_COUNT * 2].view(torch.bfloat16).float().numpy()
    assert np.array_equal(w, M.bf16(p[:M.W_COUNT]))


def test_training_lowers_the_loss(cuda):
    x, t = _data(65536, 3)
    xt = torch.from_numpy(x).to(cuda)
    tt = torch.from_numpy(t).to(cuda)
    net = StressMLP(cuda, seed=0)
    first = net.train_step(xt, tt).item()
    for _ in range(300):
        last = net.train_step(xt, tt)
    last = last.item()
    assert last < 0.1 * first, (first, last)


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 70000])
def test_tcgen05_forward_matches_oracle(cuda, n):
    """The tcgen05 / tensor-memory forward: same outputs as the oracle (and as
    the mma.sync forward) at the same bf16 rounding points."""
    x, t = _data(n, 7 + n)
    net = StressMLP(cuda, seed=3)
    xt = torch.from_numpy(x).to(cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    y = torch.full((n, M.OUT), float("nan"), device=cuda)
    A_ = net.lib
    from reduced_mpm_stress_training_gb300 import _capi as CAPI
    CAPI.check(A_.mpm_mlp_forward_tc(net.params.data_ptr(), xt.data_ptr(), y.data_ptr(), None, None, None, None,
                                     0.0, n, err.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "mpm_mlp_forward_tc")
    torch.cuda.synchronize()
    assert err.item() == 0
    ref = M.forward(net.master.cpu().numpy(), x)["y"]
    yg = y.cpu().numpy()
    assert np.isfinite(yg).all()
    assert rel(yg, ref) < 2e-3, rel(yg, ref)
    y2 = net.forward(xt).cpu().numpy()
    assert rel(yg, y2) < 2e-3


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 5000, 70000])
def test_tcgen05_backward_matches_mma_sync_and_oracle(cuda, n):
    """The tcgen05 / tensor-memory backward (weight gradients held in tensor
    memory over a CTA's tiles) against the mma.sync backward on the same
    forward outputs, and against the oracle: every weight and bias gradient."""
    x, t = _data(n, 31 + n)
    xt, tt = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    grads = {}
    for name, tc in (("tcgen05", True), ("mma_sync", False)):
        net = StressMLP(cuda, seed=13, tensor_memory=tc)
        net.loss_and_grad(xt, tt)
        torch.cuda.synchronize()
        net.check_tensor_cores()
        grads[name] = net.grad.cpu().numpy()
        p = net.master.cpu().numpy()
    o = M.forward(p, x, t, 2.0 / (n * M.OUT))
    g_ref = M.backward(p, o["cache"])
    gw, gb = M.unpack(grads["tcgen05"])
    sw, sb = M.unpack(grads["mma_sync"])
    rw, rb = M.unpack(g_ref)
    for l in range(4):
        assert np.isfinite(gw[l]).all() and np.isfinite(gb[l]).all()
        assert rel(gw[l], sw[l]) < 5e-3, ("W vs mma.sync", l, rel(gw[l], sw[l]))
        assert rel(gb[l], sb[l]) < 5e-3, ("b vs mma.sync", l, rel(gb[l], sb[l]))
        assert rel(gw[l], rw[l]) < 1e-2, ("W vs oracle", l, rel(gw[l], rw[l]))
        assert rel(gb[l], rb[l]) < 1e-2, ("b vs oracle", l, rel(gb[l], rb[l]))
    assert np.all(gw[0][:, M.IN:] == 0) and np.all(gw[3][M.OUT:, :] == 0) and np.all(gb[3][M.OUT:] == 0)
