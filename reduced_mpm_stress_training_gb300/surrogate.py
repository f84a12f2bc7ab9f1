"""Stress-surrogate network trained and run by the library's own kernels.

``StressMLP`` owns the parameters of the 12 -> 128 -> 128 -> 128 -> 6 SiLU
network (bf16 weights for the tensor cores, fp32 master copy and Adam
moments) and drives ``mpm_mlp_forward`` / ``mpm_mlp_backward`` /
``mpm_mlp_adam`` (csrc/mpm_mlp.cu).  PyTorch only provides the device
buffers; every arithmetic step of inference and training is a library
kernel.  The network has no counterpart in the reference's solver; its
nearest relative is the stress decoder ``CROMnet_secondary.NetDec``
(CROMnet_secondary.py:203-301), whose 6-component output is the stress
stored as ``[xx, xy, xz, yy, yz, zz]`` (engine_stress/mpm_solver_warp.py:383).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as A

IN, OUT, HID, N4, K1 = 12, 6, 128, 16, 16
SHAPES = [(HID, K1), (HID, HID), (HID, HID), (N4, HID)]
W_COUNT = sum(a * b for a, b in SHAPES)
B_SIZES = [HID, HID, HID, N4]
P_COUNT = W_COUNT + sum(B_SIZES)


def _ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def init_master(seed: int = 0) -> np.ndarray:
    """torch.nn.Linear-style uniform init (bound 1/sqrt(fan_in)); padded entries zero."""
    rng = np.random.default_rng(seed)
    parts_w, parts_b = [], []
    fan_in = [IN, HID, HID, HID]
    for l, (a, b) in enumerate(SHAPES):
        bound = 1.0 / np.sqrt(fan_in[l])
        w = rng.uniform(-bound, bound, size=(a, b)).astype(np.float32)
        bb = rng.uniform(-bound, bound, size=B_SIZES[l]).astype(np.float32)
        if l == 0:
            w[:, IN:] = 0.0
        if l == 3:
            w[OUT:, :] = 0.0
            bb[OUT:] = 0.0
        parts_w.append(w.ravel())
        parts_b.append(bb)
    return np.concatenate(parts_w + parts_b)


class StressMLP:
    """The surrogate network on one device, with its Adam state."""

    def __init__(self, device="cuda:0", seed: int = 0, master: np.ndarray | None = None):
        self.lib = A.load()
        if self.lib.mpm_mlp_param_bytes() != W_COUNT * 2 + (P_COUNT - W_COUNT) * 4:
            raise ImportError("libmpm_gb300 network layout differs from the binding")
        self.device = torch.device(device)
        m = init_master(seed) if master is None else np.asarray(master, np.float32)
        if m.shape != (P_COUNT,):
            raise ValueError(f"master parameters must have {P_COUNT} floats")
        self.master = torch.from_numpy(m.copy()).to(self.device)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.grad = torch.zeros_like(self.master)
        self.params = torch.empty(self.lib.mpm_mlp_param_bytes(), dtype=torch.uint8, device=self.device)
        self.refresh()
        self.step_count = 0
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self._bufs: dict = {}

    # -- parameters ---------------------------------------------------------
    def refresh(self) -> None:
        """Rewrite the bf16/fp32 blob from the fp32 master copy."""
        w = self.master[:W_COUNT].to(torch.bfloat16).view(torch.uint8)
        b = self.master[W_COUNT:].contiguous().view(torch.uint8)
        self.params.copy_(torch.cat([w, b]))

    def state_dict(self) -> dict:
        return {"master": self.master.cpu().numpy(), "m": self.m.cpu().numpy(),
                "v": self.v.cpu().numpy(), "step": self.step_count}

    def load_state_dict(self, sd: dict) -> None:
        self.master.copy_(torch.as_tensor(sd["master"]))
        self.m.copy_(torch.as_tensor(sd["m"]))
        self.v.copy_(torch.as_tensor(sd["v"]))
        self.step_count = int(sd["step"])
        self.refresh()

    # -- kernels ----------------------------------------------------------
    def _buffers(self, n: int) -> dict:
        b = self._bufs
        if b.get("n", -1) < n:
            dev = self.device
            b.update(n=n, z=torch.empty(3 * n * HID, dtype=torch.bfloat16, device=dev),
                     dy=torch.empty(n * N4, dtype=torch.bfloat16, device=dev),
                     work=torch.empty(2 * n * HID, dtype=torch.bfloat16, device=dev))
        return b

    def forward(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """y (n,6) = net(x (n,12)), x float32 contiguous on the device."""
        x = x.contiguous()
        n = x.shape[0]
        if x.shape[1:] != (IN,) or x.dtype != torch.float32:
            raise ValueError("x must be float32 (n, 12)")
        y = out if out is not None else torch.empty(n, OUT, dtype=torch.float32, device=self.device)
        A.check(self.lib.mpm_mlp_forward(_ptr(self.params), _ptr(x), _ptr(y), None, None, None, None,
                                         0.0, n, _stream(self.device)), "mpm_mlp_forward")
        return y

    def loss_and_grad(self, x: torch.Tensor, target: torch.Tensor, accumulate: bool = False,
                      grad_scale: float | None = None) -> torch.Tensor:
        """Mean squared error over the batch (device scalar); its gradient is added into self.grad."""
        x = x.contiguous()
        target = target.contiguous()
        n = x.shape[0]
        if grad_scale is None:
            grad_scale = 2.0 / (n * OUT)
        b = self._buffers(n)
        if not accumulate:
            self.grad.zero_()
        self.loss.zero_()
        st = _stream(self.device)
        A.check(self.lib.mpm_mlp_forward(_ptr(self.params), _ptr(x), None, _ptr(target), _ptr(b["z"]),
                                         _ptr(b["dy"]), _ptr(self.loss), grad_scale, n, st),
                "mpm_mlp_forward")
        A.check(self.lib.mpm_mlp_backward(_ptr(self.params), _ptr(x), _ptr(b["z"]), _ptr(b["dy"]),
                                          _ptr(b["work"]), _ptr(self.grad), n, st), "mpm_mlp_backward")
        return self.loss / (n * OUT)

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_count += 1
        A.check(self.lib.mpm_mlp_adam(_ptr(self.master), _ptr(self.m), _ptr(self.v), _ptr(self.grad),
                                      _ptr(self.params), lr, beta1, beta2, eps, self.step_count,
                                      _stream(self.device)), "mpm_mlp_adam")

    def train_step(self, x: torch.Tensor, target: torch.Tensor, lr: float = 1e-3) -> torch.Tensor:
        loss = self.loss_and_grad(x, target)
        self.adam(lr)
        return loss
