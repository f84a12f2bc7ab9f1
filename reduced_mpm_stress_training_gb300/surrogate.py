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

import ctypes as C

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

    def __init__(self, device="cuda:0", seed: int = 0, master: np.ndarray | None = None,
                 tensor_memory: bool = True):
        """tensor_memory: run the forward and the backward on the tcgen05
        tensor cores (mpm_mlp_forward_tc, mpm_mlp_backward_tc) instead of the
        mma.sync kernels."""
        self.lib = A.load()
        self.tensor_memory = bool(tensor_memory)
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
        self.tc_error = torch.zeros(1, dtype=torch.int32, device=self.device)
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
        self._forward(x, y, None, None, None, None, 0.0, n)
        return y

    def _forward(self, x, y, target, z, dy, loss, grad_scale, n) -> None:
        st = _stream(self.device)
        if self.tensor_memory:
            A.check(self.lib.mpm_mlp_forward_tc(_ptr(self.params), _ptr(x), _ptr(y), _ptr(target), _ptr(z),
                                                _ptr(dy), _ptr(loss), grad_scale, n, _ptr(self.tc_error), st),
                    "mpm_mlp_forward_tc")
        else:
            A.check(self.lib.mpm_mlp_forward(_ptr(self.params), _ptr(x), _ptr(y), _ptr(target), _ptr(z),
                                             _ptr(dy), _ptr(loss), grad_scale, n, st), "mpm_mlp_forward")

    def check_tensor_cores(self) -> None:
        """Raise if a tensor-core completion wait of the forward or backward ever ran out."""
        if int(self.tc_error.item()):
            raise RuntimeError("tcgen05 network kernels: a tensor-core completion wait timed out")

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
        self._forward(x, None, target, b["z"], b["dy"], self.loss, grad_scale, n)
        if self.tensor_memory:
            A.check(self.lib.mpm_mlp_backward_tc(_ptr(self.params), _ptr(x), _ptr(b["z"]), _ptr(b["dy"]),
                                                 _ptr(self.grad), n, _ptr(self.tc_error), st),
                    "mpm_mlp_backward_tc")
        else:
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


# ---------------------------------------------------------------------------
# Gate configuration and the in-step surrogate
# ---------------------------------------------------------------------------
# rho_min: below |F F^T - I| = 1e-4 the float32 F (and so the plain return
# map's stress, the training label) carries more than 1e-3 relative rounding
# noise in the strain; those particles keep the SVD path.
DEFAULT_CONFIG = dict(tol=1e-2, rho_min=1e-4, rho_max=2.5, nu_min=0.25, nu_max=0.35,
                      phi_min=20.0, phi_max=40.0, dgamma_max=0.1)

OUTCOMES = ("elastic", "plastic", "fb_domain", "fb_apex", "fb_step", "fb_gate", "fb_material")


def make_config(**kw) -> A.MpmSurrogateConfig:
    d = dict(DEFAULT_CONFIG)
    unknown = set(kw) - set(d)
    if unknown:
        raise ValueError(f"unknown surrogate settings {sorted(unknown)}")
    d.update(kw)
    return A.MpmSurrogateConfig(**{k: float(v) for k, v in d.items()})


def sand_scene(E: float, nu: float, friction_angle: float) -> A.MpmScene:
    """A sand MpmScene carrying only the material (for the element kernels)."""
    from .engine import dp_alpha, lame_from_E_nu

    s = A.MpmScene()
    mu, lam = lame_from_E_nu(E, nu)
    s.material = A.SAND
    s.mu, s.lam, s.alpha = mu, lam, dp_alpha(friction_angle)
    s.n_grid, s.dx, s.inv_dx = 1, 1.0, 1.0
    return s


class StressSurrogate:
    """A trained network plus its gate settings, attached to an engine with
    ``MPMEngine.set_stress_surrogate``: each substep then runs
    ``mpm_p2g2p_surrogate`` (network stress for sand particles that pass the
    gate, the SVD return map for the rest)."""

    def __init__(self, net: StressMLP, **cfg):
        self.net = net
        self.cfg = make_config(**cfg)
        self.fallback = None
        self.stats = torch.zeros(A.SUR_STATS, dtype=torch.int32, device=net.device)

    def params_ptr(self) -> int:
        return self.net.params.data_ptr()

    def bind(self, engine) -> None:
        if engine.device != self.net.device:
            raise ValueError("the network and the engine must be on the same device")
        n = max(engine.n_particles, 1)
        if self.fallback is None or self.fallback.numel() < 2 * n:
            self.fallback = torch.empty(2 * n, dtype=torch.int32, device=self.net.device)

    def reset_stats(self) -> None:
        self.stats.zero_()

    def outcome_counts(self) -> dict:
        s = self.stats.cpu().tolist()
        return {name: s[i] for i, name in enumerate(OUTCOMES)}

    def apply(self, F_trial: torch.Tensor, E: float, nu: float, friction_angle: float):
        """Element form (mpm_surrogate_apply): F_trial (n,9) -> F (n,9), stress (n,9), codes (n)."""
        F_trial = F_trial.to(self.net.device, torch.float32).reshape(-1, 9).contiguous()
        n = F_trial.shape[0]
        Fo = torch.empty_like(F_trial)
        tau = torch.empty_like(F_trial)
        codes = torch.empty(n, dtype=torch.int32, device=self.net.device)
        sc = sand_scene(E, nu, friction_angle)
        A.check(self.net.lib.mpm_surrogate_apply(C.byref(sc), self.params_ptr(), C.byref(self.cfg),
                                                 F_trial.data_ptr(), Fo.data_ptr(), tau.data_ptr(),
                                                 codes.data_ptr(), n, _stream(self.net.device)),
                "mpm_surrogate_apply")
        return Fo, tau, codes


# ---------------------------------------------------------------------------
# Training tuples (F_trial, material) -> stress of the plain return map
# ---------------------------------------------------------------------------
def haar_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """n Haar-random rotations (QR of Gaussian matrices, signs fixed, det +1)."""
    q, r = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    q = q * np.sign(np.diagonal(r, axis1=1, axis2=2))[:, None, :]
    flip = np.linalg.det(q) < 0
    q[flip, :, 0] *= -1.0
    return q


def synthetic_F(n: int, rng: np.random.Generator, max_log: float = 0.3,
                log_uniform_scale: bool = False, min_log: float = 4e-5) -> np.ndarray:
    """F = R diag(exp(s)) Q^T with Haar R, Q.  s ~ U(-max_log, max_log)^3, or
    (log_uniform_scale) s = m u with u a random unit direction and m
    log-uniform in [min_log, max_log], which covers the small strains of a
    settling column."""
    if log_uniform_scale:
        u = rng.standard_normal((n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        m = np.exp(rng.uniform(np.log(min_log), np.log(max_log), size=(n, 1)))
        s = u * m
    else:
        s = rng.uniform(-max_log, max_log, size=(n, 3))
    R = haar_rotations(n, rng)
    Q = haar_rotations(n, rng)
    F = (R * np.exp(s)[:, None, :]) @ Q.transpose(0, 2, 1)
    return F.reshape(n, 9).astype(np.float32)


def rollout_F_trial(scene, n_substeps: int, every: int, device="cuda:0") -> torch.Tensor:
    """F_trial = (I + dt C) F of every particle, sampled every ``every``
    substeps of a plain-solver rollout of ``scene`` (scenarios.Scene)."""
    from .scenarios import build_simulator

    sim = build_simulator(scene, device=device)
    out = []
    eye = torch.eye(3, device=device)
    for k in range(1, n_substeps + 1):
        sim.p2g2p(k, scene.dt)
        if k % every == 0:
            F = sim.engine.export(A.FIELD_F).reshape(-1, 3, 3)
            Cm = sim.engine.export(A.FIELD_C).reshape(-1, 3, 3)
            out.append(((eye + scene.dt * Cm) @ F).reshape(-1, 9))
    return torch.cat(out)


def label(F_trial: torch.Tensor, E: float, nu: float, friction_angle: float):
    """Network inputs x (n,12) and targets y (n,6) of one material, labelled by
    the plain return map (mpm_return_map) and mpm_surrogate_features."""
    lib = A.load()
    F_trial = F_trial.to(torch.float32).reshape(-1, 9).contiguous()
    dev = F_trial.device
    n = F_trial.shape[0]
    sc = sand_scene(E, nu, friction_angle)
    Fo = torch.empty_like(F_trial)
    tau = torch.empty_like(F_trial)
    st = _stream(dev)
    A.check(lib.mpm_return_map(C.byref(sc), F_trial.data_ptr(), None, Fo.data_ptr(), tau.data_ptr(),
                               n, st), "mpm_return_map")
    x = torch.empty(n, IN, dtype=torch.float32, device=dev)
    y = torch.empty(n, OUT, dtype=torch.float32, device=dev)
    A.check(lib.mpm_surrogate_features(C.byref(sc), F_trial.data_ptr(), tau.data_ptr(), x.data_ptr(),
                                       y.data_ptr(), n, st), "mpm_surrogate_features")
    return x, y


def sample_materials(n_groups: int, rng: np.random.Generator):
    """(E, nu, friction angle) per group: E log-uniform [1e5, 1e6] Pa,
    nu U(0.25, 0.35), friction angle U(20, 40) degrees."""
    E = np.exp(rng.uniform(np.log(1e5), np.log(1e6), n_groups))
    nu = rng.uniform(0.25, 0.35, n_groups)
    phi = rng.uniform(20.0, 40.0, n_groups)
    return list(zip(E.tolist(), nu.tolist(), phi.tolist()))


def build_training_set(n_total: int, device="cuda:0", seed: int = 0, rollout: torch.Tensor | None = None,
                       group: int = 65536, rho_min: float = DEFAULT_CONFIG["rho_min"]):
    """About n_total tuples: 40 % F = R diag(exp s) with s ~ U(-0.3, 0.3),
    30 % the same with log-uniform strain magnitude, 30 % rollout F_trial
    (when given; otherwise more of the first two).  Every group of ``group``
    tuples is labelled with its own sampled material.  Tuples with
    |F F^T - I| < rho_min (outside the gate's domain, labels dominated by
    float32 rounding) are dropped."""
    rng = np.random.default_rng(seed)
    n_roll = int(0.3 * n_total) if rollout is not None and rollout.shape[0] > 0 else 0
    n_syn = n_total - n_roll
    n_uni = int(round(n_syn * 4 / 7))
    Fs = [torch.from_numpy(synthetic_F(n_uni, rng)),
          torch.from_numpy(synthetic_F(n_syn - n_uni, rng, log_uniform_scale=True))]
    Fs = [f.to(device) for f in Fs]
    if n_roll:
        pick = torch.from_numpy(rng.choice(rollout.shape[0], n_roll, replace=n_roll > rollout.shape[0]))
        Fs.append(rollout[pick.to(rollout.device)].to(device))
    F = torch.cat(Fs)
    F = F[torch.from_numpy(rng.permutation(F.shape[0])).to(device)]
    xs, ys = [], []
    mats = sample_materials((n_total + group - 1) // group, rng)
    x9_min = (np.log10(rho_min) + 2.5) / 1.5  # the log-strain input at rho_min
    for g, (E, nu, phi) in enumerate(mats):
        x, y = label(F[g * group:(g + 1) * group], E, nu, phi)
        keep = x[:, 9] >= x9_min
        xs.append(x[keep])
        ys.append(y[keep])
    return torch.cat(xs), torch.cat(ys)


def train(net: StressMLP, x: torch.Tensor, y: torch.Tensor, steps: int, batch: int = 65536,
          lr: float = 1e-3, lr_min: float = 1e-5, seed: int = 0, log_every: int = 0) -> list:
    """Adam with a cosine decay from lr to lr_min over ``steps`` minibatches
    drawn from shuffled epochs of (x, y); returns the logged (step, loss)."""
    gen = torch.Generator(device=x.device)
    gen.manual_seed(seed)
    n = x.shape[0]
    batch = min(batch, n)
    perm = torch.randperm(n, generator=gen, device=x.device)
    pos = 0
    log = []
    for s in range(steps):
        if pos + batch > n:
            perm = torch.randperm(n, generator=gen, device=x.device)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * s / max(steps - 1, 1)))
        loss = net.loss_and_grad(x[idx], y[idx])
        net.adam(cur)
        if log_every and (s % log_every == 0 or s == steps - 1):
            log.append((s, float(loss.item())))
    net.check_tensor_cores()
    return log


def stress_errors(tau: torch.Tensor, tau_ref: torch.Tensor) -> dict:
    """Relative L2 over all rows and the per-row relative error quantiles."""
    d = (tau - tau_ref).double()
    r = tau_ref.double()
    rn = r.norm(dim=1)
    row = d.norm(dim=1) / rn.clamp_min(1e-30)
    ok = rn > 0
    q = torch.quantile(row[ok][:1_000_000].float(), torch.tensor([0.5, 0.99, 1.0], device=row.device))
    return {"rel_l2": float(d.norm() / r.norm().clamp_min(1e-30)), "row_p50": float(q[0]),
            "row_p99": float(q[1]), "row_max": float(q[2])}


def time_forward(rows: int = 1 << 20, device="cuda:0", reps: int = 20) -> dict:
    """Milliseconds per forward of ``rows`` rows: tcgen05 kernel and mma.sync
    kernel, CUDA events (random network, random inputs)."""
    dev = torch.device(device)
    g = torch.Generator(device=dev).manual_seed(0)
    x = torch.randn(rows, IN, generator=g, device=dev)
    out = {}
    for name, tc in (("tcgen05", True), ("mma_sync", False)):
        net = StressMLP(dev, seed=0, tensor_memory=tc)
        y = torch.empty(rows, OUT, device=dev)
        for _ in range(3):
            net.forward(x, out=y)
        st = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            net.forward(x, out=y)
        e1.record(st)
        torch.cuda.synchronize(dev)
        if tc:
            net.check_tensor_cores()
        ms = e0.elapsed_time(e1) / reps
        flops = 2.0 * rows * (IN * HID + HID * HID * 2 + HID * OUT)
        out[name] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12}
    return out


def time_training_step(rows: int = 65536, device="cuda:0", reps: int = 50) -> dict:
    """Milliseconds of the forward (with loss gradient), the backward and the
    Adam step on a batch of ``rows`` rows, tcgen05 and mma.sync kernels, CUDA
    events; the backward's TFLOP/s counts 2 x the forward's flops."""
    dev = torch.device(device)
    g = torch.Generator(device=dev).manual_seed(0)
    x = torch.randn(rows, IN, generator=g, device=dev)
    t = torch.tanh(torch.randn(rows, OUT, generator=g, device=dev))
    flops_fwd = 2.0 * rows * (IN * HID + HID * HID * 2 + HID * OUT)
    out = {}
    for name, tc in (("tcgen05", True), ("mma_sync", False)):
        net = StressMLP(dev, seed=0, tensor_memory=tc)
        for _ in range(3):
            net.train_step(x, t)
        b = net._buffers(rows)
        st = torch.cuda.current_stream(dev)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        acc = [0.0, 0.0, 0.0]
        for _ in range(reps):
            net.grad.zero_()
            net.loss.zero_()
            ev[0].record(st)
            net._forward(x, None, t, b["z"], b["dy"], net.loss, 2.0 / (rows * OUT), rows)
            ev[1].record(st)
            if tc:
                A.check(net.lib.mpm_mlp_backward_tc(_ptr(net.params), _ptr(x), _ptr(b["z"]), _ptr(b["dy"]),
                                                    _ptr(net.grad), rows, _ptr(net.tc_error), st.cuda_stream),
                        "mpm_mlp_backward_tc")
            else:
                A.check(net.lib.mpm_mlp_backward(_ptr(net.params), _ptr(x), _ptr(b["z"]), _ptr(b["dy"]),
                                                 _ptr(b["work"]), _ptr(net.grad), rows, st.cuda_stream),
                        "mpm_mlp_backward")
            ev[2].record(st)
            net.adam(1e-3)
            ev[3].record(st)
            torch.cuda.synchronize(dev)
            for i in range(3):
                acc[i] += ev[i].elapsed_time(ev[i + 1]) / reps
        net.check_tensor_cores()
        out[name] = {"forward_ms": acc[0], "backward_ms": acc[1], "adam_ms": acc[2],
                     "backward_tflops": 2.0 * flops_fwd / (acc[1] * 1e-3) / 1e12}
    return out


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time the stress-network kernels")
    ap.add_argument("--rows", type=int, default=1 << 20)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--training", action="store_true",
                    help="time a training step (forward, backward, Adam) instead of the forward")
    a = ap.parse_args()
    if a.training:
        print(json.dumps(time_training_step(a.rows, reps=a.reps)))
    else:
        print(json.dumps(time_forward(a.rows, reps=a.reps)))
