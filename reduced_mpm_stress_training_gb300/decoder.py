"""The reference's stress decoder in the simulation loop, on the GPU.

``StressDecoder`` holds the parameters of NetDec
(offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301) in the
packed float32 layout of ``MpmStressDecoder`` (include/mpm_gb300.h) and runs
them with the library's kernels (csrc/mpm_decoder.cu):

* ``forward(rows)`` -- NetDec.forward on (n, label_dim + 3 + mu_dim) rows ->
  (n, 6) stress components [xx, xy, xz, yy, yz, zz];
* ``stress_into(engine, label, mu)`` -- the reduced-order loop's stress
  source: each particle's row is (the frame's label, its x_initial, its mu
  row) and the decoded symmetric stress is written into the particle state,
  where the next substep's P2G reads it (the reference goes through
  load_uvstress_from_tensor, engine_stress/mpm_solver_warp.py:253-266).

Parameters come from a NetDec (or CROMnet_secondary, ``decoder.`` prefix)
state dict, or from ``StressDecoder.random`` with the reference's
initialisation (init_weights, :251-269).  The reference's trained weights are
not part of its snapshot.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _capi as A

_HIDDEN = ("dec1", "dec2", "dec3", "dec4")


def _strip(sd: dict, dtype=torch.float32) -> dict:
    if any(k.startswith("decoder.") for k in sd):
        sd = {k[len("decoder."):]: v for k, v in sd.items() if k.startswith("decoder.")}
    return {k: torch.as_tensor(v, dtype=dtype).detach().to("cpu") for k, v in sd.items()}


def pack(sd: dict, siren: bool, dtype=torch.float32) -> torch.Tensor:
    """NetDec state dict -> the packed blob (CPU; float32 is what the kernels take)."""
    sd = _strip(sd, dtype)
    prep = ("prepare.min_x_torch", "prepare.max_x_torch") if siren else \
        ("prepare.mean_x_torch", "prepare.std_x_torch")
    parts = [sd["dec0.weight"], sd["dec0.bias"]]
    parts += [sd[f"{n}.weight"] for n in _HIDDEN] + [sd[f"{n}.bias"] for n in _HIDDEN]
    parts += [sd["enc.weight"], sd["enc.bias"], sd[prep[0]], sd[prep[1]],
              sd["invStandardizeQ.mean_q_torch"], sd["invStandardizeQ.std_q_torch"]]
    return torch.cat([p.reshape(-1) for p in parts])


def netdec_state_dict(label_dim: int = 6, scale_mlp: int = 10, mu_dim: int = 1, siren: bool = False,
                      omega_0: float = 30.0, seed: int = 0, x_stats=None, q_stats=None) -> dict:
    """A NetDec state dict with the reference's initialisation (:251-269): xavier-uniform
    weights (SIREN: uniform +-sqrt(6 / in) / omega_0, the first layer +-1 / in) and
    nn.Linear's default biases (uniform +-1 / sqrt(in)), from a seeded generator.
    x_stats: (a, b) of the position preparation (mean and std, or min and max with SIREN;
    default 0 and 1), q_stats: (mean_q, std_q) (default 0 and 1)."""
    g = torch.Generator().manual_seed(seed)
    hidden = 3 * scale_mlp
    n_in = label_dim + 3 + mu_dim
    shapes = [("dec0", hidden, n_in)] + [(n, hidden, hidden) for n in _HIDDEN] + [("enc", 6, hidden)]
    sd = {}
    for name, fo, fi in shapes:
        if siren:
            lim = 1.0 / fi if name == "dec0" else math.sqrt(6.0 / fi) / omega_0
        else:
            lim = math.sqrt(6.0 / (fi + fo))
        sd[f"{name}.weight"] = (torch.rand(fo, fi, generator=g) * 2 - 1) * lim
        sd[f"{name}.bias"] = (torch.rand(fo, generator=g) * 2 - 1) / math.sqrt(fi)
    a, b = x_stats if x_stats is not None else ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    keys = ("min_x_torch", "max_x_torch") if siren else ("mean_x_torch", "std_x_torch")
    sd[f"prepare.{keys[0]}"] = torch.tensor(a, dtype=torch.float32)
    sd[f"prepare.{keys[1]}"] = torch.tensor(b, dtype=torch.float32)
    qm, qs = q_stats if q_stats is not None else ((0.0,) * 6, (1.0,) * 6)
    sd["invStandardizeQ.mean_q_torch"] = torch.tensor(qm, dtype=torch.float32)
    sd["invStandardizeQ.std_q_torch"] = torch.tensor(qs, dtype=torch.float32)
    return sd


class StressDecoder:
    """NetDec parameters on the device plus their MpmStressDecoder descriptor."""

    def __init__(self, state_dict: dict, siren: bool = False, omega_0: float = 30.0, mu_dim: int = 1,
                 device="cuda:0"):
        sd = _strip(state_dict)
        hidden, n_in = sd["dec0.weight"].shape
        if sd["enc.weight"].shape != (6, hidden):
            raise ValueError("the decoder's output layer must map hidden -> 6 stress components")
        self.hidden, self.mu_dim = int(hidden), int(mu_dim)
        self.label_dim = int(n_in) - 3 - self.mu_dim
        if self.label_dim < 0:
            raise ValueError("dec0 has fewer inputs than x (3) and mu")
        self.siren, self.omega_0 = bool(siren), float(omega_0)
        self.device = torch.device(device)
        self.state_dict = sd
        self.params = pack(sd, self.siren).to(self.device)
        self.desc = A.MpmStressDecoder(self.params.data_ptr(), self.label_dim, self.mu_dim, self.hidden,
                                       int(self.siren), self.omega_0, 0)
        lib = A.load()
        count = lib.mpm_decoder_param_count(C.byref(self.desc))
        if count != self.params.numel():
            raise ValueError(f"decoder dimensions not supported (label {self.label_dim}, mu {self.mu_dim}, "
                             f"hidden {self.hidden}): library expects {count} parameters")
        self._lib = lib

    @classmethod
    def random(cls, label_dim: int = 6, scale_mlp: int = 10, mu_dim: int = 1, siren: bool = False,
               omega_0: float = 30.0, seed: int = 0, x_stats=None, q_stats=None, device="cuda:0"):
        """A decoder with the reference's initialisation (see ``netdec_state_dict``)."""
        sd = netdec_state_dict(label_dim, scale_mlp, mu_dim, siren, omega_0, seed, x_stats, q_stats)
        return cls(sd, siren=siren, omega_0=omega_0, mu_dim=mu_dim, device=device)

    @property
    def n_in(self) -> int:
        return self.label_dim + 3 + self.mu_dim

    def forward(self, rows: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """NetDec.forward (:288-291): rows (n, label_dim + 3 + mu_dim) -> (n, 6)."""
        rows = torch.as_tensor(rows).to(self.device, torch.float32).contiguous()
        if rows.dim() != 2 or rows.shape[1] != self.n_in:
            raise ValueError(f"rows must be (n, {self.n_in})")
        n = rows.shape[0]
        if out is None:
            out = torch.empty((n, 6), dtype=torch.float32, device=self.device)
        A.check(self._lib.mpm_decoder_forward(C.byref(self.desc), rows.data_ptr(), out.data_ptr(), n,
                                              torch.cuda.current_stream(self.device).cuda_stream),
                "mpm_decoder_forward")
        return out

    def stress_into(self, engine, label, mu=None) -> None:
        """Decode every particle's stress into the engine's state (mpm_decoder_stress):
        label (label_dim,) the frame's latent, mu (n, mu_dim) in user order."""
        lab = torch.as_tensor(label).to(self.device, torch.float32).reshape(-1).contiguous()
        if lab.numel() != self.label_dim:
            raise ValueError(f"label must hold {self.label_dim} values")
        n = engine.n_particles
        mu_t = None
        if self.mu_dim:
            if mu is None:
                raise ValueError("this decoder takes a mu row per particle")
            mu_t = torch.as_tensor(mu).to(self.device, torch.float32).reshape(n, self.mu_dim).contiguous()
        A.check(self._lib.mpm_decoder_stress(C.byref(engine.buf), C.byref(self.desc),
                                             lab.data_ptr() if self.label_dim else None,
                                             mu_t.data_ptr() if mu_t is not None else None, engine.stream),
                "mpm_decoder_stress")
