"""Differentiable sand rollouts: the library's hand-written adjoint behind a
``torch.autograd.Function``.

The reference has no gradient path (no ``wp.Tape``); this module adds one
for the substep it replaces (engine_stress/mpm_solver_warp.py:156-203).
``SandRollout.forward`` advances a sand scene from an initial velocity field
and a material (E, friction angle), keeping a checkpoint of the particle
state every ``checkpoint_every`` substeps and, with ``grid_tape`` (the
default), each substep's grid (``mpm_save_substep_grid``: sorted order,
chunk list, active blocks' momentum, mass and velocity).
``SandRollout.backward`` walks the segments newest first: it restores a
segment's checkpoint and recomputes the segment's states -- with the grid
tape by G2P alone from each substep's saved grid, without it by the whole
substep (sort, P2G, grid update, G2P), saving the grids on the way -- then
for each substep (newest first) loads its grid and calls
``mpm_adjoint_substep``, which runs the reverse G2P (with the return-map
adjoint), the reverse grid update and the reverse P2G on the device.  The adjoints of the initial
velocity and of (mu, lam, alpha) come out; the chain rule to E and the
friction angle is applied here.

``rollout(v0, E, friction_angle, sand)`` is the autograd entry point: the
final positions as a differentiable function of the three inputs.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _capi as A
from .batched import scene_params
from .engine import MPMEngine, dp_alpha, lame_from_E_nu
from .scenarios import Scene


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class SandRollout:
    """One sand scene, rolled out and differentiated on one device."""

    def __init__(self, scene: Scene, n_substeps: int | None = None, checkpoint_every: int = 10,
                 device="cuda:0", chunk_size: int = 128, particles=None, initial: dict | None = None,
                 grid_tape: bool = True, ordered: bool = True):
        """particles: (x0, v0, vol, mass) arrays overriding the scene's sampling;
        initial: {field id: (n, comps) tensor} loaded after them (e.g. a
        prestrained F with its stress); grid_tape: keep every substep's grid
        from the forward pass (n_substeps x mpm_substep_grid_bytes of device
        memory) so the backward pass recomputes states by G2P alone; ordered:
        P2G sums in a fixed order (mpm_p2g_ordered), so the forward is a
        deterministic function of (v0, E, friction angle) and finite
        differences of it are meaningful at small steps."""
        if scene.material != "sand":
            raise ValueError("the adjoint covers sand (Drucker-Prager) scenes only")
        if checkpoint_every < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.scene = scene
        self.n_substeps = int(n_substeps if n_substeps is not None else scene.substeps)
        self._k = 0
        self.dt = float(scene.dt)
        self.device = torch.device(device)
        self.params = scene_params(scene)
        self.engine = MPMEngine([self.params], device=self.device, chunk_size=chunk_size)
        self.engine.ordered = bool(ordered)
        self.lib = self.engine.lib
        x0, v0, vol, mass = scene.particles() if particles is None else particles
        self.n = x0.shape[0]
        if self.n != scene.n_particles:
            raise ValueError("particle arrays and scene.n_particles differ")
        self.initial = {f: torch.as_tensor(t).to(self.device, torch.float32) for f, t in (initial or {}).items()}
        self.state_bar = None
        self.x0 = torch.from_numpy(x0).to(self.device)
        self.v0_default = torch.from_numpy(v0).to(self.device)
        self.vol = torch.from_numpy(vol).to(self.device)
        self.mass = torch.from_numpy(mass).to(self.device)
        dev = self.device
        self.grid_adj = torch.empty(self.engine.plan.total_blocks * 64 * 4, dtype=torch.float32, device=dev)
        self.theta_bar = torch.zeros(3, dtype=torch.float64, device=dev)
        self.adj = [torch.zeros(self.n * A.ADJ_WORDS, dtype=torch.float32, device=dev) for _ in range(2)]
        self.grid_tape = bool(grid_tape)
        self.tape = None
        self.k = int(checkpoint_every)
        self.E = float(scene.E)
        self.friction_angle = float(scene.friction_angle)

    @property
    def k(self) -> int:
        """Checkpoint interval (substeps per recomputed segment)."""
        return self._k

    @k.setter
    def k(self, k: int) -> None:
        """Allocate the checkpoint storage: one state buffer per checkpoint,
        k + 1 state buffers for a recomputed segment, and k saved grids when
        there is no grid tape."""
        k = int(k)
        if k < 1:
            raise ValueError("checkpoint interval must be >= 1")
        if k == self._k:
            return
        dev = self.device
        sb = self.engine.plan.state_bytes
        gb = self.lib.mpm_substep_grid_bytes(C.byref(self.engine.plan))
        n_ckpt = (self.n_substeps + k - 1) // k
        self.checkpoints = [torch.empty(sb, dtype=torch.uint8, device=dev) for _ in range(n_ckpt)]
        self.pool = [torch.empty(sb, dtype=torch.uint8, device=dev) for _ in range(k + 1)]
        self.grids = None if self.grid_tape else [torch.empty(gb, dtype=torch.uint8, device=dev) for _ in range(k)]
        if self.grid_tape and self.tape is None:
            self.tape = [torch.empty(gb, dtype=torch.uint8, device=dev) for _ in range(self.n_substeps)]
        self.have_checkpoints = False
        self._k = k

    # ------------------------------------------------------------------ forward
    def set_material(self, E: float, friction_angle: float) -> None:
        self.E, self.friction_angle = float(E), float(friction_angle)
        p = self.params
        p.mu, p.lam = lame_from_E_nu(self.E, self.scene.nu)
        p.friction_angle = self.friction_angle
        self.engine.update_scenes()

    def _start(self, v0: torch.Tensor) -> None:
        e = self.engine
        e.reinit()
        e.load(A.FIELD_X_INITIAL, self.x0)
        e.load(A.FIELD_VOL, self.vol)
        e.load(A.FIELD_MASS, self.mass)
        e.load(A.FIELD_V, v0)
        for f, t in self.initial.items():
            e.load(f, t)

    def time_of(self, step: int) -> float:
        return step * self.dt

    def forward(self, v0: torch.Tensor, E: float, friction_angle: float, keep: bool = True) -> torch.Tensor:
        """Final displacements u (n, 3) (positions are x0 + u, see
        ``positions``); with keep, checkpoints for ``backward``."""
        self.set_material(E, friction_angle)
        self._start(v0.detach().to(self.device, torch.float32).reshape(self.n, 3))
        e = self.engine
        b = e.buf
        self.have_checkpoints = False
        for step in range(self.n_substeps):
            if keep and step % self.k == 0:
                self.checkpoints[step // self.k].copy_(e._state[b.cur])
            if keep and self.grid_tape:
                t = self.time_of(step)
                e.stage("sort")
                e.stage("p2g", dt=self.dt)
                e.stage("grid", time=t, dt=self.dt)
                self._call("mpm_save_substep_grid", self.tape[step].data_ptr())
                e.stage("g2p", dt=self.dt)
            else:
                e.substep_raw(self.time_of(step), self.dt)
        self.have_checkpoints = keep
        return e.export(A.FIELD_U).reshape(self.n, 3)

    def positions(self, u: torch.Tensor) -> torch.Tensor:
        """x0 + u in float64: differences of positions keep the displacement's digits."""
        return self.x0.double() + u.double()

    # ------------------------------------------------------------------ reverse
    def _call(self, name: str, *args) -> None:
        A.check(getattr(self.lib, name)(C.byref(self.engine.buf), *args, _stream(self.device)), name)

    def backward(self, x_bar: torch.Tensor):
        """Adjoints (v0 (n,3), E, friction angle) of <x_bar, x_final> (x_bar is
        also the adjoint of the final displacement).  x_bar may instead be a
        full (n, 36) seed on the final state (x, v, C, F, stress words as in
        mpm_adjoint_substep).  The adjoint of the whole initial state is left
        in ``state_bar`` (n, 36).

        Per segment (newest first): the segment's states are recomputed from
        its checkpoint straight into ``pool`` (G2P writes each new state into
        the next pool buffer: no copies) -- from the grid tape by G2P alone,
        otherwise by whole substeps whose grids are saved after their grid
        update -- then the substeps are reversed newest first from their pool
        state and saved grid."""
        if not self.have_checkpoints:
            raise RuntimeError("run forward(keep=True) first")
        e = self.engine
        b = e.buf
        out, inp = self.adj
        out.zero_()
        seed = x_bar.to(self.device, torch.float32)
        if seed.numel() == self.n * A.ADJ_WORDS:
            out.copy_(seed.reshape(-1))
        else:
            out.view(self.n, A.ADJ_WORDS)[:, A.ADJ_X:A.ADJ_X + 3] = seed.reshape(self.n, 3)
        self.theta_bar.zero_()
        own = (b.state[0], b.state[1])
        cur0, substep0 = b.cur, b.substep
        try:
            for seg in reversed(range(len(self.checkpoints))):
                start = seg * self.k
                L = min(self.k, self.n_substeps - start)
                self.pool[0].copy_(self.checkpoints[seg])
                b.state[b.cur] = self.pool[0].data_ptr()
                b.keys_valid = 0
                self._call("mpm_clear_grid")
                for j in range(L):
                    t = self.time_of(start + j)
                    if j + 1 < L:
                        b.state[b.cur ^ 1] = self.pool[j + 1].data_ptr()
                    if self.grid_tape:
                        if j + 1 < L:
                            self._call("mpm_load_substep_grid", self.tape[start + j].data_ptr())
                            e.stage("g2p", dt=self.dt)
                        continue
                    e.stage("sort")
                    e.stage("p2g", dt=self.dt)
                    e.stage("grid", time=t, dt=self.dt)
                    self._call("mpm_save_substep_grid", self.grids[j].data_ptr())
                    if j + 1 < L:
                        e.stage("g2p", dt=self.dt)
                for j in reversed(range(L)):
                    b.state[b.cur] = self.pool[j].data_ptr()
                    blob = self.tape[start + j] if self.grid_tape else self.grids[j]
                    self._call("mpm_load_substep_grid", blob.data_ptr())
                    A.check(self.lib.mpm_adjoint_substep(C.byref(b), out.data_ptr(), inp.data_ptr(),
                                                         self.grid_adj.data_ptr(), self.theta_bar.data_ptr(),
                                                         self.time_of(start + j), self.dt, _stream(self.device)),
                            "mpm_adjoint_substep")
                    out, inp = inp, out
        finally:
            b.state[0], b.state[1] = own
            b.cur, b.substep = cur0, substep0
            b.keys_valid = 0
            self._call("mpm_clear_grid")
        self.state_bar = out.view(self.n, A.ADJ_WORDS).clone()
        v0_bar = self.state_bar[:, A.ADJ_V:A.ADJ_V + 3].clone()
        mu_b, lam_b, alpha_b = (float(x) for x in self.theta_bar.cpu())
        nu = self.scene.nu
        E_bar = mu_b / (2.0 * (1.0 + nu)) + lam_b * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
        # alpha = sqrt(2/3) 2 sin(phi) / (3 - sin(phi)), phi in degrees (mpm_solver_warp.py:113-116)
        pi = 3.14159265
        s = math.sin(self.friction_angle / 180.0 * pi)
        dalpha_dphi = math.sqrt(2.0 / 3.0) * 6.0 / (3.0 - s) ** 2 * math.cos(self.friction_angle / 180.0 * pi) * pi / 180.0
        return v0_bar, E_bar, alpha_b * dalpha_dphi

    def alpha(self) -> float:
        return dp_alpha(self.friction_angle)


class _RolloutFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0, E, friction_angle, sand: SandRollout):
        u = sand.forward(v0, float(E), float(friction_angle), keep=True)
        ctx.sand = sand
        ctx.dtypes = (E.dtype, friction_angle.dtype, v0.dtype)
        return sand.positions(u)

    @staticmethod
    def backward(ctx, x_bar):
        v0_bar, E_bar, phi_bar = ctx.sand.backward(x_bar)
        dev = x_bar.device
        return (v0_bar.to(ctx.dtypes[2]), torch.tensor(E_bar, dtype=ctx.dtypes[0], device=dev),
                torch.tensor(phi_bar, dtype=ctx.dtypes[1], device=dev), None)


def rollout(v0: torch.Tensor, E: torch.Tensor, friction_angle: torch.Tensor, sand: SandRollout) -> torch.Tensor:
    """Final particle positions (n, 3, float64: x0 + u) of ``sand``'s scene,
    differentiable in the initial velocity v0 (n, 3), Young's modulus E and
    the friction angle (degrees), both 0-d tensors."""
    E = torch.as_tensor(E, dtype=torch.float64)
    friction_angle = torch.as_tensor(friction_angle, dtype=torch.float64)
    return _RolloutFunction.apply(v0, E, friction_angle, sand)
