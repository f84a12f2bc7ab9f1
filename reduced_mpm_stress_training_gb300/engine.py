"""Host side of the GB300 substep: buffers, scene table, stages, status.

``MPMEngine`` owns the device memory (PyTorch tensors) of one or many scenes
and drives libmpm_gb300.so through its C ABI on the current PyTorch CUDA
stream.  The single-scene drop-in ``MPM_Simulator_WARP`` (solver.py) and
the batched multi-scene runner (batched.py) are both thin layers over it.

Particle data crosses this boundary only in the reference's layout -- AoS,
user particle order, vec3 = 3 floats, mat33 = 9 floats row-major
(engine_stress/warp_utils.py:5-43) -- and lives on the device in the
library's sorted structure-of-arrays layout in between.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import warnings

import torch

from . import _capi as A

_MATERIALS = {"jelly": A.JELLY, "metal": A.METAL, "sand": A.SAND}


class MPMStatusError(RuntimeError):
    """The device status word reported a physics fault (see ``status_text``)."""

    def __init__(self, bits: int):
        self.bits = bits
        super().__init__(f"MPM status 0x{bits:x}: {A.status_text(bits)}")


def material_code(material) -> int:
    """engine_stress/mpm_solver_warp.py:90-94 (TypeError on an unknown name)."""
    if isinstance(material, int) and material in (0, 1, 2):
        return material
    if material not in _MATERIALS:
        raise TypeError("Undefined material type")
    return _MATERIALS[material]


def lame_from_E_nu(E: float, nu: float) -> tuple[float, float]:
    """engine_stress/mpm_solver_warp.py:41-42"""
    return E / 2.0 / (1.0 + nu), E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)


def dp_alpha(friction_angle: float) -> float:
    """Drucker-Prager alpha, engine_stress/mpm_solver_warp.py:113-116."""
    sin_phi = math.sin(friction_angle / 180.0 * 3.14159265)
    return math.sqrt(2.0 / 3.0) * 2.0 * sin_phi / (3.0 - sin_phi)


@dataclasses.dataclass
class Collider:
    """Dirichlet_collider (engine_stress/warp_utils.py:126-151) of one of the
    reference's grid boundary conditions (engine_stress/mpm_solver_warp.py:407-720)."""
    kind: int
    point: tuple = (0.0, 0.0, 0.0)
    normal: tuple = (0.0, 0.0, 1.0)
    surface_type: int = 0
    friction: float = 0.0
    start_time: float = 0.0
    end_time: float = 999.0
    reset: int = 0
    velocity: tuple = (0.0, 0.0, 0.0)
    threshold: float = 0.0
    radius: float = 0.0
    width: float = 0.0
    height: float = 0.0
    v_scale: float = 0.0
    x_unit: tuple = (1.0, 0.0, 0.0)
    y_unit: tuple = (0.0, 1.0, 0.0)
    R: float = 0.0

    @staticmethod
    def _unit(v):
        scale = 1.0 / math.sqrt(sum(x ** 2 for x in v))
        return tuple(scale * x for x in v)

    @staticmethod
    def surface(point, normal, surface="sticky", friction=0.0, start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:407-428 (normal normalised, sticky needs friction 0)."""
        if surface == "sticky" and friction != 0:
            raise ValueError("friction must be 0 on sticky surfaces.")
        st = 0 if surface == "sticky" else (1 if surface == "slip" else 2)
        return Collider(A.COLLIDER_SURFACE, tuple(point), Collider._unit(normal), st, friction,
                        start_time, end_time)

    @staticmethod
    def bounding_box(start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:499-503"""
        return Collider(A.COLLIDER_BOX, start_time=start_time, end_time=end_time)

    @staticmethod
    def velocity_plane(point, normal, velocity, threshold, start_time=0.0, end_time=999.0, reset=0):
        """engine_stress/mpm_solver_warp.py:527-543: the slab |(x - point).normal| <=
        threshold takes `velocity` and moves with it."""
        return Collider(A.COLLIDER_VPLANE, tuple(point), Collider._unit(normal), start_time=start_time,
                        end_time=end_time, reset=int(reset), velocity=tuple(velocity),
                        threshold=float(threshold))

    @staticmethod
    def circle_column(R, radius, height, v_scale, start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:570-579: a vertical column (radius,
        half-height) whose bottom point starts at (0.5, 0.069, 0.5 + R) and
        circles about (0.5, *, 0.5) at speed v_scale."""
        return Collider(A.COLLIDER_CIRCLE, (0.5, 0.069, 0.5 + R), start_time=start_time, end_time=end_time,
                        radius=float(radius), height=float(height), v_scale=float(v_scale), R=float(R))

    @staticmethod
    def rotating_disk(point, normal, radius, width, v_scale, start_time=0.0, end_time=999.0, reset=0):
        """engine_stress/mpm_solver_warp.py:609-633: in-plane axes from the
        normalised normal as the reference builds them.  The reference's axis
        search never advances past normal[0] (it loops forever when
        |normal[0]| <= 0.1); that case raises here instead."""
        n = Collider._unit(normal)
        if not abs(n[0]) > 1e-1:
            raise ValueError("set_rotation_on_disk needs |normal[0]| > 0.1 after normalisation "
                             "(the reference's local-axis search does not terminate otherwise)")
        x = [1.0, 1.0, 1.0]
        x[0] = -(n[0] + n[1] + n[2] - n[0]) / n[0]
        y = [n[1] * x[2] - n[2] * x[1], n[2] * x[0] - n[0] * x[2], n[0] * x[1] - n[1] * x[0]]
        return Collider(A.COLLIDER_DISK, tuple(point), n, start_time=start_time, end_time=end_time,
                        reset=int(reset), radius=float(radius), width=float(width), v_scale=float(v_scale),
                        x_unit=Collider._unit(x), y_unit=Collider._unit(y))

    @staticmethod
    def velocity_cube(point, width, velocity, start_time=0.0, end_time=999.0, reset=0):
        """engine_stress/mpm_solver_warp.py:667-679: nodes within `width` of
        the point (each axis) take `velocity`; the cube moves with it."""
        return Collider(A.COLLIDER_CUBE, tuple(point), start_time=start_time, end_time=end_time,
                        reset=int(reset), velocity=tuple(velocity), width=float(width))

    @staticmethod
    def sphere(center, radius, velocity, start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:697-707 (add_sphere_leader)."""
        return Collider(A.COLLIDER_SPHERE, tuple(center), start_time=start_time, end_time=end_time,
                        velocity=tuple(velocity), radius=float(radius))

    def to_struct(self) -> A.MpmCollider:
        c = A.MpmCollider()
        c.kind = self.kind
        c.surface_type = self.surface_type
        for i in range(3):
            c.point[i] = self.point[i]
            c.normal[i] = self.normal[i]
            c.velocity[i] = self.velocity[i]
            c.x_unit[i] = self.x_unit[i]
            c.y_unit[i] = self.y_unit[i]
        c.friction = self.friction
        c.start_time = self.start_time
        c.end_time = self.end_time
        c.reset = self.reset
        c.threshold = self.threshold
        c.radius = self.radius
        c.width = self.width
        c.height = self.height
        c.v_scale = self.v_scale
        c.R = self.R
        return c


@dataclasses.dataclass
class SceneParams:
    """MPMModelStruct (engine_stress/warp_utils.py:61-81) of one scene."""
    n_particles: int
    n_grid: int = 100
    grid_lim: float = 1.0
    material: int = A.JELLY
    mu: float = 1000 / 2.0 / 1.3           # E=1000, nu=0.3 defaults (:39-42)
    lam: float = 1000 * 0.3 / 1.3 / 0.4
    friction_angle: float = 25.0           # (:46-48)
    hardening: int = 0
    xi: float = 0.0
    gravity: tuple = (0.0, 0.0, 0.0)       # reference default g = 0 (:49)
    colliders: list = dataclasses.field(default_factory=list)

    @property
    def dx(self) -> float:
        return self.grid_lim / self.n_grid

    @property
    def inv_dx(self) -> float:
        return float(self.n_grid / self.grid_lim)

    def to_struct(self, particle_begin: int) -> A.MpmScene:
        s = A.MpmScene()
        s.n_grid = self.n_grid
        s.material = self.material
        s.hardening = int(self.hardening)
        if len(self.colliders) > A.MPM_MAX_COLLIDERS:
            raise ValueError(f"at most {A.MPM_MAX_COLLIDERS} colliders per scene")
        s.n_colliders = len(self.colliders)
        s.dx = self.dx
        s.inv_dx = self.inv_dx
        s.mu = self.mu
        s.lam = self.lam
        s.alpha = dp_alpha(self.friction_angle)
        s.xi = self.xi
        for i in range(3):
            s.gravity[i] = self.gravity[i]
        s.particle_begin = particle_begin
        s.particle_count = self.n_particles
        for k, c in enumerate(self.colliders):
            s.colliders[k] = c.to_struct()
        return s


def _stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class MPMEngine:
    """Device buffers + C-ABI driver for one or more scenes (concatenated)."""

    def __init__(self, scenes: list[SceneParams], device="cuda:0", chunk_size: int = 128):
        self.lib = A.load()
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("MPMEngine runs on a CUDA device only (no CPU path)")
        self.scenes = list(scenes)
        self.chunk_size = chunk_size
        self.on_error = "raise"
        self._pending = None
        self.surrogate = None
        self._ordered_scratch = None
        self._allocate(fresh=True)

    # ------------------------------------------------------------------ layout
    @property
    def n_particles(self) -> int:
        return sum(s.n_particles for s in self.scenes)

    def _scene_table(self):
        arr = (A.MpmScene * len(self.scenes))()
        begin = 0
        for i, s in enumerate(self.scenes):
            arr[i] = s.to_struct(begin)
            begin += s.n_particles
        return arr

    def _allocate(self, fresh: bool) -> None:
        """Plan and allocate; fresh=False keeps the particle state (grid change)."""
        if not fresh:
            self._sync_moving_colliders()
        table = self._scene_table()
        plan = A.MpmPlan()
        A.check(self.lib.mpm_plan(table, len(self.scenes), self.n_particles, self.chunk_size,
                                  C.byref(plan)), "mpm_plan")
        self.table = table
        self.plan = plan
        dev = self.device
        with torch.cuda.device(dev):
            if fresh:
                self._state = [torch.empty(plan.state_bytes, dtype=torch.uint8, device=dev)
                               for _ in range(2)]
                self._status = torch.zeros(1, dtype=torch.int32, device=dev)
                self._status_host = torch.zeros(1, dtype=torch.int32).pin_memory()
                self._status_event = torch.cuda.Event()
            self._workspace = torch.zeros(plan.workspace_bytes, dtype=torch.uint8, device=dev)
            self._scenes_dev = torch.empty(C.sizeof(A.MpmScene) * len(self.scenes),
                                           dtype=torch.uint8, device=dev)
        b = A.MpmBuffers() if fresh else self.buf
        b.state[0] = self._state[0].data_ptr()
        b.state[1] = self._state[1].data_ptr()
        b.workspace = self._workspace.data_ptr()
        b.scenes = self._scenes_dev.data_ptr()
        b.status = self._status.data_ptr()
        b.plan = plan
        self.buf = b
        self._upload(sync=False)  # moving points were read back above (the device table is new)
        if fresh:
            A.check(self.lib.mpm_init(C.byref(b), self.stream), "mpm_init")
        else:
            b.keys_valid = 0  # block keys depend on the grid
        if self._ordered_scratch is not None:  # sized by the plan's grid blocks
            self._ordered_scratch = None
            self.ordered = True

    def _sync_moving_colliders(self) -> None:
        """Moving colliders advance on the device (mpm_grid_update); copy their
        current points back into the scene parameters before a re-upload."""
        if getattr(self, "table", None) is None or not (self.buf.collider_flags & A.CF_MOVING):
            return
        dev = (A.MpmScene * len(self.scenes)).from_buffer_copy(self._scenes_dev.cpu().numpy().tobytes())
        for i, sp in enumerate(self.scenes):
            for k, c in enumerate(sp.colliders[:dev[i].n_colliders]):
                if c.kind in A.MOVING_COLLIDERS and dev[i].colliders[k].kind == c.kind:
                    c.point = tuple(float(x) for x in dev[i].colliders[k].point)

    def _upload(self, sync: bool = True) -> None:
        if sync:
            self._sync_moving_colliders()
        table = self._scene_table()
        A.check(self.lib.mpm_plan(table, len(self.scenes), self.n_particles, self.chunk_size,
                                  C.byref(A.MpmPlan())), "mpm_plan")
        self.table = table
        A.check(self.lib.mpm_upload_scenes(C.byref(self.buf), table, len(self.scenes),
                                           self.stream), "mpm_upload_scenes")

    def update_scenes(self, regrid: bool = False) -> None:
        """Push changed scene parameters; regrid=True when n_grid/grid_lim changed."""
        if regrid:
            self._allocate(fresh=False)
        else:
            self._upload()

    @property
    def stream(self) -> int:
        return _stream_handle(self.device)

    # ------------------------------------------------------------------ data
    def _as_input(self, t, comps: int) -> torch.Tensor:
        t = torch.as_tensor(t)
        n = self.n_particles
        if t.numel() != n * comps:
            raise ValueError(f"expected {n} x {comps} values, got shape {tuple(t.shape)}")
        return t.detach().to(device=self.device, dtype=torch.float32).reshape(n * comps).contiguous()

    def load(self, field: int, t) -> None:
        src = self._as_input(t, A.FIELD_COMPONENTS[field])
        # src is stream-ordered on the current stream, so the caching
        # allocator cannot hand its memory out before the load kernel ran
        A.check(self.lib.mpm_load(C.byref(self.buf), field, src.data_ptr(), 0, self.stream),
                "mpm_load")

    def load_host(self, field: int, host: torch.Tensor) -> None:
        """Load from a (pinned) host tensor through the library's staging copy."""
        assert host.device.type == "cpu" and host.dtype == torch.float32 and host.is_contiguous()
        A.check(self.lib.mpm_load(C.byref(self.buf), field, host.data_ptr(), 1, self.stream),
                "mpm_load")

    def export(self, field: int, out: torch.Tensor | None = None) -> torch.Tensor:
        comps = A.FIELD_COMPONENTS[field]
        n = self.n_particles
        if out is None:
            out = torch.empty(n * comps, dtype=torch.float32, device=self.device)
        on_host = out.device.type == "cpu"
        A.check(self.lib.mpm_export(C.byref(self.buf), field, out.data_ptr(), int(on_host),
                                    self.stream), "mpm_export")
        return out

    def load_uvstress(self, u: torch.Tensor, v: torch.Tensor, stress: torch.Tensor) -> None:
        """u (n,3), v (n,3), stress (n,3,3) in one pass (mpm_load_uvstress):
        straight from pinned float32 host tensors through the staging copy,
        anything else by way of device tensors."""
        n = self.n_particles
        ts = (u, v, stress)
        if all(t.device.type == "cpu" and t.is_pinned() and t.dtype == torch.float32 and t.is_contiguous()
               and t.numel() == n * c for t, c in zip(ts, (3, 3, 9))):
            ts = [t.reshape(-1) for t in ts]
            A.check(self.lib.mpm_load_uvstress(C.byref(self.buf), ts[0].data_ptr(), ts[1].data_ptr(),
                                               ts[2].data_ptr(), 1, self.stream), "mpm_load_uvstress")
            return
        src = [self._as_input(t, c) for t, c in zip((u, v, stress), (3, 3, 9))]
        A.check(self.lib.mpm_load_uvstress(C.byref(self.buf), src[0].data_ptr(), src[1].data_ptr(),
                                           src[2].data_ptr(), 0, self.stream), "mpm_load_uvstress")

    def export_uvFstress(self, out: tuple | None = None, wait: bool = True) -> tuple:
        """(u, v, F_disp, stress) flat float32 tensors in one pass
        (mpm_export_uvFstress): into `out` (four device tensors, or four
        pinned host tensors of n*3, n*3, n*9, n*9 floats) or new device ones.
        Host tensors with wait=False are filled asynchronously: call
        ``sync_transfers()`` (or synchronize the device) before reading them."""
        n = self.n_particles
        if out is None:
            out = tuple(torch.empty(n * c, dtype=torch.float32, device=self.device) for c in (3, 3, 9, 9))
        on_host = out[0].device.type == "cpu"
        for t, c in zip(out, (3, 3, 9, 9)):
            assert t.dtype == torch.float32 and t.is_contiguous() and t.numel() == n * c
            assert (t.device.type == "cpu") == on_host
        mode = (1 if wait else 2) if on_host else 0
        A.check(self.lib.mpm_export_uvFstress(C.byref(self.buf), *(t.data_ptr() for t in out), mode,
                                              self.stream), "mpm_export_uvFstress")
        return out

    def sync_transfers(self) -> None:
        """Wait for host copies left in flight by load_uvstress / export_uvFstress."""
        A.check(self.lib.mpm_sync_transfers(), "mpm_sync_transfers")

    def export_grid(self, scene: int = 0):
        ng = self.scenes[scene].n_grid
        gm = torch.empty((ng, ng, ng), dtype=torch.float32, device=self.device)
        gvin = torch.empty((ng, ng, ng, 3), dtype=torch.float32, device=self.device)
        gvout = torch.empty((ng, ng, ng, 3), dtype=torch.float32, device=self.device)
        A.check(self.lib.mpm_export_grid(C.byref(self.buf), scene, gm.data_ptr(), gvin.data_ptr(),
                                         gvout.data_ptr(), self.stream), "mpm_export_grid")
        return gm, gvin, gvout

    # ------------------------------------------------------------------ stepping
    def set_stress_surrogate(self, surrogate) -> None:
        """Route the return map + stress of sand particles through a trained
        ``surrogate.StressSurrogate`` (None restores the SVD path)."""
        if surrogate is not None:
            surrogate.bind(self)
        self.surrogate = surrogate

    @property
    def ordered(self) -> bool:
        """True: substeps use the ordered P2G (mpm_p2g2p_ordered), whose sums do
        not depend on the order in which warps run, so a run is a deterministic
        function of its inputs (finite-difference gradient checks need that)."""
        return self._ordered_scratch is not None

    @ordered.setter
    def ordered(self, on: bool) -> None:
        if on and self._ordered_scratch is None:
            nbytes = int(self.lib.mpm_p2g_ordered_bytes(C.byref(self.plan)))
            self._ordered_scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        elif not on:
            self._ordered_scratch = None

    def _p2g2p(self, time: float, dt: float) -> None:
        sur = self.surrogate
        if sur is None and self._ordered_scratch is not None:
            A.check(self.lib.mpm_p2g2p_ordered(C.byref(self.buf), self._ordered_scratch.data_ptr(), time, dt,
                                               self.stream), "mpm_p2g2p_ordered")
        elif sur is None:
            A.check(self.lib.mpm_p2g2p(C.byref(self.buf), time, dt, self.stream), "mpm_p2g2p")
        else:
            A.check(self.lib.mpm_p2g2p_surrogate(C.byref(self.buf), sur.params_ptr(), C.byref(sur.cfg),
                                                 sur.fallback.data_ptr(), sur.stats.data_ptr(), time,
                                                 dt, self.stream), "mpm_p2g2p_surrogate")

    def substep(self, time: float, dt: float) -> None:
        self.poll_status()
        self._p2g2p(time, dt)
        self._queue_status()

    def substep_raw(self, time: float, dt: float) -> None:
        """One substep without the lazy status bookkeeping (safe inside a
        CUDA-graph capture)."""
        self._p2g2p(time, dt)

    def graph(self, n_substeps: int, time: float, dt: float) -> "SubstepGraph":
        """Capture n_substeps substeps in one CUDA graph (see SubstepGraph)."""
        return SubstepGraph(self, n_substeps, time, dt)

    def stage(self, name: str, time: float = 0.0, dt: float = 0.0) -> None:
        b = C.byref(self.buf)
        s = self.stream
        if name == "sort":
            A.check(self.lib.mpm_sort(b, s), "mpm_sort")
        elif name == "p2g" and self._ordered_scratch is not None:
            A.check(self.lib.mpm_p2g_ordered(b, self._ordered_scratch.data_ptr(), dt, s), "mpm_p2g_ordered")
        elif name == "p2g":
            A.check(self.lib.mpm_p2g(b, dt, s), "mpm_p2g")
        elif name == "grid":
            A.check(self.lib.mpm_grid_update(b, time, dt, s), "mpm_grid_update")
        elif name == "g2p":
            A.check(self.lib.mpm_g2p(b, dt, s), "mpm_g2p")
        else:
            raise ValueError(name)

    # ------------------------------------------------------------------ reduced substep
    def _single_scene(self, what: str) -> None:
        if len(self.scenes) != 1:
            raise ValueError(f"{what} serves single-scene engines")

    def p2g2p_reduced(self, grid: "ReducedGrid", time: float, dt: float) -> None:
        """The reduced sampled-quadrature substep into ``grid`` (mpm_p2g2p_reduced)."""
        self._single_scene("p2g2p_reduced")
        g = grid.struct(self)
        self.poll_status()
        A.check(self.lib.mpm_p2g2p_reduced(C.byref(self.buf), C.byref(g), time, dt, self.stream),
                "mpm_p2g2p_reduced")
        self._queue_status()

    def mark_neighboring_cells_grid_v(self, grid: "ReducedGrid") -> None:
        """Add the -2..4 marks of the sample points (mpm_mark_neighboring_cells_grid_v)."""
        self._single_scene("experiment_for_C")
        g = grid.struct(self)
        self.poll_status()
        A.check(self.lib.mpm_mark_neighboring_cells_grid_v(C.byref(self.buf), C.byref(g), self.stream),
                "mpm_mark_neighboring_cells_grid_v")
        self._queue_status()

    def g2p_sample(self, grid: "ReducedGrid", dt: float) -> None:
        """The sample points' gather from grid.grid_v_out (mpm_g2p_sample)."""
        self._single_scene("g2p_sample")
        g = grid.struct(self)
        self.poll_status()
        A.check(self.lib.mpm_g2p_sample(C.byref(self.buf), C.byref(g), dt, self.stream), "mpm_g2p_sample")
        self._queue_status()

    # ------------------------------------------------------------------ checkpoints
    def reinit(self) -> None:
        """Back to the freshly initialised state (mpm_init: zero state, F = I,
        identity order); the caller reloads the particle fields."""
        A.check(self.lib.mpm_init(C.byref(self.buf), self.stream), "mpm_init")

    def snapshot(self) -> tuple:
        """Device copy of the live particle state (records and cell keys) with
        the host-side control needed to resume from it."""
        b = self.buf
        return (self._state[b.cur].clone(), int(b.cur), int(b.substep))

    def restore(self, snap: tuple) -> None:
        """Resume from a snapshot (the grid is rebuilt by the next substep)."""
        data, cur, substep = snap
        b = self.buf
        self._state[cur].copy_(data)
        b.cur = cur
        b.substep = substep
        b.keys_valid = 0  # the workspace histograms belong to another state

    # ------------------------------------------------------------------ status
    def _queue_status(self) -> None:
        self._status_host.copy_(self._status, non_blocking=True)
        self._status_event.record(torch.cuda.current_stream(self.device))
        self._pending = True

    def poll_status(self, wait: bool = False) -> int:
        """Read the status word copied after the last substep (lazy; no sync
        unless wait=True) and act on it per ``on_error``."""
        if not self._pending:
            return 0
        if not wait and not self._status_event.query():
            return 0
        self._status_event.synchronize()
        self._pending = False
        bits = int(self._status_host.item())
        if bits:
            self._status.zero_()
            if self.on_error == "raise":
                raise MPMStatusError(bits)
            if self.on_error == "warn":
                warnings.warn(str(MPMStatusError(bits)))
        return bits

    def status(self) -> int:
        """Synchronously read (without clearing) the device status word."""
        return int(self._status.item())

    def clear_status(self) -> None:
        self._status.zero_()
        self._pending = False


class ReducedGrid:
    """Buffers of the reduced sampled-quadrature substep (MpmReducedGrid).

    The dense (n, n, n) grids of the reference's state -- grid_m, grid_v_in,
    grid_v_out and the int32 marks neighboring_cells / neighboring_cells_grid_v
    (engine_stress/warp_utils.py:109-120) -- plus a float4 accumulation
    scratch; and, set by the caller before each call, the user-order sample
    list (int32), F_disp (n, 3, 3) and density (n) the kernels read.
    """

    def __init__(self, n_grid: int, device):
        ng = int(n_grid)
        dev = torch.device(device)
        f32 = torch.float32
        self.n_grid = ng
        self.grid_m = torch.zeros((ng, ng, ng), dtype=f32, device=dev)
        self.grid_v_in = torch.zeros((ng, ng, ng, 3), dtype=f32, device=dev)
        self.grid_v_out = torch.zeros((ng, ng, ng, 3), dtype=f32, device=dev)
        self.neighboring_cells = torch.zeros((ng, ng, ng), dtype=torch.int32, device=dev)
        self.neighboring_cells_grid_v = torch.zeros((ng, ng, ng), dtype=torch.int32, device=dev)
        self.grid_acc = torch.zeros((ng ** 3, 4), dtype=f32, device=dev)
        self.sample_index: torch.Tensor | None = None
        self.f_disp: torch.Tensor | None = None
        self.density: torch.Tensor | None = None

    def struct(self, engine: MPMEngine) -> A.MpmReducedGrid:
        n = engine.n_particles
        dev = engine.device
        checks = ((self.sample_index, torch.int32, None), (self.f_disp, torch.float32, n * 9),
                  (self.density, torch.float32, n))
        def on_dev(t):
            return t.device.type == dev.type and (dev.index is None or t.device.index == dev.index)

        for t, dt, numel in checks:
            if t is None or not on_dev(t) or t.dtype != dt or not t.is_contiguous() or \
                    (numel is not None and t.numel() != numel):
                raise ValueError("reduced substep: sample_index (int32), f_disp (n x 9) and density (n) "
                                 "must be contiguous tensors on the engine's device")
        if engine.scenes[0].n_grid != self.n_grid:
            raise ValueError("reduced substep: the grid was sized for another n_grid")
        g = A.MpmReducedGrid()
        g.sample_index = self.sample_index.data_ptr()
        g.n_samples = self.sample_index.numel()
        g.f_disp = self.f_disp.data_ptr()
        g.density = self.density.data_ptr()
        g.grid_acc = self.grid_acc.data_ptr()
        g.grid_m = self.grid_m.data_ptr()
        g.grid_v_in = self.grid_v_in.data_ptr()
        g.grid_v_out = self.grid_v_out.data_ptr()
        g.neighboring_cells = self.neighboring_cells.data_ptr()
        g.neighboring_cells_grid_v = self.neighboring_cells_grid_v.data_ptr()
        g.n_grid = self.n_grid
        return g


class SubstepGraph:
    """n substeps captured once in a CUDA graph and replayed.

    The library's host-side control (live state buffer, substep counter) moves
    as the substeps are recorded; a replay runs the recorded launches with the
    recorded buffer pointers.  Every substep flips the live state buffer, so
    n must be even, and the block keys must be valid when capturing (take one
    eager substep first).  ``time`` is frozen at capture: colliders with finite time windows
    need eager stepping.  The status word is not read inside the graph; call
    ``engine.status()`` after replays.
    """

    def __init__(self, engine: MPMEngine, n: int, time: float, dt: float):
        b = engine.buf
        if not b.keys_valid:
            raise RuntimeError("take one eager substep before capturing (block keys invalid)")
        self.engine = engine
        self.n = n
        cur0, step0 = b.cur, b.substep
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream(engine.device)
        stream.wait_stream(torch.cuda.current_stream(engine.device))
        with torch.cuda.graph(self.graph, stream=stream):
            for _ in range(n):
                engine.substep_raw(time, dt)
        if b.cur != cur0:
            b.cur = cur0
            b.substep = step0
            raise ValueError("a captured window must hold an even number of substeps")
        b.substep = step0  # nothing has run yet

    def replay(self) -> None:
        self.graph.replay()
        self.engine.buf.substep += self.n
