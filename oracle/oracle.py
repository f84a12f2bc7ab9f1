"""ctypes front end of the CPU oracle (test infrastructure, not product).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use
this module; it is the checker, never the thing measured for the GPU path.

``OracleSim`` holds the reference's own arrays (engine_stress/mpm_solver_warp.py:52-69:
AoS vec3 / row-major mat33 per particle, dense (n,n,n) grid) as NumPy arrays
in float32 or float64 and advances them with the C restatement in
``mpm_oracle.c``.  Pinned to the reference's own outputs: the reference
ships no golden vectors and Warp is not installed, so its unmodified solver
was run on the CPU through a test-only Warp stand-in (``tests/refshim``)
and the oracle is checked against those runs (``tests/golden/ref_*.npz``,
``tests/test_ref_fixtures_cpu.py``).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import build as _build

ST_OUT_OF_DOMAIN = 1
ST_CFL = 2
ST_NONFINITE = 4
ST_BAD_INPUT = 16


class OrcModel(C.Structure):
    _fields_ = [
        ("n_grid", C.c_int32),
        ("material", C.c_int32),
        ("hardening", C.c_int32),
        ("pad0", C.c_int32),
        ("dx", C.c_double),
        ("inv_dx", C.c_double),
        ("mu", C.c_double),
        ("lam", C.c_double),
        ("alpha", C.c_double),
        ("xi", C.c_double),
        ("gravity", C.c_double * 3),
    ]


class OrcCollider(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("surface_type", C.c_int32),
        ("point", C.c_double * 3),
        ("normal", C.c_double * 3),
        ("friction", C.c_double),
        ("start_time", C.c_double),
        ("end_time", C.c_double),
        ("reset", C.c_int32),
        ("pad", C.c_int32),
        ("velocity", C.c_double * 3),
        ("threshold", C.c_double),
        ("radius", C.c_double),
        ("width", C.c_double),
        ("height", C.c_double),
        ("v_scale", C.c_double),
        ("x_unit", C.c_double * 3),
        ("y_unit", C.c_double * 3),
        ("R", C.c_double),
    ]


_STATE_FIELDS = ["x0", "x", "u", "v", "C", "F", "F_trial", "F_disp", "stress", "mass", "vol",
                 "yield_", "grid_m", "grid_v_in", "grid_v_out"]

_libs: dict[int, C.CDLL] = {}


def lib(bits: int) -> C.CDLL:
    if bits not in _libs:
        _build.build()
        _libs[bits] = C.CDLL(_build.lib_path(bits))
    return _libs[bits]


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.c_void_p)


def max_threads() -> int:
    f = lib(32).orc32_max_threads
    f.restype = C.c_int
    return int(f())


def material_code(material: str) -> int:
    """engine_stress/mpm_solver_warp.py:90-94"""
    codes = {"jelly": 0, "metal": 1, "sand": 2}
    if material not in codes:
        raise TypeError("Undefined material type")
    return codes[material]


def make_model(n_grid: int, grid_lim: float = 1.0, material: str = "sand", E: float | None = None,
               nu: float | None = None, mu: float | None = None, lam: float | None = None,
               friction_angle: float = 25.0, gravity=(0.0, 0.0, 0.0), hardening: int = 0,
               xi: float = 0.0) -> OrcModel:
    """Parameter conversions of engine_stress/mpm_solver_warp.py:37-48, :101, :113-116."""
    m = OrcModel()
    m.n_grid = n_grid
    m.material = material_code(material)
    m.hardening = hardening
    m.dx = grid_lim / n_grid
    m.inv_dx = float(n_grid / grid_lim)
    if E is not None:
        nu = 0.3 if nu is None else nu
        mu = E / 2.0 / (1.0 + nu)
        lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)
    m.mu = mu
    m.lam = lam
    sin_phi = math.sin(friction_angle / 180.0 * 3.14159265)
    m.alpha = math.sqrt(2.0 / 3.0) * 2.0 * sin_phi / (3.0 - sin_phi)
    m.xi = xi
    for c in range(3):
        m.gravity[c] = gravity[c]
    return m


def surface_collider(point, normal, surface="sticky", friction=0.0, start_time=0.0,
                     end_time=999.0) -> OrcCollider:
    """engine_stress/mpm_solver_warp.py:407-428"""
    col = OrcCollider()
    col.kind = 0
    scale = 1.0 / math.sqrt(sum(x * x for x in normal))
    for c in range(3):
        col.point[c] = point[c]
        col.normal[c] = scale * normal[c]
    if surface == "sticky" and friction != 0:
        raise ValueError("friction must be 0 on sticky surfaces.")
    col.surface_type = 0 if surface == "sticky" else (1 if surface == "slip" else 2)
    col.friction = friction
    col.start_time = start_time
    col.end_time = end_time
    return col


def bounding_box(start_time=0.0, end_time=999.0) -> OrcCollider:
    """engine_stress/mpm_solver_warp.py:499-503"""
    col = OrcCollider()
    col.kind = 1
    col.start_time = start_time
    col.end_time = end_time
    return col


def _f32(x) -> float:
    """the value a wp.vec3 / float field of Dirichlet_collider holds"""
    return float(np.float32(x))


def _moving(kind, point, start_time, end_time, **kw) -> OrcCollider:
    col = OrcCollider()
    col.kind = kind
    for c in range(3):
        col.point[c] = _f32(point[c])
    col.start_time = _f32(start_time)
    col.end_time = _f32(end_time)
    for k, v in kw.items():
        if isinstance(v, (tuple, list)):
            for c in range(3):
                getattr(col, k)[c] = _f32(v[c])
        else:
            setattr(col, k, v if k == "reset" else _f32(v))
    return col


def _unit(v):
    scale = 1.0 / math.sqrt(sum(x * x for x in v))
    return [scale * x for x in v]


def velocity_plane(point, normal, velocity, threshold, start_time=0.0, end_time=999.0, reset=0):
    """engine_stress/mpm_solver_warp.py:527-543"""
    return _moving(2, point, start_time, end_time, normal=_unit(normal), velocity=velocity,
                   threshold=threshold, reset=int(reset))


def circle_column(R, radius, height, v_scale, start_time=0.0, end_time=999.0):
    """engine_stress/mpm_solver_warp.py:570-579"""
    return _moving(3, (0.5, 0.069, 0.5 + R), start_time, end_time, radius=radius, height=height,
                   v_scale=v_scale, R=R)


def rotating_disk(point, normal, radius, width, v_scale, start_time=0.0, end_time=999.0, reset=0):
    """engine_stress/mpm_solver_warp.py:609-633 (the axis search of :615-618
    only ever tests normal[0]; other normals do not terminate there)"""
    n = _unit(normal)
    if not abs(n[0]) > 1e-1:
        raise ValueError("normal[0] must exceed 0.1 in magnitude")
    x = [1.0, 1.0, 1.0]
    x[0] = -(n[0] + n[1] + n[2] - n[0]) / n[0]
    y = list(np.cross(np.array(n), np.array(x)))
    return _moving(4, point, start_time, end_time, normal=n, x_unit=_unit(x), y_unit=_unit(y),
                   radius=radius, width=width, v_scale=v_scale, reset=int(reset))


def velocity_cube(point, width, velocity, start_time=0.0, end_time=999.0, reset=0):
    """engine_stress/mpm_solver_warp.py:667-679"""
    return _moving(5, point, start_time, end_time, width=width, velocity=velocity, reset=int(reset))


def sphere_leader(center, radius, velocity, start_time=0.0, end_time=999.0):
    """engine_stress/mpm_solver_warp.py:697-707"""
    return _moving(6, center, start_time, end_time, radius=radius, velocity=velocity)


def advance_collider(col: OrcCollider, time: float, dt: float) -> None:
    """The reference's modify_bc callbacks (mpm_solver_warp.py:561-565,
    :594-603, :690-693, :716-718), run on the host after each substep's
    collider kernels: time and dt in double, the point stored back in float."""
    if col.kind not in (2, 3, 5, 6) or not (time >= col.start_time and time < col.end_time):
        return
    if col.kind == 3:
        f = np.float32
        z0, z1, z2 = f(col.point[0]) - f(0.5), f(col.point[1]), f(col.point[2]) - f(0.5)
        c = z0 / np.sqrt(z0 * z0 + z1 * z1 + z2 * z2)
        th = np.arccos(np.clip(c, f(-1), f(1)))
        if z2 < 0:
            th = -th
        vel = (f(-col.v_scale) * np.sin(th), f(0.0), f(col.v_scale) * np.cos(th))
    else:
        vel = tuple(col.velocity)
    for c in range(3):
        col.point[c] = _f32(col.point[c] + dt * float(vel[c]))


class OracleSim:
    """Reference-layout simulator state advanced by the C oracle."""

    def __init__(self, model: OrcModel, x0: np.ndarray, mass: np.ndarray, vol: np.ndarray,
                 v: np.ndarray | None = None, bits: int = 32, colliders=(), yield_stress=None):
        self.bits = bits
        self.dtype = np.float32 if bits == 32 else np.float64
        self.model = model
        self.colliders = list(colliders)
        n = x0.shape[0]
        self.n = n
        dt = self.dtype
        ng = model.n_grid
        self.x0 = np.ascontiguousarray(x0, dtype=dt).reshape(n, 3)
        self.x = self.x0.copy()
        self.u = np.zeros((n, 3), dt)
        self.v = np.zeros((n, 3), dt) if v is None else np.ascontiguousarray(v, dtype=dt).reshape(n, 3).copy()
        self.C = np.zeros((n, 9), dt)
        self.F = np.tile(np.eye(3, dtype=dt).reshape(1, 9), (n, 1))
        self.F_trial = np.zeros((n, 9), dt)
        self.F_disp = np.zeros((n, 9), dt)
        self.stress = np.zeros((n, 9), dt)
        self.mass = np.ascontiguousarray(mass, dtype=dt).reshape(n).copy()
        self.vol = np.ascontiguousarray(vol, dtype=dt).reshape(n).copy()
        ys = 0.0 if yield_stress is None else yield_stress
        self.yield_ = np.broadcast_to(np.asarray(ys, dtype=dt), (n,)).copy()
        self.grid_m = np.zeros((ng, ng, ng), dt)
        self.grid_v_in = np.zeros((ng, ng, ng, 3), dt)
        self.grid_v_out = np.zeros((ng, ng, ng, 3), dt)
        self.time = 0.0
        self.status = C.c_int32(0)
        # reduced sampled-quadrature state (warp_utils.py:106, :117-120; mpm_solver_warp.py:62, :81-83)
        self.density = np.zeros(n, dt)
        self.neighboring_cells = np.zeros((ng, ng, ng), np.int32)
        self.neighboring_cells_grid_v = np.zeros((ng, ng, ng), np.int32)
        self.sample_particle_index_short = np.zeros(1, np.int32)

    def _fn(self, name):
        return getattr(lib(self.bits), f"orc{self.bits}_{name}")

    def _state(self):
        bits = self.bits

        class State(C.Structure):
            _fields_ = [(f, C.c_void_p) for f in _STATE_FIELDS]

        s = State()
        for f in _STATE_FIELDS:
            setattr(s, f, _ptr(getattr(self, f)).value)
        return s

    def _real(self, x):
        return C.c_float(x) if self.bits == 32 else C.c_double(x)

    def p2g2p(self, dt: float, nthreads_p2g: int = 1) -> None:
        """One substep, engine_stress/mpm_solver_warp.py:156-199 (time += dt)."""
        s = self._state()
        ncol = len(self.colliders)
        arr = (OrcCollider * max(ncol, 1))(*self.colliders)
        self._fn("p2g2p")(C.byref(self.model), C.byref(s), C.c_int64(self.n), arr, C.c_int(ncol),
                          C.c_double(self.time), self._real(dt), C.c_int(nthreads_p2g),
                          C.byref(self.status))
        for col in self.colliders:
            advance_collider(col, self.time, dt)
        self.time = self.time + dt

    # ---- individual kernels (same order as p2g2p) for per-stage checks ----
    def stage_p2g(self, dt: float) -> None:
        nn = self.model.n_grid ** 3
        self._fn("update_x_from_u")(C.c_int64(self.n), _ptr(self.x0), _ptr(self.u), _ptr(self.x))
        self._fn("zero_grid")(C.c_int64(nn), _ptr(self.grid_m), _ptr(self.grid_v_in),
                              _ptr(self.grid_v_out))
        self._fn("p2g_apic_stress_given")(C.byref(self.model), C.c_int64(self.n), _ptr(self.x),
                                          _ptr(self.v), _ptr(self.C), _ptr(self.stress),
                                          _ptr(self.mass), _ptr(self.vol), self._real(dt),
                                          _ptr(self.grid_m), _ptr(self.grid_v_in),
                                          C.byref(self.status), C.c_int(1))

    def stage_grid(self, dt: float) -> None:
        self._fn("grid_normalization_and_gravity")(C.byref(self.model), self._real(dt),
                                                   _ptr(self.grid_m), _ptr(self.grid_v_in),
                                                   _ptr(self.grid_v_out))
        for col in self.colliders:
            if col.kind >= 2:
                self._fn("collide_extended")(C.byref(self.model), C.byref(col), C.c_double(self.time),
                                             self._real(dt), _ptr(self.grid_v_out))
                continue
            name = "collide_surface" if col.kind == 0 else "collide_bounding_box"
            self._fn(name)(C.byref(self.model), C.byref(col), C.c_double(self.time),
                           _ptr(self.grid_v_out))
        for col in self.colliders:
            advance_collider(col, self.time, dt)

    def stage_g2p(self, dt: float) -> None:
        self._fn("g2p_apic_and_stress")(C.byref(self.model), C.c_int64(self.n), self._real(dt),
                                        _ptr(self.grid_v_out), _ptr(self.x), _ptr(self.v),
                                        _ptr(self.C), _ptr(self.F_trial), _ptr(self.F),
                                        _ptr(self.stress), _ptr(self.yield_),
                                        C.byref(self.status))
        self._fn("update_u_from_x")(C.c_int64(self.n), _ptr(self.x), _ptr(self.x0), _ptr(self.u))
        self._fn("update_F_disp_from_F")(C.c_int64(self.n), _ptr(self.F), _ptr(self.F_disp))
        self.time = self.time + dt


    # ---- reduced sampled-quadrature substep (mpm_solver_warp.py:207-227) ----
    def _samples(self):
        idx = np.ascontiguousarray(self.sample_particle_index_short, dtype=np.int32).reshape(-1)
        return idx, C.c_int64(idx.shape[0])

    def p2g2p_reduced(self, dt: float, nthreads_p2g: int = 1) -> None:
        """p2g2p_reduced (mpm_solver_warp.py:214-227): the grid of the sampled
        particles' neighbourhood; particles are not moved (time += dt)."""
        s = self._state()
        ncol = len(self.colliders)
        arr = (OrcCollider * max(ncol, 1))(*self.colliders)
        idx, ns = self._samples()
        self.density = np.ascontiguousarray(self.density, dtype=self.dtype)
        self._fn("p2g2p_reduced")(C.byref(self.model), C.byref(s), C.c_int64(self.n), _ptr(self.density), ns,
                                  _ptr(idx), _ptr(self.neighboring_cells), _ptr(self.neighboring_cells_grid_v),
                                  arr, C.c_int(ncol), C.c_double(self.time), self._real(dt),
                                  C.c_int(nthreads_p2g), C.byref(self.status))
        for col in self.colliders:
            advance_collider(col, self.time, dt)
        self.time = self.time + dt

    def experiment_for_C(self) -> np.ndarray:
        """experiment_for_C (mpm_solver_warp.py:207-209): add the -2..4 marks."""
        idx, ns = self._samples()
        self._fn("update_neighboring_cells")(C.byref(self.model), ns, _ptr(idx), C.c_int64(self.n), _ptr(self.x),
                                             C.c_int(4), _ptr(self.neighboring_cells_grid_v), C.byref(self.status))
        return self.neighboring_cells_grid_v

    def g2p_sample(self, dt: float) -> None:
        """g2p_sample (mpm_utils.py:415-471) over the sample list."""
        idx, ns = self._samples()
        self._fn("g2p_sample")(C.byref(self.model), ns, _ptr(idx), C.c_int64(self.n), self._real(dt),
                               _ptr(self.grid_v_out), _ptr(self.x), _ptr(self.x0), _ptr(self.v), _ptr(self.u),
                               _ptr(self.F), _ptr(self.F_disp), _ptr(self.yield_), C.byref(self.status))


def svd3(A: np.ndarray, bits: int = 32):
    """Batch 3x3 SVD with the oracle's convention. A: (n, 9) or (n,3,3)."""
    dt = np.float32 if bits == 32 else np.float64
    A = np.ascontiguousarray(A, dtype=dt).reshape(-1, 9)
    n = A.shape[0]
    U = np.zeros((n, 9), dt)
    s = np.zeros((n, 3), dt)
    V = np.zeros((n, 9), dt)
    getattr(lib(bits), f"orc{bits}_svd3_batch")(C.c_int64(n), _ptr(A), _ptr(U), _ptr(s), _ptr(V))
    return U.reshape(n, 3, 3), s, V.reshape(n, 3, 3)


def return_map(model: OrcModel, F_trial: np.ndarray, yield_stress=None, bits: int = 32):
    """Return map + Kirchhoff stress as g2p_apic_and_stress does (mpm_utils.py:284-306)."""
    dt = np.float32 if bits == 32 else np.float64
    Ft = np.ascontiguousarray(F_trial, dtype=dt).reshape(-1, 9)
    n = Ft.shape[0]
    Fo = np.zeros((n, 9), dt)
    tau = np.zeros((n, 9), dt)
    y = None
    if yield_stress is not None:
        y = np.broadcast_to(np.asarray(yield_stress, dt), (n,)).copy()
    getattr(lib(bits), f"orc{bits}_return_map_batch")(C.byref(model), C.c_int64(n), _ptr(Ft),
                                                      _ptr(y), _ptr(Fo), _ptr(tau))
    return Fo, tau, y
