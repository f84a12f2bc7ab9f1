"""mpm_p2g2p_noalloc: the substep for callers that cannot allocate device memory
(a host framework that keeps all device memory in its own pool, or code that
runs where cudaMalloc is not allowed).  Its scratch lives in a library-owned
16 MiB device array instead of the caller's workspace.

The test drives it through the C ABI and checks it against the regular
mpm_p2g2p on the same inputs, for two calls in a row: x, v, F within 1e-5
relative (the per-substep tolerance of the parity tests), C and stress within
the float32 noise floor used there.  It also checks that an oversized plan is
rejected with MPM_ERR_SIZE, that a plan whose host-transfer staging (which
this call never uses) takes the workspace over 16 MiB is still accepted, and
that calls from two simulators of different sizes may alternate.  Kept in
its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S

from helpers import gpu_sim, gpu_state, oracle_sim, rel, within_fp32_floor

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5


def _bind(lib):
    fn = lib.mpm_p2g2p_noalloc
    fn.argtypes = [C.POINTER(A.MpmBuffers), C.c_float, C.c_float, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _perturbed(sc, seed=11):
    rng = np.random.default_rng(seed)
    x0, v0, vol, mass = sc.particles()
    n = sc.n_particles
    v0 = (0.1 * rng.normal(size=(n, 3))).astype(np.float32)
    Cm = (0.5 * rng.normal(size=(n, 9))).astype(np.float32)
    tau = (1e3 * rng.normal(size=(n, 9))).astype(np.float32)
    sim = gpu_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    sim.load_C_from_tensor(torch.from_numpy(Cm))
    sim.load_uvstress_from_tensor(torch.zeros(n, 3), torch.from_numpy(v0), torch.from_numpy(tau))
    return sim, (x0, v0, vol, mass, Cm, tau)


def test_noalloc_substep_matches_regular_substep(cuda):
    lib = A.load()
    noalloc = _bind(lib)
    sc = S.small_column(8192, 32)
    regular, data = _perturbed(sc)
    other, _ = _perturbed(sc)
    x0, v0, vol, mass, Cm, tau = data
    o32 = oracle_sim(sc, x0=x0, v0=v0, vol=vol, mass=mass)
    o64 = oracle_sim(sc, bits=64, x0=x0, v0=v0, vol=vol, mass=mass)
    for o in (o32, o64):
        o.C[:] = Cm
        o.stress[:] = tau
    eng = other._engine
    for call in range(2):
        regular.p2g2p(call, sc.dt)
        # the no-alloc path ignores the caller's workspace: hand it none
        saved = eng.buf.workspace
        eng.buf.workspace = None
        stream = torch.cuda.current_stream().cuda_stream
        code = noalloc(C.byref(eng.buf), float(other.time), sc.dt, stream)
        eng.buf.workspace = saved
        assert code == A.MPM_OK, lib.mpm_error_string(code)
        other.time += sc.dt
        o32.p2g2p(sc.dt)
        o64.p2g2p(sc.dt)
        torch.cuda.synchronize()
        a, b = gpu_state(regular), gpu_state(other)
        for f in ("x", "v", "F"):
            assert rel(b[f], a[f]) < TOL_STEP, (call, f, rel(b[f], a[f]))
        for f in ("C", "stress"):
            ok, info = within_fp32_floor(b[f], getattr(o32, f), getattr(o64, f))
            assert ok, (call, f, info)
    assert int(other._engine.status()) == 0


def _noalloc_step(noalloc, sim, dt):
    eng = sim._engine
    saved = eng.buf.workspace
    eng.buf.workspace = None
    code = noalloc(C.byref(eng.buf), float(sim.time), dt, torch.cuda.current_stream().cuda_stream)
    eng.buf.workspace = saved
    sim.time += dt
    return code


def test_noalloc_accepts_plans_whose_staging_exceeds_the_array(cuda):
    """A 64^3 grid with 131,072 particles: the whole workspace (with the
    host-transfer staging) is over 16 MiB, the substep's part is not, so the
    call runs and matches the regular substep."""
    lib = A.load()
    noalloc = _bind(lib)
    sc = S.small_column(131072, 64)
    regular = gpu_sim(sc)
    other = gpu_sim(sc)
    assert other._engine.plan.workspace_bytes > 16 << 20
    for call in range(2):
        regular.p2g2p(call, sc.dt)
        code = _noalloc_step(noalloc, other, sc.dt)
        assert code == A.MPM_OK, lib.mpm_error_string(code)
        torch.cuda.synchronize()
        a, b = gpu_state(regular), gpu_state(other)
        for f in ("x", "v", "F"):
            assert rel(b[f], a[f]) < TOL_STEP, (call, f, rel(b[f], a[f]))
    assert int(other._engine.status()) == 0


def test_noalloc_calls_alternating_between_simulators(cuda):
    """Calls from two simulators of different sizes (32^3 / 8,192 and 48^3 /
    20,000 particles) alternate on the shared array; each must match its own
    regular run, so nothing the larger plan left in the array leaks into the
    smaller one."""
    lib = A.load()
    noalloc = _bind(lib)
    scenes = [S.small_column(20000, 48, seed=3), S.small_column(8192, 32, seed=4)]
    pairs = [(gpu_sim(sc), gpu_sim(sc)) for sc in scenes]
    for call in range(3):
        for sc, (regular, other) in zip(scenes, pairs):
            regular.p2g2p(call, sc.dt)
            code = _noalloc_step(noalloc, other, sc.dt)
            assert code == A.MPM_OK, lib.mpm_error_string(code)
    torch.cuda.synchronize()
    for regular, other in pairs:
        a, b = gpu_state(regular), gpu_state(other)
        for f in ("x", "v", "F"):
            assert rel(b[f], a[f]) < TOL_STEP, (f, rel(b[f], a[f]))
        assert int(other._engine.status()) == 0


def test_noalloc_rejects_oversized_plans(cuda):
    lib = A.load()
    noalloc = _bind(lib)
    big = S.sand_column_1m()
    sim = S.build_simulator(big)
    code = noalloc(C.byref(sim._engine.buf), 0.0, big.dt, torch.cuda.current_stream().cuda_stream)
    assert code == A.MPM_ERR_SIZE
    assert sim._engine.plan.workspace_bytes > 16 << 20
