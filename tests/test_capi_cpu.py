"""CPU checks of the C ABI library and the host logic (no GPU, no compute).

The library must load with ctypes, export every function declared in
include/*.h, agree with the Python binding on struct sizes, and plan buffer
layouts on the host."""
import ctypes as C
import glob
import math
import os
import re

import pytest

from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300.engine import (Collider, SceneParams, dp_alpha,
                                                      lame_from_E_nu, material_code)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+[\s\*]+(mpm_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_loads_and_exports_every_declared_symbol(built):
    lib = A.load()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_binding(built):
    lib = A.load()
    out = (C.c_int64 * 6)()
    lib.mpm_struct_sizes(out)
    assert list(out) == [C.sizeof(A.MpmCollider), C.sizeof(A.MpmScene), C.sizeof(A.MpmPlan),
                         C.sizeof(A.MpmBuffers), C.sizeof(A.MpmReducedGrid), C.sizeof(A.MpmStressDecoder)]
    assert C.sizeof(A.MpmReducedGrid) == 88 and C.sizeof(A.MpmStressDecoder) == 32
    assert lib.mpm_abi_version() == 3


def _plan(scenes, n, chunk=128):
    lib = A.load()
    table = (A.MpmScene * len(scenes))()
    begin = 0
    for i, s in enumerate(scenes):
        table[i] = s.to_struct(begin)
        begin += s.n_particles
    p = A.MpmPlan()
    code = lib.mpm_plan(table, len(scenes), n, chunk, C.byref(p))
    return code, p, table


def test_plan_sizes_for_the_1m_column(built):
    sp = SceneParams(n_particles=1048576, n_grid=128, material=A.SAND)
    code, p, table = _plan([sp], 1048576)
    assert code == 0
    assert p.total_blocks == 32 ** 3
    assert p.particle_stride == 1048576
    assert p.state_bytes == 41 * 1048576 * 4
    assert table[0].n_blocks_axis == 32 and table[0].block_begin == 0
    # grid: two float4 per node; staging 9 floats per particle
    assert p.workspace_bytes > 2 * 32 ** 3 * 64 * 16 + 9 * 1048576 * 4


def test_plan_rejects_bad_arguments(built):
    sp = SceneParams(n_particles=100, n_grid=32)
    assert _plan([sp], 100, chunk=100)[0] == A.MPM_ERR_ARG
    assert _plan([sp], 99)[0] == A.MPM_ERR_ARG  # ranges must tile [0, n)
    bad = SceneParams(n_particles=100, n_grid=2)
    assert _plan([bad], 100)[0] == A.MPM_ERR_ARG


def test_plan_multi_scene_block_offsets(built):
    scenes = [SceneParams(n_particles=10, n_grid=48), SceneParams(n_particles=20, n_grid=64),
              SceneParams(n_particles=5, n_grid=97)]
    code, p, table = _plan(scenes, 35)
    assert code == 0
    assert [table[i].block_begin for i in range(3)] == [0, 12 ** 3, 12 ** 3 + 16 ** 3]
    assert table[2].n_blocks_axis == 25
    assert p.total_blocks == 12 ** 3 + 16 ** 3 + 25 ** 3


def test_error_strings(built):
    lib = A.load()
    assert lib.mpm_error_string(A.MPM_ERR_ARG) == b"invalid argument"
    with pytest.raises(A.MPMLibraryError):
        A.check(A.MPM_ERR_SIZE, "x")


def test_parameter_conversions():
    mu, lam = lame_from_E_nu(2e5, 0.3)
    assert mu == pytest.approx(76923.0769, rel=1e-9)
    assert lam == pytest.approx(115384.615, rel=1e-8)
    assert dp_alpha(30.0) == pytest.approx(math.sqrt(2 / 3) * 2 * 0.5 / 2.5, rel=1e-8)
    assert material_code("sand") == 2 and material_code("metal") == 1
    with pytest.raises(TypeError):
        material_code("water")


def test_surface_collider_normalises_and_rejects_sticky_friction():
    c = Collider.surface((0, 0.58, 0), (0, 2.0, 0))
    assert c.normal == (0.0, 1.0, 0.0) and c.surface_type == 0
    with pytest.raises(ValueError):
        Collider.surface((0, 0, 0), (0, 1, 0), "sticky", 0.5)
    assert Collider.surface((0, 0, 0), (0, 1, 0), "slip").surface_type == 1
    assert Collider.surface((0, 0, 0), (0, 1, 0), "separate", 0.3).surface_type == 2


def test_plain_c_caller(built, tmp_path):
    """The header compiles as strict C99 and a C program links the library and plans
    buffers through it, agreeing with the ctypes binding (host-only calls)."""
    import os
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(A.lib_path())
    exe = str(tmp_path / "c_abi_plan")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "c_abi_plan.c"), "-L", libdir, "-lmpm_gb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    abi = out[0].split()
    assert int(abi[1]) == 3
    assert [int(x) for x in abi[3:]] == [C.sizeof(A.MpmCollider), C.sizeof(A.MpmScene), C.sizeof(A.MpmPlan),
                                         C.sizeof(A.MpmBuffers), C.sizeof(A.MpmReducedGrid),
                                         C.sizeof(A.MpmStressDecoder)]
    from reduced_mpm_stress_training_gb300.engine import SceneParams

    lib = A.load()
    table = (A.MpmScene * 1)()
    table[0] = SceneParams(n_particles=1024, n_grid=32, grid_lim=1.0, material=A.SAND, mu=1.0, lam=1.0,
                           friction_angle=30.0, gravity=(0.0, 0.0, 0.0)).to_struct(0)
    plan = A.MpmPlan()
    assert lib.mpm_plan(table, 1, 1024, 0, C.byref(plan)) == 0
    got = [int(x) for x in out[1].split()[1:]]
    assert got == [plan.state_bytes, plan.workspace_bytes, plan.total_blocks, plan.particle_stride, plan.chunk_size]
    assert out[2].split() == ["bad", str(A.MPM_ERR_ARG)]


def test_c_example_compiles_and_links(built, tmp_path):
    """A complete C caller of the substep (tests/c_abi_substep.c) compiles as C99
    against the header and the CUDA runtime and links the library."""
    import os
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if cc is None or not os.path.exists(os.path.join(cuda, "include", "cuda_runtime.h")):
        pytest.skip("no C compiler or CUDA runtime headers")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(A.lib_path())
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(root, "include"),
                    "-I", os.path.join(cuda, "include"), os.path.join(root, "tests", "c_abi_substep.c"),
                    "-L", libdir, "-lmpm_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart", "-lm",
                    "-Wl,-rpath," + libdir, "-o", str(tmp_path / "c_abi_substep")], check=True)
