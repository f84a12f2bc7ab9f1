"""ctypes binding of libmpm_gb300.so (include/mpm_gb300.h).

The structs below mirror the header field for field; ``check_abi`` compares
their sizes with the library's own ``mpm_struct_sizes``.  Loading fails
loudly when the library has not been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

MPM_ABI_VERSION = 3
MPM_MAX_COLLIDERS = 8
MPM_OK, MPM_ERR_ARG, MPM_ERR_CUDA, MPM_ERR_SIZE = 0, -1, -2, -3
ST_OUT_OF_DOMAIN, ST_CFL, ST_NONFINITE, ST_INTERNAL, ST_BAD_INPUT = 1, 2, 4, 8, 16
JELLY, METAL, SAND = 0, 1, 2
(COLLIDER_SURFACE, COLLIDER_BOX, COLLIDER_VPLANE, COLLIDER_CIRCLE, COLLIDER_DISK, COLLIDER_CUBE,
 COLLIDER_SPHERE) = range(7)
MOVING_COLLIDERS = (COLLIDER_VPLANE, COLLIDER_CIRCLE, COLLIDER_CUBE, COLLIDER_SPHERE)
CF_EXTENDED, CF_MOVING = 1, 2
MLP_IN, MLP_OUT, MLP_HIDDEN, MLP_PARAMS = 12, 6, 128, 37264

(FIELD_X_INITIAL, FIELD_U, FIELD_V, FIELD_C, FIELD_F, FIELD_STRESS, FIELD_MASS, FIELD_VOL,
 FIELD_YIELD, FIELD_X, FIELD_F_DISP) = range(11)
FIELD_COMPONENTS = {FIELD_X_INITIAL: 3, FIELD_U: 3, FIELD_V: 3, FIELD_C: 9, FIELD_F: 9,
                    FIELD_STRESS: 9, FIELD_MASS: 1, FIELD_VOL: 1, FIELD_YIELD: 1, FIELD_X: 3,
                    FIELD_F_DISP: 9}

STATUS_NAMES = {ST_OUT_OF_DOMAIN: "particle stencil outside the grid (particle frozen)",
                ST_CFL: "CFL violated: |v| > dx/dt",
                ST_NONFINITE: "non-finite F or stress",
                ST_INTERNAL: "particle outside its sorted block",
                ST_BAD_INPUT: "reduced substep: sample index outside [0, n) or grid size mismatch"}


class MpmCollider(C.Structure):
    _fields_ = [("kind", C.c_int32), ("surface_type", C.c_int32), ("point", C.c_float * 3),
                ("normal", C.c_float * 3), ("friction", C.c_float), ("start_time", C.c_float),
                ("end_time", C.c_float), ("reset", C.c_int32), ("velocity", C.c_float * 3),
                ("threshold", C.c_float), ("radius", C.c_float), ("width", C.c_float),
                ("height", C.c_float), ("v_scale", C.c_float), ("x_unit", C.c_float * 3),
                ("y_unit", C.c_float * 3), ("R", C.c_float), ("pad0", C.c_float)]


class MpmScene(C.Structure):
    _fields_ = [("n_grid", C.c_int32), ("material", C.c_int32), ("hardening", C.c_int32),
                ("n_colliders", C.c_int32), ("dx", C.c_float), ("inv_dx", C.c_float),
                ("mu", C.c_float), ("lam", C.c_float), ("alpha", C.c_float), ("xi", C.c_float),
                ("gravity", C.c_float * 3), ("n_blocks_axis", C.c_int32),
                ("particle_begin", C.c_int64), ("particle_count", C.c_int64),
                ("block_begin", C.c_int64), ("colliders", MpmCollider * MPM_MAX_COLLIDERS)]


class MpmPlan(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("particle_stride", C.c_int64),
                ("total_blocks", C.c_int64), ("max_chunks", C.c_int64),
                ("state_bytes", C.c_int64), ("workspace_bytes", C.c_int64),
                ("chunk_size", C.c_int32), ("n_scenes", C.c_int32)]


class MpmBuffers(C.Structure):
    _fields_ = [("state", C.c_void_p * 2), ("workspace", C.c_void_p), ("scenes", C.c_void_p),
                ("status", C.c_void_p), ("plan", MpmPlan), ("cur", C.c_int32),
                ("keys_valid", C.c_int32), ("collider_flags", C.c_int32), ("pad0", C.c_int32),
                ("substep", C.c_int64)]


class MpmReducedGrid(C.Structure):
    _fields_ = [("sample_index", C.c_void_p), ("n_samples", C.c_int64), ("f_disp", C.c_void_p),
                ("density", C.c_void_p), ("grid_acc", C.c_void_p), ("grid_m", C.c_void_p),
                ("grid_v_in", C.c_void_p), ("grid_v_out", C.c_void_p), ("neighboring_cells", C.c_void_p),
                ("neighboring_cells_grid_v", C.c_void_p), ("n_grid", C.c_int32), ("pad0", C.c_int32)]


class MpmStressDecoder(C.Structure):
    _fields_ = [("params", C.c_void_p), ("label_dim", C.c_int32), ("mu_dim", C.c_int32),
                ("hidden", C.c_int32), ("siren", C.c_int32), ("omega_0", C.c_float), ("pad0", C.c_int32)]


class MpmSurrogateConfig(C.Structure):
    _fields_ = [("tol", C.c_float), ("rho_min", C.c_float), ("rho_max", C.c_float),
                ("nu_min", C.c_float), ("nu_max", C.c_float), ("phi_min", C.c_float),
                ("phi_max", C.c_float), ("dgamma_max", C.c_float)]


(SUR_ELASTIC, SUR_PLASTIC, SUR_FB_DOMAIN, SUR_FB_APEX, SUR_FB_STEP, SUR_FB_GATE,
 SUR_FB_MATERIAL, SUR_LAST_FALLBACKS) = range(8)
SUR_STATS = 8
ADJ_WORDS = 36
ADJ_X, ADJ_V, ADJ_C, ADJ_F, ADJ_STRESS = 0, 3, 6, 15, 24


class MPMLibraryError(RuntimeError):
    """A libmpm_gb300 call returned an error code."""


_lib: C.CDLL | None = None

_SIGS = {
    "mpm_plan": ([C.POINTER(MpmScene), C.c_int32, C.c_int64, C.c_int32, C.POINTER(MpmPlan)], C.c_int),
    "mpm_init": ([C.POINTER(MpmBuffers), C.c_void_p], C.c_int),
    "mpm_upload_scenes": ([C.POINTER(MpmBuffers), C.POINTER(MpmScene), C.c_int32, C.c_void_p], C.c_int),
    "mpm_load": ([C.POINTER(MpmBuffers), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "mpm_export": ([C.POINTER(MpmBuffers), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "mpm_load_uvstress": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p],
                          C.c_int),
    "mpm_export_uvFstress": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                              C.c_void_p], C.c_int),
    "mpm_sync_transfers": ([], C.c_int),
    "mpm_export_frame": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p], C.c_int),
    "mpm_p2g2p": ([C.POINTER(MpmBuffers), C.c_float, C.c_float, C.c_void_p], C.c_int),
    "mpm_sort": ([C.POINTER(MpmBuffers), C.c_void_p], C.c_int),
    "mpm_p2g_ordered_bytes": ([C.POINTER(MpmPlan)], C.c_int64),
    "mpm_p2g_ordered": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "mpm_p2g2p_ordered": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "mpm_p2g": ([C.POINTER(MpmBuffers), C.c_float, C.c_void_p], C.c_int),
    "mpm_grid_update": ([C.POINTER(MpmBuffers), C.c_float, C.c_float, C.c_void_p], C.c_int),
    "mpm_g2p": ([C.POINTER(MpmBuffers), C.c_float, C.c_void_p], C.c_int),
    "mpm_export_grid": ([C.POINTER(MpmBuffers), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p], C.c_int),
    "mpm_p2g2p_reduced": ([C.POINTER(MpmBuffers), C.POINTER(MpmReducedGrid), C.c_float, C.c_float, C.c_void_p],
                          C.c_int),
    "mpm_mark_neighboring_cells_grid_v": ([C.POINTER(MpmBuffers), C.POINTER(MpmReducedGrid), C.c_void_p], C.c_int),
    "mpm_g2p_sample": ([C.POINTER(MpmBuffers), C.POINTER(MpmReducedGrid), C.c_float, C.c_void_p], C.c_int),
    "mpm_decoder_param_count": ([C.POINTER(MpmStressDecoder)], C.c_int64),
    "mpm_decoder_forward": ([C.POINTER(MpmStressDecoder), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "mpm_decoder_stress": ([C.POINTER(MpmBuffers), C.POINTER(MpmStressDecoder), C.c_void_p, C.c_void_p, C.c_void_p],
                           C.c_int),
    "mpm_svd3": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "mpm_return_map": ([C.POINTER(MpmScene), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                        C.c_int64, C.c_void_p], C.c_int),
    "mpm_mlp_param_bytes": ([], C.c_int64),
    "mpm_mlp_forward": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_float, C.c_int64, C.c_void_p], C.c_int),
    "mpm_mlp_forward_tc": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_void_p, C.c_float, C.c_int64, C.c_void_p, C.c_void_p], C.c_int),
    "mpm_mlp_backward": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                          C.c_int64, C.c_void_p], C.c_int),
    "mpm_mlp_backward_tc": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                             C.c_void_p, C.c_void_p], C.c_int),
    "mpm_mlp_adam": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                      C.c_float, C.c_float, C.c_float, C.c_int32, C.c_void_p], C.c_int),
    "mpm_surrogate_features": ([C.POINTER(MpmScene), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_int64, C.c_void_p], C.c_int),
    "mpm_surrogate_apply": ([C.POINTER(MpmScene), C.c_void_p, C.POINTER(MpmSurrogateConfig), C.c_void_p,
                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "mpm_g2p_surrogate": ([C.POINTER(MpmBuffers), C.c_void_p, C.POINTER(MpmSurrogateConfig),
                           C.c_void_p, C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "mpm_p2g2p_surrogate": ([C.POINTER(MpmBuffers), C.c_void_p, C.POINTER(MpmSurrogateConfig),
                             C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "mpm_adjoint_substep": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_float, C.c_float, C.c_void_p], C.c_int),
    "mpm_substep_grid_bytes": ([C.POINTER(MpmPlan)], C.c_int64),
    "mpm_save_substep_grid": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p], C.c_int),
    "mpm_load_substep_grid": ([C.POINTER(MpmBuffers), C.c_void_p, C.c_void_p], C.c_int),
    "mpm_clear_grid": ([C.POINTER(MpmBuffers), C.c_void_p], C.c_int),
    "mpm_return_map_vjp": ([C.POINTER(MpmScene), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "mpm_abi_version": ([], C.c_int),
    "mpm_struct_sizes": ([C.POINTER(C.c_int64)], None),
    "mpm_error_string": ([C.c_int], C.c_char_p),
    "mpm_last_cuda_error": ([], C.c_char_p),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libmpm_gb300.so; raises if it is absent (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"libmpm_gb300.so is not built ({path}); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`")
        _build.build()
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    check_abi(lib)
    return lib


def check_abi(lib: C.CDLL) -> None:
    if lib.mpm_abi_version() != MPM_ABI_VERSION:
        raise ImportError(f"libmpm_gb300 ABI version {lib.mpm_abi_version()}, binding {MPM_ABI_VERSION}: rebuild")
    out = (C.c_int64 * 6)()
    lib.mpm_struct_sizes(out)
    mine = [C.sizeof(MpmCollider), C.sizeof(MpmScene), C.sizeof(MpmPlan), C.sizeof(MpmBuffers),
            C.sizeof(MpmReducedGrid), C.sizeof(MpmStressDecoder)]
    if list(out) != mine:
        raise ImportError(f"libmpm_gb300 ABI mismatch: library {list(out)} vs binding {mine}")


def check(code: int, what: str) -> None:
    if code != MPM_OK:
        lib = load()
        msg = lib.mpm_error_string(code).decode()
        if code == MPM_ERR_CUDA:
            msg += ": " + lib.mpm_last_cuda_error().decode()
        raise MPMLibraryError(f"{what} failed ({code}): {msg}")


def status_text(bits: int) -> str:
    return "; ".join(t for b, t in STATUS_NAMES.items() if bits & b) or "ok"
