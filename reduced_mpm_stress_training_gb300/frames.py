"""Frame files of the reference's training-data loop.

The reference writes one file per frame from its simulator state
(save_data_at_frame, engine_stress/mpm_solver_warp.py:339-404) and reads
initial samplings and frames back (load_from_sampling :129-153,
load_uvFstress_from_h5 :268-303).  A frame holds, all transposed to
(components, n):

  x (3, n) x_initial   q (3, n) u   time (1, 1)   masses (1, n)
  f_tensor (9, n) F_disp row-major   stress (6, n) components 0,1,2,4,5,8
  v (3, n)   mu (1, n) the friction angle   C (9, n) row-major

The device side assembles the float32 arrays in this layout in one pass
(``mpm_export_frame``); this module names, writes and reads the files.  HDF5
needs ``h5py``; where it is not importable the same datasets go to a NumPy
``.npz`` file of the same name stem (``h5_f_XXXXXXXXXX.npz``), and the
readers take either.
"""
from __future__ import annotations

import os

import numpy as np

FRAME_DATASETS = ("x", "q", "time", "masses", "f_tensor", "stress", "v", "mu", "C")
STRESS_COMPONENTS = (0, 1, 2, 4, 5, 8)  # of the row-major 3x3 (mpm_solver_warp.py:383)


def h5py_module():
    """h5py if importable, else None."""
    try:
        import h5py  # noqa: F401
    except ImportError:
        return None
    return h5py


def frame_filename(dir_name: str, frame: int) -> str:
    """dir_name + '/h5_f_' + 10-digit frame + '.h5' (mpm_solver_warp.py:342); '.npz' without h5py."""
    ext = ".h5" if h5py_module() is not None else ".npz"
    return dir_name + "/h5_f_" + str(frame).zfill(10) + ext


def write_frame(path: str, arrays: dict) -> None:
    """Write the datasets in the given order: HDF5 for '.h5' (h5py), else '.npz'."""
    if os.path.exists(path):
        os.remove(path)
    if path.endswith(".h5"):
        h5py = h5py_module()
        if h5py is None:
            raise ImportError("writing .h5 frame files needs h5py")
        with h5py.File(path, "w") as f:
            for k, a in arrays.items():
                f.create_dataset(k, data=a)
        return
    with open(path, "wb") as fh:  # np.savez would append '.npz' to other names
        np.savez(fh, **arrays)


def read_frame(path: str) -> dict:
    """All datasets of a frame or sampling file ('.h5' through h5py, else '.npz')."""
    if path.endswith(".h5"):
        h5py = h5py_module()
        if h5py is None:
            raise ImportError("reading .h5 frame files needs h5py")
        with h5py.File(path, "r") as f:
            return {k: f[k][()] for k in f.keys()}
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def resolve(path: str) -> str:
    """The reference prefixes the working directory (os.getcwd() + name,
    :130, :269); a path that exists as given is taken as it is."""
    for cand in (os.getcwd() + path, path):
        if os.path.exists(cand):
            return cand
    raise FileNotFoundError(f"h5 file cannot be found at {os.getcwd() + path}")


def split_frame_buffer(buf: np.ndarray, n: int) -> dict:
    """The (34 n) float32 output of mpm_export_frame as the frame's arrays."""
    b = np.asarray(buf, np.float32).reshape(-1)
    assert b.size == 34 * n
    out, o = {}, 0
    for name, rows in (("x", 3), ("q", 3), ("masses", 1), ("f_tensor", 9), ("stress", 6), ("v", 3), ("C", 9)):
        out[name] = b[o * n:(o + rows) * n].reshape(rows, n)
        o += rows
    return out


def stress_from_components(stress6: np.ndarray) -> np.ndarray:
    """(n, 6) [xx, xy, xz, yy, yz, zz] -> (n, 3, 3) symmetric (mpm_solver_warp.py:283-292)."""
    s = np.asarray(stress6)
    full = np.zeros((s.shape[0], 3, 3), dtype=s.dtype)
    full[:, 0, 0], full[:, 0, 1], full[:, 0, 2] = s[:, 0], s[:, 1], s[:, 2]
    full[:, 1, 0], full[:, 1, 1], full[:, 1, 2] = s[:, 1], s[:, 3], s[:, 4]
    full[:, 2, 0], full[:, 2, 1], full[:, 2, 2] = s[:, 2], s[:, 4], s[:, 5]
    return full


def obj_lines(points: np.ndarray, colors) -> str:
    """'v x y z r g b' lines as the reference's OBJ writers print them
    (str of each float32 coordinate and of each color value, :312-336)."""
    pts = np.asarray(points, np.float32)
    out = []
    for i in range(pts.shape[0]):
        c = colors[i]
        out.append("v " + str(pts[i][0]) + " " + str(pts[i][1]) + " " + str(pts[i][2]) + " " +
                   " ".join(str(x) for x in c) + "\n")
    return "".join(out)
