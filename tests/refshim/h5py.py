"""Stand-in for ``h5py``: a File keeps its datasets in a NumPy ``.npz``
container under the name it is given, so the reference's frame writer
(engine_stress/mpm_solver_warp.py:339-404) and sampling loader (:129-153)
run unchanged.  Test infrastructure only."""
import os

import numpy as np


class Dataset:
    def __init__(self, arr):
        self._a = np.asarray(arr)

    def __getitem__(self, idx):
        if idx == ():
            return self._a.copy()
        return self._a[idx]

    def __array__(self, dtype=None, copy=None):
        return self._a if dtype is None else self._a.astype(dtype)

    @property
    def shape(self):
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype


class File:
    def __init__(self, name, mode="r"):
        self.name = name
        self.mode = mode
        self._d = {}
        if mode == "r":
            with open(name, "rb") as f:
                z = np.load(f, allow_pickle=False)
                self._d = {k: z[k] for k in z.files}

    def __getitem__(self, key):
        return Dataset(self._d[key])

    def keys(self):
        return self._d.keys()

    def create_dataset(self, name, data=None, **_kw):
        self._d[name] = np.asarray(data)
        self._flush()
        return Dataset(self._d[name])

    def _flush(self):
        with open(self.name, "wb") as f:
            np.savez(f, **self._d)

    def close(self):
        if self.mode != "r":
            self._flush()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
