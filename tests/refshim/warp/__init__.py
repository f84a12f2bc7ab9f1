"""Test-only stand-in for the ``warp`` package, enough to execute the
reference's Warp kernels unmodified as plain Python on the CPU.

Test infrastructure: only ``tests/golden/make_ref_fixtures.py`` puts this
directory on ``sys.path``.  Nothing in the library imports it.

The reference (engine_stress/mpm_utils.py, warp_utils.py, mpm_solver_warp.py)
writes its kernels in Warp's Python DSL.  Warp is not installed here, so
this module gives those names plain-Python meanings that follow Warp's
documented semantics:

* ``@wp.kernel`` keeps the function; ``wp.launch(kernel, dim, inputs)`` calls
  it once per thread index, ``wp.tid()`` returning that index (an int, or a
  tuple for a 3-D launch).  Arguments annotated ``float`` are rounded to
  float32 and ``@wp.struct`` arguments are passed by value with their float
  fields in float32, as a Warp launch packs them.
* ``@wp.func`` is the function itself (called from kernel code).
* ``vec3`` / ``mat33`` hold float32 NumPy arrays; every arithmetic operation
  rounds to float32 once (no fused multiply-add), in Python's left-to-right
  evaluation order, which is also the order of Warp's generated code.
  Matrix products accumulate ``sum_k a[i,k] b[k,j]`` over k = 0, 1, 2.
* ``mat33(c0, c1, c2)`` from three vectors builds the matrix from COLUMNS
  (Warp's matrix-from-vectors constructor of that era).  The reference relies
  on it: its weight matrix ``w = mat33(wa*wa/2, 0.75 - wb*wb, wc*wc/2)`` is
  indexed ``w[axis, i]`` (mpm_utils.py:207-219), which is the i-th quadratic
  B-spline weight along ``axis`` only with column construction.
  ``mat33(m00, m01, ..., m22)`` from nine scalars is row-major.
* ``svd3`` is the one piece of Warp arithmetic with no statement in the
  reference: it is computed in float64 by LAPACK and rounded to float32,
  with U and V proper rotations, singular values in descending order and
  the sign of det(A) carried by the last one.  The reference consumes it
  only through quantities invariant to the remaining choices (U diag V^T
  products, |sigma| and log sigma).
* Arrays are NumPy arrays on the host; ``atomic_add`` is a plain
  read-modify-write (one thread runs at a time).
"""
from __future__ import annotations

import builtins as _b
import ctypes
import inspect
import math

import numpy as np

from . import types  # noqa: F401  (warp.types is an attribute of the package)

f32 = np.float32

# --------------------------------------------------------------------- config
class _Config:
    verify_cuda = False
    mode = "release"


config = _Config()


def init():
    return None


# --------------------------------------------------------------- value types
def _scalar(x):
    return f32(x)


class vec3:
    __slots__ = ("a",)
    __array_ufunc__ = None  # numpy scalars defer to vec3's reflected operators

    def __init__(self, *args):
        if len(args) == 0:
            self.a = np.zeros(3, f32)
        elif len(args) == 1:
            x = args[0]
            if isinstance(x, vec3):
                self.a = x.a.copy()
            elif np.ndim(x) == 0:
                self.a = np.full(3, f32(x), f32)
            else:
                self.a = np.asarray(x, f32).reshape(3).copy()
        elif len(args) == 3:
            self.a = np.array([f32(args[0]), f32(args[1]), f32(args[2])], f32)
        else:
            raise TypeError("vec3 takes 0, 1 or 3 arguments")

    @staticmethod
    def _wrap(a):
        v = vec3.__new__(vec3)
        v.a = a
        return v

    def __getitem__(self, i):
        return self.a[i]

    def __setitem__(self, i, x):
        self.a[i] = f32(x)

    def __len__(self):
        return 3

    def __iter__(self):
        return iter(self.a)

    def __add__(self, o):
        return vec3._wrap(self.a + o.a)

    def __sub__(self, o):
        return vec3._wrap(self.a - o.a)

    def __neg__(self):
        return vec3._wrap(-self.a)

    def __mul__(self, s):
        if isinstance(s, (vec3, mat33)):
            raise TypeError("vec3 * vector/matrix is not a Warp operator used here")
        return vec3._wrap(self.a * f32(s))

    def __rmul__(self, s):
        return vec3._wrap(f32(s) * self.a)

    def __truediv__(self, s):
        return vec3._wrap(self.a / f32(s))

    def __repr__(self):
        return f"vec3({self.a[0]}, {self.a[1]}, {self.a[2]})"


class mat33:
    __slots__ = ("a",)
    __array_ufunc__ = None

    def __init__(self, *args):
        if len(args) == 0:
            self.a = np.zeros((3, 3), f32)
        elif len(args) == 1:
            x = args[0]
            if isinstance(x, mat33):
                self.a = x.a.copy()
            elif np.ndim(x) == 0:
                self.a = np.full((3, 3), f32(x), f32)
            else:
                self.a = np.asarray(x, f32).reshape(3, 3).copy()
        elif len(args) == 3:
            # matrix from three vectors: the vectors are the columns
            self.a = np.stack([vec3(c).a for c in args], axis=1).astype(f32)
        elif len(args) == 9:
            self.a = np.array([f32(v) for v in args], f32).reshape(3, 3)
        else:
            raise TypeError("mat33 takes 0, 1, 3 or 9 arguments")

    @staticmethod
    def _wrap(a):
        m = mat33.__new__(mat33)
        m.a = a
        return m

    def __getitem__(self, idx):
        if isinstance(idx, tuple):
            return self.a[idx]
        return vec3._wrap(self.a[idx].copy())  # a row

    def __setitem__(self, idx, x):
        if isinstance(idx, tuple):
            self.a[idx] = f32(x)
        else:
            self.a[idx] = vec3(x).a

    def __add__(self, o):
        return mat33._wrap(self.a + o.a)

    def __sub__(self, o):
        return mat33._wrap(self.a - o.a)

    def __neg__(self):
        return mat33._wrap(-self.a)

    def __mul__(self, o):
        if isinstance(o, mat33):
            a, b = self.a, o.a
            r = a[:, 0:1] * b[0:1, :]
            r = r + a[:, 1:2] * b[1:2, :]
            r = r + a[:, 2:3] * b[2:3, :]
            return mat33._wrap(r)
        if isinstance(o, vec3):
            a, v = self.a, o.a
            r = a[:, 0] * v[0]
            r = r + a[:, 1] * v[1]
            r = r + a[:, 2] * v[2]
            return vec3._wrap(r)
        return mat33._wrap(self.a * f32(o))

    def __rmul__(self, s):
        return mat33._wrap(f32(s) * self.a)

    def __truediv__(self, s):
        return mat33._wrap(self.a / f32(s))

    def __repr__(self):
        return f"mat33({self.a.tolist()})"


float32 = f32
int32 = np.int32


def _elem(dtype):
    """(numpy dtype, element shape, wrapper) of a Warp element type."""
    if dtype is vec3:
        return f32, (3,), vec3._wrap
    if dtype is mat33:
        return f32, (3, 3), mat33._wrap
    if dtype in (_b.float, f32):
        return f32, (), f32
    if dtype in (_b.int, np.int32):
        return np.int32, (), int
    raise TypeError(f"unsupported array dtype {dtype!r}")


# ---------------------------------------------------------------------- arrays
class array:
    """Host array of Warp elements.  Constructed with no data it is only a type
    annotation (``wp.array(dtype=float)``)."""

    def __init__(self, data=None, dtype=_b.float, shape=None, ptr=None, ndim=None, copy=True,
                 owner=True, requires_grad=False, device=None, **_kw):
        self.dtype = dtype
        self.device = device
        self.requires_grad = requires_grad
        npdt, esh, _ = _elem(dtype)
        if data is None and ptr is None and shape is None:
            self.data = None  # a type annotation
            self.ndim = ndim or 1
            return
        if ptr is not None:
            shp = (shape,) if isinstance(shape, _b.int) else tuple(shape)
            count = int(np.prod(shp + esh))
            ctype = ctypes.c_float if npdt == f32 else ctypes.c_int32
            buf = (ctype * count).from_address(ptr)
            self.data = np.ctypeslib.as_array(buf).reshape(shp + esh)
        elif data is not None:
            d = np.asarray(data, npdt)
            self.data = d.copy() if copy else d
            if shape is not None:
                shp = (shape,) if isinstance(shape, _b.int) else tuple(shape)
                self.data = self.data.reshape(shp + esh)
        else:
            shp = (shape,) if isinstance(shape, _b.int) else tuple(shape)
            self.data = np.zeros(shp + esh, npdt)
        self.ndim = self.data.ndim - len(esh)

    @property
    def shape(self):
        return self.data.shape[: self.ndim]

    def __len__(self):
        return self.data.shape[0]

    def __getitem__(self, idx):
        _, esh, wrap = _elem(self.dtype)
        x = self.data[idx]
        if esh:
            return wrap(x.copy())
        return wrap(x)

    def __setitem__(self, idx, value):
        if isinstance(value, (vec3, mat33)):
            self.data[idx] = value.a
        else:
            self.data[idx] = value

    def numpy(self):
        return self.data


def zeros(shape=None, dtype=_b.float, device=None, requires_grad=False, **_kw):
    return array(shape=shape, dtype=dtype, device=device, requires_grad=requires_grad)


def empty(shape=None, dtype=_b.float, device=None, requires_grad=False, **_kw):
    return array(shape=shape, dtype=dtype, device=device, requires_grad=requires_grad)


def from_numpy(arr, dtype=None, shape=None, device=None, requires_grad=False):
    npdt, esh, _ = _elem(dtype if dtype is not None else _b.float)
    d = np.array(arr, npdt)
    n_el = len(esh)
    if n_el and d.shape[-n_el:] != esh:
        d = d.reshape((-1,) + esh)
    return array(data=d, dtype=dtype if dtype is not None else _b.float, device=device, copy=False)


def from_torch(t, dtype=None, requires_grad=None):
    """Warp's from_torch takes (tensor, dtype, requires_grad) only."""
    dt = dtype if dtype is not None else _b.float
    return array(data=t.detach().cpu().numpy(), dtype=dt, copy=False)


def to_torch(a):
    import torch

    return torch.from_numpy(a.data)


# --------------------------------------------------------------------- structs
def _kernel_value(t, v):
    """A struct field or kernel argument as a kernel sees it (float32 scalars)."""
    if t is _b.float:
        return f32(v)
    if t is _b.int:
        return _b.int(v)
    if t is vec3:
        return vec3(v)
    if t is mat33:
        return mat33(v)
    return v


def _default(t):
    if t is _b.float:
        return 0.0
    if t is _b.int:
        return 0
    if t is vec3:
        return vec3()
    if t is mat33:
        return mat33()
    return None


def struct(cls):
    fields = dict(cls.__annotations__)

    def __init__(self):
        for k, t in fields.items():
            object.__setattr__(self, k, _default(t))

    def _kernel_view(self):
        v = object.__new__(type(self))
        for k, t in fields.items():
            object.__setattr__(v, k, _kernel_value(t, getattr(self, k)))
        return v

    ns = {"__init__": __init__, "_kernel_view": _kernel_view, "_wp_fields": fields,
          "__module__": cls.__module__, "__qualname__": cls.__qualname__}
    return type(cls.__name__, (), ns)


# --------------------------------------------------------------------- kernels
_TID = [0]


def tid():
    return _TID[0]


class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.key = fn.__name__
        sig = inspect.signature(fn)
        self.params = list(sig.parameters.values())


def kernel(fn):
    return Kernel(fn)


def func(fn):
    return fn


def _arg(p, v):
    ann = p.annotation
    if hasattr(v, "_kernel_view"):
        return v._kernel_view()
    if ann is _b.float:
        return f32(v)
    if ann is _b.int:
        return _b.int(v)
    if ann is vec3:
        return vec3(v)
    return v


def launch(kernel, dim, inputs=(), outputs=(), device=None, **_kw):
    args = list(inputs) + list(outputs)
    args = [_arg(p, v) for p, v in zip(kernel.params, args)]
    fn = kernel.fn
    if isinstance(dim, _b.int):
        for i in range(dim):
            _TID[0] = i
            fn(*args)
    else:
        dims = tuple(dim)
        for idx in np.ndindex(*dims):
            _TID[0] = tuple(_b.int(i) for i in idx)
            fn(*args)


def synchronize():
    return None


# -------------------------------------------------------------------- builtins
def int(x):  # noqa: A001  (wp.int: truncation toward zero)
    return _b.int(x)


def float(x):  # noqa: A001  (wp.float: to float32)
    return f32(x)


def _is_vec(x):
    return isinstance(x, (vec3, mat33))


def add(a, b):
    return a + b


def sub(a, b):
    return a - b


def dot(a, b):
    r = a.a[0] * b.a[0]
    r = r + a.a[1] * b.a[1]
    return r + a.a[2] * b.a[2]


def length(v):
    return f32(np.sqrt(dot(v, v)))


def normalize(v):
    n = length(v)
    if n > f32(0.0):
        return v * (f32(1.0) / n)
    return vec3()


def cw_mul(a, b):
    return vec3._wrap(a.a * b.a)


def outer(a, b):
    return mat33._wrap(a.a[:, None] * b.a[None, :])


def transpose(m):
    return mat33._wrap(m.a.T.copy())


def diag(v):
    m = np.zeros((3, 3), f32)
    m[0, 0], m[1, 1], m[2, 2] = v.a[0], v.a[1], v.a[2]
    return mat33._wrap(m)


def determinant(m):
    a = m.a
    return (a[0, 0] * (a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2])
            + a[0, 1] * (a[1, 2] * a[2, 0] - a[1, 0] * a[2, 2])
            + a[0, 2] * (a[1, 0] * a[2, 1] - a[1, 1] * a[2, 0]))


def svd3(A, U, sigma, V):
    """float64 LAPACK SVD rounded to float32 (U, V rotations, sigma descending,
    sign of det A on the last); writes into U, sigma and V as Warp does."""
    a = A.a.astype(np.float64)
    u, s, vt = np.linalg.svd(a)
    v = vt.T.copy()
    s = s.copy()
    if np.linalg.det(u) < 0:
        u[:, 2] = -u[:, 2]
        s[2] = -s[2]
    if np.linalg.det(v) < 0:
        v[:, 2] = -v[:, 2]
        s[2] = -s[2]
    U.a[...] = u.astype(f32)
    V.a[...] = v.astype(f32)
    sigma.a[...] = s.astype(f32)


def _unary(npf):
    def f(x):
        return f32(npf(f32(x)))
    return f


log = _unary(np.log)
exp = _unary(np.exp)
sqrt = _unary(np.sqrt)
sin = _unary(np.sin)
cos = _unary(np.cos)
acos = _unary(np.arccos)


def abs(x):  # noqa: A001
    return f32(np.abs(f32(x)))


def max(a, b):  # noqa: A001
    return f32(np.maximum(f32(a), f32(b)))


def min(a, b):  # noqa: A001
    return f32(np.minimum(f32(a), f32(b)))


def atomic_add(arr, *args):
    *idx, value = args
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    if isinstance(value, (vec3, mat33)):
        arr.data[idx] = arr.data[idx] + value.a
    else:
        arr.data[idx] = arr.data[idx] + f32(value)


__all__ = [n for n in dir() if not n.startswith("_")]
_ = math
