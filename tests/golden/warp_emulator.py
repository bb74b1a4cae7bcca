"""A minimal CPU stand-in for the parts of the ``warp`` API the reference's GPU package uses.

Test infrastructure for ``make_golden.py``.  Warp itself is not installed here, so the
reference's own kernels (direbm/warp/physics.py, propagation.py, simulator.py, lbm.py) cannot
run as published.  Installed as ``sys.modules["warp"]``, this module lets the reference's code run
unchanged on the host:
  - ``@wp.kernel`` / ``@wp.func`` functions are plain Python;
  - ``wp.launch`` calls the kernel once per thread index, in index order, with ``wp.tid()``
    returning that index and each scalar argument converted to its annotated type;
  - arithmetic is numpy float32 / int32 scalars and float32 vectors.  Each operation is rounded on
    its own (IEEE round-to-nearest, no fused multiply-add), the convention of this library's
    oracle;
  - ``wp.hash_grid_query`` visits, in increasing point index, the points of the grid cells up to
    one cell beyond the query radius, so every point whose FP32 distance passes the kernel's own
    test is visited.  ``wp.hash_grid_query_next`` writes the next index into its
    by-reference argument, as Warp's does; ``wp.int32`` values are mutable cells for that reason;
  - ``wp.atomic_add`` adds in launch order;
  - ``wp.utils.radix_sort_pairs`` is a stable sort, ``runlength_encode`` and ``array_scan`` as
    documented by Warp.
Sums whose order Warp leaves open (hash-grid visits, atomics) are therefore one valid order of
the reference's algorithm; exact-arithmetic decisions (cells, radius tests, thresholds) are the
reference's own.  Slow (one Python call per thread): sized for fixtures of a few thousand
components.
"""

from __future__ import annotations

import inspect
import types

import numpy as np

F32 = np.float32
I32 = np.int32

_tid = [0]
_grids: dict[int, "HashGrid"] = {}


# ---- scalar and vector types -----------------------------------------------------------------

class _MutInt:
    """A Warp int32 local: a mutable cell (so hash_grid_query_next can write it) that behaves as
    np.int32 in arithmetic, comparisons and indexing."""

    __slots__ = ("v",)
    __array_ufunc__ = None  # numpy scalars defer to the reflected operators below

    def __init__(self, v=0):
        self.v = I32(int(v))

    def __index__(self):
        return int(self.v)

    __int__ = __index__

    def __repr__(self):
        return f"int32({int(self.v)})"

    def __hash__(self):
        return hash(int(self.v))


def _binop(name):
    def f(self, other):
        o = other.v if isinstance(other, _MutInt) else other
        return getattr(self.v, name)(o)
    return f


for _n in ("add", "sub", "mul", "floordiv", "mod", "and", "or", "xor", "lshift", "rshift", "truediv"):
    setattr(_MutInt, f"__{_n}__", _binop(f"__{_n}__"))
    setattr(_MutInt, f"__r{_n}__", _binop(f"__r{_n}__"))
for _n in ("lt", "le", "gt", "ge", "eq", "ne"):
    setattr(_MutInt, f"__{_n}__", _binop(f"__{_n}__"))
_MutInt.__neg__ = lambda self: -self.v
_MutInt.__bool__ = lambda self: bool(self.v)


def int32(v=0):
    return _MutInt(v)


int32._np = I32


def float32(v=0.0):
    return F32(v)


float32._np = F32


def uint32(v=0):
    return np.uint32(v)


uint32._np = np.uint32


def uint64(v=0):
    return int(v)


uint64._np = None
float64 = np.float64
int64 = np.int64


class _Vec:
    _n = 0

    def __new__(cls, *a):
        if len(a) == 0:
            a = (0.0,) * cls._n
        return np.array([F32(x) for x in a], dtype=F32)


class vec2(_Vec):
    _n = 2


class vec3(_Vec):
    _n = 3


def _width(dtype):
    return getattr(dtype, "_n", 0)


def _np_dtype(dtype):
    if dtype in (None, float, float32, vec2, vec3):
        return F32
    if dtype in (int, int32):
        return I32
    if dtype is uint32:
        return np.uint32
    if dtype is uint64:
        return np.uint64
    if dtype in (np.float64, float64):
        return np.float64
    return np.dtype(dtype).type


# ---- arrays --------------------------------------------------------------------------------------

def _ix(k):
    if isinstance(k, tuple):
        return tuple(int(i) for i in k)
    return int(k)


class array:
    """A Warp array on the host: numpy storage; vector dtypes keep a trailing axis of their width.
    ``array(dtype=...)`` without data is only a type annotation in a kernel signature."""

    def __init__(self, data=None, dtype=None, shape=None, device=None, ndim=None):
        self.dtype = dtype
        self.device = device
        w = _width(dtype)
        if data is None and shape is None:
            self.a = None  # annotation only
            return
        if data is None:
            shape = (shape,) if np.isscalar(shape) else tuple(shape)
            self.a = np.zeros(shape + ((w,) if w else ()), dtype=_np_dtype(dtype))
        else:
            self.a = np.array(data, dtype=_np_dtype(dtype), copy=True)
            if w and self.a.ndim == 1:
                self.a = self.a.reshape(-1, w)

    @property
    def shape(self):
        return self.a.shape[:-1] if _width(self.dtype) else self.a.shape

    def __len__(self):
        return self.shape[0]

    def numpy(self):
        return self.a.copy()

    def __getitem__(self, k):
        v = self.a[_ix(k)]
        return v.copy() if isinstance(v, np.ndarray) else v

    def __setitem__(self, k, v):
        self.a[_ix(k)] = v

    @property
    def ptr(self):
        return id(self)


def array2d(dtype=None):
    return array(dtype=dtype)


def array3d(dtype=None):
    return array(dtype=dtype)


def zeros(shape, dtype=float32, device=None):
    return array(dtype=dtype, shape=shape, device=device)


# ---- builtins ------------------------------------------------------------------------------------

def tid():
    return _tid[0]


def floor(x):
    return F32(np.floor(F32(x)))


def exp(x):
    return F32(np.exp(F32(x)))


def sqrt(x):
    return F32(np.sqrt(F32(x)))


def dot(a, b):
    s = F32(a[0] * b[0])
    for i in range(1, len(a)):
        s = F32(s + F32(a[i] * b[i]))
    return s


def length(v):
    return sqrt(dot(v, v))


def atomic_add(arr, *args):
    *idx, value = args
    k = _ix(tuple(idx)) if len(idx) > 1 else _ix(idx[0])
    arr.a[k] = arr.a[k] + value


def min(a, b):  # noqa: A001 - Warp's name
    return a if a < b else b


def max(a, b):  # noqa: A001 - Warp's name
    return a if a > b else b


# ---- kernels ---------------------------------------------------------------------------------------

def func(f):
    return f


def kernel(f=None, **_):
    if f is None:
        return lambda g: g
    return f


def _convert(arg, ann):
    conv = getattr(ann, "_np", "absent")
    if conv == "absent" or isinstance(arg, array):
        return arg
    if ann is uint64:
        return int(arg)
    if ann is int32:
        return I32(int(arg))
    if ann in (vec2, vec3):
        return np.asarray(arg, dtype=F32)
    return conv(arg)


def launch(kern, dim, inputs=(), outputs=(), device=None, **_):
    params = list(inspect.signature(kern).parameters.values())
    args = [_convert(a, p.annotation) for a, p in zip(list(inputs) + list(outputs), params)]
    if np.isscalar(dim) or len(dim) == 1:
        for i in range(int(dim if np.isscalar(dim) else dim[0])):
            _tid[0] = i
            kern(*args)
    else:  # wp.tid() unpacks to one index per launch dimension, the last fastest
        for ix in np.ndindex(*tuple(int(d) for d in dim)):
            _tid[0] = tuple(int(i) for i in ix)
            kern(*args)


def init():
    pass


def synchronize():
    pass


def get_cuda_devices():
    return []


# ---- hash grid -------------------------------------------------------------------------------------

class HashGrid:
    def __init__(self, dim_x, dim_y, dim_z, device=None):
        self.id = len(_grids) + 1
        _grids[self.id] = self
        self.cells = {}
        self.cell = 1.0

    def build(self, points, radius):
        self.cell = float(radius)
        p = np.asarray(points.a, dtype=np.float64)
        keys = np.floor(p / self.cell).astype(np.int64)
        self.cells = {}
        for i, k in enumerate(map(tuple, keys)):
            self.cells.setdefault(k, []).append(i)


class _Query:
    __slots__ = ("cand", "pos")

    def __init__(self, cand):
        self.cand = cand
        self.pos = 0


def hash_grid_query(grid_id, point, radius):
    g = _grids[int(grid_id)]
    c = np.floor(np.asarray(point, dtype=np.float64) / g.cell).astype(np.int64)
    # one cell beyond the radius: a point whose FP32 distance rounds down onto the radius can sit
    # in the next cell but one, and the kernel's own distance test decides
    reach = int(np.ceil(float(radius) / g.cell)) + 1
    cand = []
    rng = range(-reach, reach + 1)
    for dz in (rng if len(c) > 2 else (0,)):
        for dy in rng:
            for dx in rng:
                key = (c[0] + dx, c[1] + dy) + ((c[2] + dz,) if len(c) > 2 else ())
                cand.extend(g.cells.get(key, ()))
    return _Query(sorted(cand))


def hash_grid_query_next(query, index):
    if query.pos >= len(query.cand):
        return False
    index.v = I32(query.cand[query.pos])
    query.pos += 1
    return True


# ---- wp.utils ----------------------------------------------------------------------------------------

def _radix_sort_pairs(keys, values, count):
    n = int(count)
    order = np.argsort(keys.a[:n], kind="stable")
    keys.a[:n] = keys.a[:n][order]
    values.a[:n] = values.a[:n][order]


def _runlength_encode(values, run_values, run_lengths, run_count=None, value_count=None):
    n = int(value_count) if value_count is not None else len(values)
    v = values.a[:n]
    if n == 0:
        if run_count is not None:
            run_count.a[0] = 0
        return 0
    head = np.ones(n, dtype=bool)
    head[1:] = v[1:] != v[:-1]
    starts = np.flatnonzero(head)
    lens = np.diff(np.append(starts, n))
    run_values.a[: len(starts)] = v[starts]
    run_lengths.a[: len(starts)] = lens
    if run_count is not None:
        run_count.a[0] = len(starts)
    return len(starts)


def _array_scan(src, dst, inclusive=True):
    c = np.cumsum(src.a, dtype=src.a.dtype)
    dst.a[:] = c if inclusive else np.concatenate([[0], c[:-1]]).astype(src.a.dtype)


utils = types.SimpleNamespace(radix_sort_pairs=_radix_sort_pairs, runlength_encode=_runlength_encode,
                              array_scan=_array_scan)


def install():
    """Register this module as ``warp`` (before the reference's ``direbm.warp`` is imported)."""
    import sys

    sys.modules["warp"] = sys.modules[__name__]
