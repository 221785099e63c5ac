"""A numpy stand-in for the Taichi names that DiffTactile's simulation methods use, so that those
methods' own source text runs as plain sequential Python in float64.  Used only by the fixture
scripts of this folder (make_substep.py), which read the methods out of a reference checkout with
`ast` and execute them on this module's fields.

Semantics taken for the Taichi primitives (the documented behaviour of Taichi 1.6):
  - a kernel's outermost loop runs its iterations; `+=` on a field element accumulates (Taichi makes
    it atomic; sequential execution here only fixes the summation order);
  - reading a field element gives a copy (`field[k][i] = x` still writes the field);
    `x.cast(int)` truncates toward zero;
  - `v.norm(eps) = sqrt(v.v + eps)`, `v.normalized(eps) = v / (|v| + eps)`;
  - `ti.math.sign(0) = +1` (never reached by the fixtures' inputs);
  - `ti.svd(F) = (U, diag(s), V)` with det U = det V = +1, the last singular value carrying the sign
    of det F (numpy's SVD with that normalisation), singular values in descending magnitude.
Indices outside a field's shape raise (Taichi leaves them undefined), so a fixture whose stencil or
contact search would leave its arrays fails instead of wrapping around.
"""
from __future__ import annotations

import itertools
import sys
import types

import numpy as np

i32, f32, f64 = int, float, float


class Arr(np.ndarray):
    """A Taichi vector or matrix value."""

    def __new__(cls, a, dtype=None):
        return np.array(a, dtype=dtype).view(cls)

    def cast(self, t):
        if t in (int, i32):
            return np.trunc(np.asarray(self, np.float64)).astype(np.int64).view(Arr)
        return np.asarray(self, np.float64).view(Arr)

    def norm_sqr(self):
        return float(np.sum(np.asarray(self, np.float64) ** 2))

    def norm(self, eps=0.0):
        return float(np.sqrt(self.norm_sqr() + eps))

    def normalized(self, eps=0.0):
        return self / (self.norm() + eps)

    def outer_product(self, o):
        return np.outer(np.asarray(self), np.asarray(o)).view(Arr)

    def cross(self, o):
        return np.cross(np.asarray(self), np.asarray(o)).view(Arr)

    def determinant(self):
        return float(np.linalg.det(np.asarray(self, np.float64)))

    def inverse(self):
        return np.linalg.inv(np.asarray(self, np.float64)).view(Arr)


class Elem(Arr):
    """A field element as read: a copy (arithmetic and `+=` on it stay local, as in Taichi), except
    that a component assignment made straight through the read, `field[k][i] = x`, also writes the
    field, which is what that form does in Taichi.  (The reference methods run here never assign a
    component of an element they stored in a local name.)"""

    _home = None

    def __array_finalize__(self, obj):
        self._home = None

    def __setitem__(self, i, v):
        super().__setitem__(i, v)
        if self._home is not None:
            a, k = self._home
            a[k][i] = v


class Field:
    """A Taichi field: ``shape`` indices, each element a scalar or an ``elem``-shaped value."""

    def __init__(self, shape, elem=(), dtype=np.float64):
        self.a = np.zeros(tuple(shape) + tuple(elem), dtype)
        self.shape = tuple(shape)

    def _key(self, key):
        if key is None:
            key = ()
        if not isinstance(key, tuple):
            key = (key,)
        out = []
        for k in key:
            if isinstance(k, np.ndarray) and k.ndim == 1:
                out.extend(int(c) for c in k)
            else:
                out.append(int(k))
        if len(out) != len(self.shape) or any(not 0 <= k < n for k, n in zip(out, self.shape)):
            raise IndexError(f"index {tuple(out)} outside a field of shape {self.shape}")
        return tuple(out)

    def __getitem__(self, key):
        k = self._key(key)
        v = self.a[k]
        if not isinstance(v, np.ndarray):
            return v.item()
        e = v.copy().view(Elem)
        e._home = (self.a, k)
        return e

    def __setitem__(self, key, val):
        self.a[self._key(key)] = np.asarray(val)

    def fill(self, v):
        self.a.fill(v)


def scalar(v):
    f = Field(())
    f[None] = v
    return f


# ---- decorators and compile-time helpers ----
def kernel(fn):
    return fn


func = kernel
data_oriented = kernel


def static(x):
    return x


def ndrange(*ns):
    return itertools.product(*[range(*n) if isinstance(n, tuple) else range(n) for n in ns])


def grouped(x):
    """Index vectors of a field's shape or of an ndrange."""
    it = ndrange(*x.shape) if isinstance(x, Field) else x
    return (Arr(i, np.int64) for i in it)


def cast(x, dtype):
    if dtype in (int, i32):
        return np.trunc(np.asarray(x, np.float64)).astype(np.int64).view(Arr)
    return np.asarray(x, np.float64).view(Arr) if isinstance(x, np.ndarray) else float(x)


# ---- values ----
class _Vector:
    def __call__(self, a, dt=None):
        a = list(a)
        ints = all(isinstance(c, (int, np.integer)) and not isinstance(c, bool) for c in a)
        return Arr(a, np.int64 if ints else np.float64)

    @staticmethod
    def zero(dtype, n):
        return Arr(np.zeros(n, np.int64 if dtype in (int, i32) else np.float64))


class _Matrix:
    def __call__(self, rows, dt=None):
        return Arr(np.array(rows, np.float64))

    @staticmethod
    def zero(dtype, n, m):
        return Arr(np.zeros((n, m)))

    @staticmethod
    def identity(dtype=None, n=None, dt=None):
        return Arr(np.eye(n))

    @staticmethod
    def diag(dim, val):
        return Arr(np.eye(dim) * val)

    @staticmethod
    def cols(cs):
        return Arr(np.stack([np.asarray(c, np.float64) for c in cs], 1))


Vector = _Vector()
Matrix = _Matrix()


def _ew(fn):
    def g(*a):
        r = fn(*[np.asarray(x) if isinstance(x, np.ndarray) else x for x in a])
        return r.view(Arr) if isinstance(r, np.ndarray) else float(r)
    return g


max = _ew(np.maximum)  # noqa: A001 - Taichi's names
min = _ew(np.minimum)  # noqa: A001
abs = _ew(np.abs)      # noqa: A001
log = _ew(np.log)
exp = _ew(np.exp)
sqrt = _ew(np.sqrt)
cos = _ew(np.cos)
sin = _ew(np.sin)
acos = _ew(np.arccos)
atan2 = _ew(np.arctan2)


def svd(F, dt=None):
    U, s, Vt = np.linalg.svd(np.asarray(F, np.float64))
    V = Vt.T.copy()
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(V) < 0:
        V[:, 2] *= -1
        s[2] *= -1
    return Arr(U), Arr(np.diag(s)), Arr(V)


math = types.SimpleNamespace(
    cross=lambda a, b: np.cross(np.asarray(a), np.asarray(b)).view(Arr),
    sign=lambda x: 1.0 if x >= 0 else -1.0,
    radians=lambda x: (np.asarray(x, np.float64) * (np.pi / 180.0)).view(Arr),
    clamp=lambda x, lo, hi: _ew(np.clip)(x, lo, hi),
    pi=np.pi,
)


def _defs(path, body, names, extra):
    import ast

    defs = [n for n in body if isinstance(n, ast.FunctionDef) and n.name in names]
    missing = set(names) - {d.name for d in defs}
    if missing:
        raise KeyError(f"{path} has no {sorted(missing)}")
    ns = {"ti": sys.modules[__name__], "np": np, **(extra or {})}
    exec(compile(ast.Module(body=defs, type_ignores=[]), path, "exec"), ns)
    return ns


def functions(path, names, extra=None):
    """The module-level functions ``names`` of the source file ``path``, executed with this module
    as ``ti`` (and the names of ``extra`` in scope)."""
    import ast

    ns = _defs(path, ast.parse(open(path).read(), path).body, names, extra)
    return {n: ns[n] for n in names}


def methods(path, cls_name, names, obj, extra=None):
    """Bind the methods ``names`` of class ``cls_name`` in the source file ``path`` to ``obj``, their
    source executed with this module as ``ti`` (and the names of ``extra`` in scope)."""
    import ast

    tree = ast.parse(open(path).read(), path)
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls_name)
    ns = _defs(path, cls.body, names, extra)
    for n in names:
        setattr(obj, n, types.MethodType(ns[n], obj))
    return obj
