"""A minimal numpy stand-in for the parts of the Taichi API that the
reference's solver functions use -- TEST INFRASTRUCTURE ONLY.

It lets ``make_reference_vectors.py`` execute the reference's own Python
source (distance.py, lbvh_cell.py, XPBD.py, collision_constraints_x.py) on
small seeded inputs in a container where Taichi cannot be installed, to
produce golden vectors for the CPU oracle.  Semantics:

* kernels run serially in Python; a parallel ``for`` runs in ascending index,
  which is one of the orders Taichi's parallel loop with atomic ``+=`` may
  take, and the order the oracle fixes;
* scalars are numpy float32 / int32, so every arithmetic operation rounds to
  IEEE float32 (no fused multiply-add);
* vector and matrix operations follow Taichi's definitions in Python scope:
  ``dot`` = sum of products left to right, ``cross`` the usual component
  formula, ``norm`` = sqrt(dot(v, v)), ``normalized`` = (1 / (norm + eps)) * v,
  a 2x2 ``inverse`` = (1 / det) * adjugate with det = a00 a11 - a01 a10, and
  ``A @ v`` sums its products left to right;
* fields are numpy arrays; vector fields hand out copies on read.

Taichi's compiled kernels may contract or reassociate floating-point
operations (its default fast-math), so this pins the reference's source-level
algorithm (expression order, branches, quirks) under strict IEEE float32
arithmetic, not the last bits of a Taichi build.
"""
from __future__ import annotations

import ast
import inspect
import sys
import textwrap
import types as _pytypes

import numpy as np

_F = np.float32


class _Type:
    def __init__(self, np_type):
        self.np = np_type

    def __call__(self, *a, **k):  # ti.template() and friends
        return self


float32 = _Type(np.float32)
int32 = _Type(np.int32)
uint32 = _Type(np.uint32)
uint64 = _Type(np.uint64)
int64 = _Type(np.int64)
float64 = _Type(np.float64)
u8 = _Type(np.uint8)
f64 = float64
template = _Type(None)


def _cast_scalar(v, t):
    if isinstance(t, _Type) and t.np is not None:
        return t.np(v)
    return v


def _atomic_field(op, f, idx, v):
    """Atomic read-modify-write of a field element; returns the old value."""
    old = f[idx]
    if op == "add":
        f[idx] = old + v
    elif op == "sub":
        f[idx] = old - v
    elif op == "max":
        f[idx] = old if old > v else v
    else:
        f[idx] = old if old < v else v
    return old


class _AtomicRewrite(ast.NodeTransformer):
    """ti.atomic_op(name, v) on a local becomes an augmented assignment;
    ti.atomic_op(field[i], v) becomes _atomic_field(op, field, i, v)."""

    OPS = {"atomic_add": "add", "atomic_sub": "sub", "atomic_max": "max", "atomic_min": "min"}

    @classmethod
    def _is_atomic(cls, node):
        return (isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute)
                and isinstance(node.func.value, ast.Name) and node.func.value.id == "ti"
                and node.func.attr in cls.OPS)

    def visit_Expr(self, node):
        if self._is_atomic(node.value) and isinstance(node.value.args[0], ast.Name):
            call = node.value
            name = call.args[0].id
            op = self.OPS[call.func.attr]
            if op in ("add", "sub"):
                return ast.copy_location(ast.AugAssign(target=ast.Name(name, ast.Store()),
                                                       op=ast.Add() if op == "add" else ast.Sub(),
                                                       value=call.args[1]), node)
            fn = "max" if op == "max" else "min"
            return ast.copy_location(ast.Assign(targets=[ast.Name(name, ast.Store())],
                                                value=ast.Call(ast.Name(fn, ast.Load()),
                                                               [ast.Name(name, ast.Load()), call.args[1]], [])),
                                     node)
        return self.generic_visit(node)

    def visit_Call(self, node):
        self.generic_visit(node)
        if self._is_atomic(node) and isinstance(node.args[0], ast.Subscript):
            sub = node.args[0]
            return ast.copy_location(
                ast.Call(ast.Attribute(ast.Name("ti", ast.Load()), "_atomic_field", ast.Load()),
                         [ast.Constant(self.OPS[node.func.attr]), sub.value, sub.slice, node.args[1]], []), node)
        return node


def _rewrite(fn):
    """The function recompiled from its source outside any class (so that, as
    in Taichi's own front end, names such as ``module.__vt_st`` are not
    mangled), with the atomics rewritten (see _AtomicRewrite)."""
    try:
        src = textwrap.dedent(inspect.getsource(fn))
    except (OSError, TypeError):
        return fn
    if "atomic_" not in src and "__" not in src.split(":", 1)[-1]:
        return fn
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_AtomicRewrite().visit(tree))
    ns = {}
    exec(compile(tree, inspect.getsourcefile(fn) or "<reference>", "exec"), fn.__globals__, ns)
    return ns[fdef.name]


def kernel(fn):
    fn = _rewrite(fn)
    sig = inspect.signature(fn)

    def run(*args, **kwargs):
        bound = sig.bind(*args, **kwargs)
        for name, val in list(bound.arguments.items()):
            ann = sig.parameters[name].annotation
            if isinstance(ann, _Type) and ann.np is not None and np.isscalar(val):
                bound.arguments[name] = ann.np(val)
        return fn(*bound.args, **bound.kwargs)

    run.__wrapped__ = fn
    return run


def func(fn):
    return _rewrite(fn)


def data_oriented(cls):
    return cls


def loop_config(*a, **k):
    pass


class StructField:
    """Field of a ti.dataclass: one numpy array per member."""

    def __init__(self, members, shape):
        shape = (shape,) if np.isscalar(shape) else tuple(shape)
        object.__setattr__(self, "_m", {})
        for name, ann in members.items():
            if ann is math.vec3:
                self._m[name] = Field(np.zeros(shape + (3,), np.float32), 3)
            else:
                t = ann.np if isinstance(ann, _Type) and ann.np is not None else np.int32
                self._m[name] = Field(np.zeros(shape, t))

    def __getattr__(self, k):
        return self._m[k]

    def __getitem__(self, i):
        return _StructRef(self, int(i))


class _StructRef:
    def __init__(self, sf, i):
        object.__setattr__(self, "_sf", sf)
        object.__setattr__(self, "_i", i)

    def __getattr__(self, k):
        return self._sf._m[k][self._i]

    def __setattr__(self, k, v):
        self._sf._m[k][self._i] = v


def dataclass(cls):
    members = dict(getattr(cls, "__annotations__", {}))
    cls.field = staticmethod(lambda shape=(), **k: StructField(members, shape))
    return cls


def static(x, *a):
    return x


def cast(v, t):
    if isinstance(v, Vec):
        return Vec([_cast_scalar(c, t) for c in v.c])
    if isinstance(t, _Type) and t.np is not None and np.issubdtype(t.np, np.integer):
        if isinstance(v, (float, np.floating)):
            return t.np(np.trunc(v))
    return _cast_scalar(v, t)


def sqrt(x):
    return np.sqrt(x if isinstance(x, (np.floating, np.ndarray)) else _F(x))


def abs(x):  # noqa: A001
    return np.abs(x)


def min(a, b):  # noqa: A001
    if isinstance(a, Vec):
        return Vec([x if x < y else y for x, y in zip(a.c, b.c)])
    return a if a < b else b


def max(a, b):  # noqa: A001
    if isinstance(a, Vec):
        return Vec([x if x > y else y for x, y in zip(a.c, b.c)])
    return a if a > b else b


class Vec:
    """A small float32 (or int) vector with Taichi's Python-scope operations."""

    __array_priority__ = 100

    def __init__(self, comps):
        if isinstance(comps, Vec):
            comps = comps.c
        self.c = [x for x in comps]

    @property
    def n(self):
        return len(self.c)

    def __len__(self):
        return len(self.c)

    def __getitem__(self, i):
        return self.c[i]

    def __setitem__(self, i, v):
        self.c[i] = v

    @property
    def x(self):
        return self.c[0]

    @property
    def y(self):
        return self.c[1]

    @property
    def z(self):
        return self.c[2]

    def _bin(self, o, op):
        if isinstance(o, Vec):
            return Vec([op(a, b) for a, b in zip(self.c, o.c)])
        return Vec([op(a, o) for a in self.c])

    def _rbin(self, o, op):
        return Vec([op(o, a) for a in self.c])

    def __add__(self, o):
        return self._bin(o, lambda a, b: a + b)

    def __radd__(self, o):
        return self._rbin(o, lambda a, b: a + b)

    def __sub__(self, o):
        return self._bin(o, lambda a, b: a - b)

    def __rsub__(self, o):
        return self._rbin(o, lambda a, b: a - b)

    def __mul__(self, o):
        return self._bin(o, lambda a, b: a * b)

    def __rmul__(self, o):
        return self._rbin(o, lambda a, b: a * b)

    def __truediv__(self, o):
        return self._bin(o, lambda a, b: a / b)

    def __rtruediv__(self, o):
        return self._rbin(o, lambda a, b: a / b)

    def __neg__(self):
        return Vec([-a for a in self.c])

    def sum(self):
        r = self.c[0]
        for a in self.c[1:]:
            r = r + a
        return r

    def dot(self, o):
        return (self * o).sum()

    def cross(self, o):
        a, b = self.c, o.c
        return Vec([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])

    def norm_sqr(self):
        return self.dot(self)

    def norm(self, eps=0):
        return np.sqrt(self.norm_sqr() + eps)

    def normalized(self, eps=0):
        invlen = 1 / (self.norm() + eps)
        return invlen * self

    def outer_product(self, o):
        return Mat([[a * b for b in o.c] for a in self.c])

    def to_numpy(self):
        return np.array(self.c)

    def cast(self, t):
        if t is int or (isinstance(t, _Type) and t.np is not None and np.issubdtype(t.np, np.integer)):
            return Vec([int(np.trunc(np.float64(x))) for x in self.c])
        return Vec([_F(x) for x in self.c])


class Mat:
    def __init__(self, rows):
        if isinstance(rows, Mat):
            rows = rows.r
        self.r = [[x for x in row] for row in rows]

    def __call__(self, i, j):
        return self.r[i][j]

    def __getitem__(self, ij):
        i, j = ij
        return self.r[i][j]

    def determinant(self):
        if len(self.r) == 2:
            return self.r[0][0] * self.r[1][1] - self.r[0][1] * self.r[1][0]
        raise NotImplementedError("determinant of this size")

    def inverse(self):
        if len(self.r) == 2:
            inv_det = 1.0 / self.determinant()
            return Mat([[inv_det * self.r[1][1], inv_det * -self.r[0][1]],
                        [inv_det * -self.r[1][0], inv_det * self.r[0][0]]])
        raise NotImplementedError("inverse of this size")

    def __matmul__(self, v):
        if isinstance(v, Vec):
            out = []
            for row in self.r:
                acc = row[0] * v.c[0]
                for j in range(1, len(row)):
                    acc = acc + row[j] * v.c[j]
                out.append(acc)
            return Vec(out)
        raise NotImplementedError("matrix product")

    def __mul__(self, o):
        return Mat([[a * o for a in row] for row in self.r])

    def __rmul__(self, o):
        return Mat([[o * a for a in row] for row in self.r])


def _vec_ctor(n, dtype=np.float32):
    def make(*args):
        if len(args) == 1 and isinstance(args[0], (list, tuple, Vec, np.ndarray)):
            comps = list(args[0])
        elif len(args) == 1:
            comps = [args[0]] * n
        else:
            comps = list(args)
        if dtype is int:
            return Vec([int(c) for c in comps])
        return Vec([dtype(c) for c in comps])

    return make


def _mat_ctor(n):
    def make(rows):
        return Mat([[_F(x) for x in row] for row in rows])

    return make


math = _pytypes.SimpleNamespace(
    vec2=_vec_ctor(2), vec3=_vec_ctor(3), vec4=_vec_ctor(4), ivec2=_vec_ctor(2, int),
    ivec3=_vec_ctor(3, int), mat2=_mat_ctor(2), mat3=_mat_ctor(3),
    clamp=lambda x, lo, hi: (lo if x < lo else (hi if x > hi else x)),
    sqrt=sqrt, min=lambda a, b: min(a, b), max=lambda a, b: max(a, b), dot=lambda a, b: a.dot(b), cross=lambda a, b: a.cross(b),
    normalize=lambda a: a.normalized(), length=lambda a: a.norm(),
    clz=lambda v: 32 - int(np.uint32(v)).bit_length(),
)


class Field:
    """A scalar (n = None) or vector field backed by a numpy array."""

    def __init__(self, data, n=None):
        self.a = data
        self.n = n

    def __getitem__(self, i):
        if isinstance(i, tuple):
            i = tuple(int(k) for k in i)
        else:
            i = int(i)
        if self.n is None:
            v = self.a[i]
            return int(v) if np.issubdtype(self.a.dtype, np.integer) else v
        return Vec(list(self.a[i]))

    def __setitem__(self, i, v):
        if isinstance(i, tuple):
            i = tuple(int(k) for k in i)
        else:
            i = int(i)
        if self.n is None:
            self.a[i] = v
        else:
            self.a[i] = np.asarray(v.c if isinstance(v, Vec) else v, dtype=self.a.dtype)

    def fill(self, v):
        self.a[...] = v

    def copy_from(self, other):
        self.a[...] = other.a

    def to_numpy(self):
        return self.a.copy()

    def from_numpy(self, arr):
        self.a[...] = arr

    @property
    def shape(self):
        return self.a.shape if self.n is None else self.a.shape[:-1]


def field(dtype, shape=(), **kw):
    t = dtype.np if isinstance(dtype, _Type) else dtype
    return Field(np.zeros(shape, dtype=t))


class _VectorNS:
    @staticmethod
    def field(n, dtype, shape=(), **kw):
        t = dtype.np if isinstance(dtype, _Type) else dtype
        shape = (shape,) if np.isscalar(shape) else tuple(shape)
        return Field(np.zeros(shape + (n,), dtype=t), n)

    def __call__(self, comps, dt=None):
        comps = list(comps)
        if all(isinstance(c, int) for c in comps):
            return Vec(comps)
        return Vec([_F(c) for c in comps])


Vector = _VectorNS()
Matrix = Mat


class _PrefixSumExecutor:
    """ti.algorithms.PrefixSumExecutor: inclusive prefix sum in place."""

    def __init__(self, n):
        self.n = n

    def run(self, f):
        f.a[...] = np.cumsum(f.a, dtype=np.int64).astype(f.a.dtype)


algorithms = _pytypes.SimpleNamespace(PrefixSumExecutor=_PrefixSumExecutor)


def ndrange(*dims):
    """ti.ndrange: ascending indices (tuples for more than one dimension)."""
    import itertools

    rs = [range(d) if np.isscalar(d) else range(d[0], d[1]) for d in dims]
    return rs[0] if len(rs) == 1 else itertools.product(*rs)
types = _pytypes.SimpleNamespace(ndarray=template, template=template, vector=lambda *a, **k: None,
                                 matrix=lambda *a, **k: None)


f32 = float32
i32 = int32
u32 = uint32
u64 = uint64
i64 = int64


def install():
    """Register this module as ``taichi`` for the imports that follow."""
    mod = sys.modules[__name__]
    sys.modules["taichi"] = mod
    return mod
