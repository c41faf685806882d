"""A CPU emulator of the small part of the NVIDIA Warp API that the reference MPM backend uses.

warp-lang (pinned as 1.18.0 by the reference's add-on manifest, ``>=1.18`` in its pyproject) is not
installed here and cannot be. Installing this module as ``sys.modules["warp"]`` lets the reference's own
``mpm_core/backends/warp/{kernels,colliders,solver}.py`` import and run unchanged on the CPU, one kernel
thread at a time, so that their outputs can be saved as golden fixtures. Only the fixture generator
(``make_golden.py`` beside this file) uses it; nothing in the package or in the tests imports it.

Arithmetic model: every kernel value is IEEE float32 (numpy ``float32``), operations run in source order
and matrix products are spelled out term by term, so no BLAS reassociation or FMA contraction creeps in.
Kernel threads run sequentially in thread-id order, which makes float atomics deterministic.

Warp's own built-ins that the reference calls are restated here from published methods, not from Warp:
  * ``svd3``: singular value decomposition with rotation factors U, V (det +1), singular values sorted
    in decreasing order and the sign of det(F) carried by the last one, the convention of McAdams et al.
    2011 ("Computing the SVD of 3x3 matrices with minimal branching ..."). Computed in float64 with LAPACK
    and rounded to float32.
  * mesh queries: exact closest point on a triangle (Ericson, Real-Time Collision Detection, 5.1.5) by
    brute force over all triangles; inside/outside sign from the angle-weighted pseudonormal of the
    closest feature (Baerentzen and Aanaes 2005).
  * ``quat_slerp``: q0 (q0^-1 q1)^s; ``inverse``: float64 LAPACK inverse rounded to float32.
These are the parts of the golden fixtures that are not pinned to Warp itself.
"""

from __future__ import annotations

import builtins
import math
from types import SimpleNamespace

import numpy as np

f32 = np.float32

config = SimpleNamespace(quiet=True)


def init() -> None:
    pass


def get_preferred_device() -> str:
    return "cpu"


def get_cuda_device_count() -> int:
    return 0


def constant(x):
    return x


# -- value types -------------------------------------------------------------------------------------------


class Mat:
    """Square float32 matrix with Warp's operator meaning: ``*`` is the matrix product."""

    __array_ufunc__ = None  # make numpy defer to our reflected operators

    def __init__(self, a):
        self.a = np.array(a, dtype=f32)

    def copy(self) -> Mat:
        return Mat(self.a.copy())

    def __getitem__(self, ij):
        return self.a[ij]

    def __add__(self, o):
        return Mat(self.a + o.a)

    def __sub__(self, o):
        return Mat(self.a - o.a)

    def __neg__(self):
        return Mat(-self.a)

    def __truediv__(self, s):
        return Mat(self.a / f32(s))

    def __mul__(self, o):
        if isinstance(o, Mat):
            n = self.a.shape[0]
            out = self.a[:, 0:1] * o.a[0:1, :]
            for k in range(1, n):
                out = out + self.a[:, k:k + 1] * o.a[k:k + 1, :]
            return Mat(out)
        if isinstance(o, np.ndarray) and o.ndim == 1:
            out = self.a[:, 0] * o[0]
            for k in range(1, self.a.shape[0]):
                out = out + self.a[:, k] * o[k]
            return out.astype(f32)
        return Mat(self.a * f32(o))

    def __rmul__(self, s):
        return Mat(f32(s) * self.a)


def _vec_ctor(n, dtype):
    def ctor(*args):
        if len(args) == 0:
            return np.zeros(n, dtype)
        if len(args) == 1:
            a = np.asarray(args[0])
            if a.ndim == 0:
                return np.full(n, args[0], dtype)
            return np.array(a, dtype).reshape(n)
        return np.array(args, dtype)
    ctor.width = n
    ctor.np_dtype = dtype
    return ctor


vec3 = _vec_ctor(3, f32)
vec4 = _vec_ctor(4, f32)
vec3i = _vec_ctor(3, np.int32)
quat = _vec_ctor(4, f32)


def _mat_ctor(n):
    def ctor(*args):
        if len(args) == 0:
            return Mat(np.zeros((n, n), f32))
        if len(args) == 1:
            return Mat(np.asarray(args[0], f32).reshape(n, n))
        return Mat(np.array(args, f32).reshape(n, n))
    ctor.width = n
    return ctor


mat33 = _mat_ctor(3)
mat44 = _mat_ctor(4)


class uint64:  # noqa: N801 - Warp's spelling
    pass


def struct(cls):
    """Plain attribute record with Warp's zero defaults for vector/matrix/quaternion fields."""
    fields = dict(cls.__annotations__)

    class Record:
        __slots__ = tuple(fields)

        def __init__(self):
            for name, t in fields.items():
                setattr(self, name, t())

    Record.__name__ = cls.__name__
    Record.fields = fields
    return Record


# -- arrays --------------------------------------------------------------------------------------------------


def _np_dtype(dtype):
    if dtype is float:
        return f32, ()
    if dtype is int:
        return np.int32, ()
    if dtype is uint64:
        return np.uint64, ()
    if dtype in (vec3, vec4, vec3i, quat):
        return dtype.np_dtype, (dtype.width,)
    if dtype in (mat33, mat44):
        return f32, (dtype.width, dtype.width)
    return object, ()


class Array:
    """Host-resident Warp array; element reads return copies (Warp values are passed by value)."""

    def __init__(self, data, dtype):
        self.dtype = dtype
        self.data = data

    @property
    def shape(self):
        t = _np_dtype(self.dtype)[1]
        return self.data.shape[:self.data.ndim - len(t)] if t else self.data.shape

    def __len__(self):
        return self.shape[0]

    def __getitem__(self, idx):
        v = self.data[idx]
        if self.dtype in (mat33, mat44):
            return Mat(v.copy())
        if isinstance(v, np.ndarray):
            return v.copy()
        return v

    def __setitem__(self, idx, value):
        self.data[idx] = value.a if isinstance(value, Mat) else value

    def numpy(self) -> np.ndarray:
        return self.data.copy()

    def zero_(self) -> None:
        self.data[...] = 0


def array(data=None, dtype=float, device=None, shape=None):  # noqa: ARG001 - device is ignored on the CPU
    if data is None:  # used as a type annotation in a kernel signature
        return ("array", dtype)
    npt, tail = _np_dtype(dtype)
    if isinstance(data, Array):
        data = data.data
    if npt is object:
        buf = np.empty(len(data), object)
        for i, d in enumerate(data):
            buf[i] = d
        return Array(buf, dtype)
    if isinstance(data, (list, tuple)) and len(data) and isinstance(data[0], Mat):
        data = [d.a for d in data]
    a = np.array(data, npt)
    if a.size == 0:
        a = a.reshape((0,) + tail)
    else:
        a = a.reshape((-1,) + tail)
    return Array(a, dtype)


def array3d(dtype=float):
    return ("array3d", dtype)


def zeros(shape, dtype=float, device=None):  # noqa: ARG001
    npt, tail = _np_dtype(dtype)
    shape = (shape,) if isinstance(shape, int) else tuple(shape)
    return Array(np.zeros(shape + tail, npt), dtype)


def empty(shape, dtype=float, device=None):
    return zeros(shape, dtype, device)


def copy(dest: Array, src: Array, dest_offset: int = 0, src_offset: int = 0, count: int = 0) -> None:
    n = count or len(src)
    dest.data[dest_offset:dest_offset + n] = src.data[src_offset:src_offset + n]


# `wp.array(dtype=...)` is also used as a type annotation in kernel signatures; the call above serves both.


# -- kernels -------------------------------------------------------------------------------------------------

_tid = [0]


def tid():
    return _tid[0]


def _copy_value(a):
    if isinstance(a, Mat):
        return a.copy()
    if isinstance(a, np.ndarray):
        return a.copy()
    return a


def func(fn):
    def wrapped(*args):
        return fn(*(_copy_value(a) for a in args))
    wrapped.__name__ = fn.__name__
    return wrapped


class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.__name__ = fn.__name__


def kernel(fn):
    return Kernel(fn)


def _scalar_arg(a):
    if isinstance(a, bool):
        return int(a)
    if isinstance(a, float):
        return f32(a)
    if isinstance(a, (np.floating,)):
        return f32(a)
    return a


def launch(k: Kernel, dim, inputs=(), device=None):  # noqa: ARG001
    args = [_scalar_arg(a) for a in inputs]
    if isinstance(dim, int):
        for t in range(dim):
            _tid[0] = t
            k.fn(*args)
    else:
        for t in np.ndindex(*dim):
            _tid[0] = tuple(int(i) for i in t)
            k.fn(*args)


# -- scalar built-ins ----------------------------------------------------------------------------------------


def floor(x):
    return f32(np.floor(f32(x)))


def ceil(x):
    return f32(np.ceil(f32(x)))


def round(x):  # noqa: A001 - Warp's name; halfway cases go away from zero
    x = f32(x)
    return f32(math.copysign(math.floor(builtins.abs(float(x)) + 0.5), float(x)))


def exp(x):
    return f32(np.exp(f32(x)))


def log(x):
    return f32(np.log(f32(x)))


def sqrt(x):
    return f32(np.sqrt(f32(x)))


def abs(x):  # noqa: A001
    return f32(np.abs(f32(x)))


def _ints(*xs):
    return all(isinstance(x, (int, np.integer)) and not isinstance(x, bool) for x in xs)


def min(a, b):  # noqa: A001 - integer arguments give an integer, as in Warp
    if _ints(a, b):
        return builtins.min(int(a), int(b))
    a, b = f32(a), f32(b)
    return a if a < b else b


def max(a, b):  # noqa: A001
    if _ints(a, b):
        return builtins.max(int(a), int(b))
    a, b = f32(a), f32(b)
    return a if a > b else b


def clamp(x, lo, hi):
    if _ints(x, lo, hi):
        return builtins.min(builtins.max(int(x), int(lo)), int(hi))
    x, lo, hi = f32(x), f32(lo), f32(hi)
    return lo if x < lo else (hi if x > hi else x)


def isfinite(x):
    return bool(np.isfinite(x))


def where(cond, a, b):
    return a if cond else b


def atomic_add(arr: Array, *idx_value):
    idx, value = tuple(int(i) for i in idx_value[:-1]), idx_value[-1]
    arr.data[idx] = arr.data[idx] + value


def atomic_max(arr: Array, *idx_value):
    idx, value = tuple(int(i) for i in idx_value[:-1]), idx_value[-1]
    if value > arr.data[idx]:  # a NaN never wins the comparison
        arr.data[idx] = value


# -- vector / matrix built-ins -------------------------------------------------------------------------------


def dot(a, b):
    a = np.asarray(a, f32)
    b = np.asarray(b, f32)
    s = a[0] * b[0]
    for i in range(1, len(a)):
        s = s + a[i] * b[i]
    return f32(s)


def length(a):
    return f32(np.sqrt(dot(a, a)))


def normalize(a):
    n = length(a)
    return (np.asarray(a, f32) / n).astype(f32) if n > 0 else np.zeros_like(np.asarray(a, f32))


def cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], f32)


def outer(a, b):
    return Mat(np.asarray(a, f32)[:, None] * np.asarray(b, f32)[None, :])


def diag(v):
    return Mat(np.diag(np.asarray(v, f32)))


def transpose(m: Mat) -> Mat:
    return Mat(m.a.T.copy())


def identity(n=3, dtype=float):  # noqa: ARG001
    return Mat(np.eye(n, dtype=f32))


def inverse(m: Mat) -> Mat:
    return Mat(np.linalg.inv(m.a.astype(np.float64)).astype(f32))


def transform_point(m: Mat, p):
    a = m.a
    out = a[:3, 0] * p[0] + a[:3, 1] * p[1] + a[:3, 2] * p[2]
    return (out + a[:3, 3]).astype(f32)


def transform_vector(m: Mat, v):
    a = m.a
    return (a[:3, 0] * v[0] + a[:3, 1] * v[1] + a[:3, 2] * v[2]).astype(f32)


def svd3(A: Mat, U: Mat, sig, V: Mat) -> None:
    """Outputs by mutation, like Warp's: U, V rotations, sig descending with sign(det A) on sig[2]."""
    u, s, vt = np.linalg.svd(A.a.astype(np.float64))
    v = vt.T
    if np.linalg.det(u) < 0:
        u[:, 2] = -u[:, 2]
        s[2] = -s[2]
    if np.linalg.det(v) < 0:
        v[:, 2] = -v[:, 2]
        s[2] = -s[2]
    U.a[...] = u
    V.a[...] = v
    sig[...] = s


# -- quaternions (x, y, z, w) ---------------------------------------------------------------------------------


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw,
                     aw * bw - ax * bx - ay * by - az * bz])


def quat_slerp(q0, q1, s):
    q0 = np.asarray(q0, np.float64)
    q1 = np.asarray(q1, np.float64)
    d = _qmul(q0 * np.array([-1, -1, -1, 1]), q1)  # q0^-1 q1 for unit q0
    w = np.clip(d[3], -1.0, 1.0)
    angle = 2.0 * math.acos(w)
    axis_n = np.linalg.norm(d[:3])
    if axis_n < 1e-12:
        return q0.astype(f32)
    axis = d[:3] / axis_n
    h = 0.5 * float(s) * angle
    step = np.array([*(axis * math.sin(h)), math.cos(h)])
    return _qmul(q0, step).astype(f32)


def quat_to_matrix(q) -> Mat:
    x, y, z, w = (float(c) for c in q)
    return Mat(np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]))


# -- meshes -----------------------------------------------------------------------------------------------------

_meshes: dict[int, Mesh] = {}


class Mesh:
    def __init__(self, points: Array, indices: Array):
        self.points = np.asarray(points.data, np.float64).reshape(-1, 3)
        self.tris = np.asarray(indices.data, np.int64).reshape(-1, 3)
        self.id = len(_meshes) + 1
        _meshes[self.id] = self
        p = self.points[self.tris]
        n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        self.face_n = n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-300)
        # edge pseudonormals: sum of the unit normals of the faces sharing the edge
        self.edge_n: dict[tuple[int, int], np.ndarray] = {}
        for f, t in enumerate(self.tris):
            for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
                key = (builtins.min(a, b), builtins.max(a, b))
                self.edge_n[key] = self.edge_n.get(key, 0) + self.face_n[f]
        # vertex pseudonormals: incident face normals weighted by the face angle at the vertex
        self.vert_n = np.zeros_like(self.points)
        for f, t in enumerate(self.tris):
            for c in range(3):
                v0, v1, v2 = p[f, c], p[f, (c + 1) % 3], p[f, (c + 2) % 3]
                e1, e2 = v1 - v0, v2 - v0
                cosang = np.dot(e1, e2) / max(np.linalg.norm(e1) * np.linalg.norm(e2), 1e-300)
                self.vert_n[t[c]] += math.acos(float(np.clip(cosang, -1.0, 1.0))) * self.face_n[f]


def closest_point_triangles(p, a, b, c):
    """Vectorised Ericson 5.1.5. Returns (closest points (T,3), barycentrics (T,3), region codes (T,)).

    Region codes: 0 face interior, 1/2/3 vertex a/b/c, 4 edge ab, 5 edge bc, 6 edge ca.
    """
    T = len(a)
    ab, ac, ap = b - a, c - a, p - a
    d1 = np.einsum("ij,ij->i", ab, ap)
    d2 = np.einsum("ij,ij->i", ac, ap)
    bp = p - b
    d3 = np.einsum("ij,ij->i", ab, bp)
    d4 = np.einsum("ij,ij->i", ac, bp)
    cp = p - c
    d5 = np.einsum("ij,ij->i", ab, cp)
    d6 = np.einsum("ij,ij->i", ac, cp)
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    bary = np.zeros((T, 3))
    region = np.full(T, -1)
    done = np.zeros(T, bool)

    def put(mask, w, code):
        nonlocal done
        m = mask & ~done
        bary[m] = w[m] if w.ndim == 2 else w
        region[m] = code
        done |= m

    one = np.ones(T)
    zero = np.zeros(T)
    put((d1 <= 0) & (d2 <= 0), np.stack([one, zero, zero], 1), 1)
    put((d3 >= 0) & (d4 <= d3), np.stack([zero, one, zero], 1), 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        v_ab = d1 / (d1 - d3)
        put((vc <= 0) & (d1 >= 0) & (d3 <= 0), np.stack([1 - v_ab, v_ab, zero], 1), 4)
        put((d6 >= 0) & (d5 <= d6), np.stack([zero, zero, one], 1), 3)
        w_ac = d2 / (d2 - d6)
        put((vb <= 0) & (d2 >= 0) & (d6 <= 0), np.stack([1 - w_ac, zero, w_ac], 1), 6)
        w_bc = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        put((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), np.stack([zero, 1 - w_bc, w_bc], 1), 5)
        denom = 1.0 / (va + vb + vc)
        v = vb * denom
        w = vc * denom
        put(np.ones(T, bool), np.stack([1 - v - w, v, w], 1), 0)
    pts = bary[:, 0:1] * a + bary[:, 1:2] * b + bary[:, 2:3] * c
    return pts, bary, region


def _pseudonormal(mesh: Mesh, face: int, region: int) -> np.ndarray:
    t = mesh.tris[face]
    if region == 0:
        return mesh.face_n[face]
    if region in (1, 2, 3):
        return mesh.vert_n[t[region - 1]]
    a, b = {4: (t[0], t[1]), 5: (t[1], t[2]), 6: (t[2], t[0])}[region]
    return mesh.edge_n[(builtins.min(a, b), builtins.max(a, b))]


def mesh_query_point_sign_normal(mesh_id, point, max_dist, epsilon=1e-3):  # noqa: ARG001
    mesh = _meshes[int(mesh_id)]
    p = np.asarray(point, np.float64)
    tri = mesh.points[mesh.tris]
    cps, bary, region = closest_point_triangles(p, tri[:, 0], tri[:, 1], tri[:, 2])
    d2 = ((cps - p) ** 2).sum(1)
    face = int(np.argmin(d2))
    if d2[face] > float(max_dist) ** 2:
        return SimpleNamespace(result=False, sign=f32(1.0), face=0, u=f32(0), v=f32(0))
    n = _pseudonormal(mesh, face, int(region[face]))
    sign = 1.0 if np.dot(p - cps[face], n) >= 0.0 else -1.0
    return SimpleNamespace(result=True, sign=f32(sign), face=face, u=f32(bary[face, 0]), v=f32(bary[face, 1]))


def mesh_eval_position(mesh_id, face, u, v):
    mesh = _meshes[int(mesh_id)]
    a, b, c = mesh.points[mesh.tris[face]]
    u, v = float(u), float(v)
    return (u * a + v * b + (1.0 - u - v) * c).astype(f32)


def mesh_eval_face_normal(mesh_id, face):
    return _meshes[int(mesh_id)].face_n[face].astype(f32)
