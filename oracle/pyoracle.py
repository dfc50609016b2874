"""numpy front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py``; never by the product.  Wraps ``oracle/_build/liboracle.so`` (a CPU
restatement of the reference algorithms, see oracle.cpp for the file:line each
function follows) and provides :class:`OracleSolver`, which strings the pieces
together exactly like ``Solver.forward`` (``framework/physics/XPBD.py:443-469``)
with the iteration and rebuild options of the GPU solver.

Parity status: pinned against the reference's own source, executed on the CPU
through a numpy stand-in for the Taichi API (tests/golden/taichi_standin.py,
tests/golden/make_reference_vectors.py -> tests/golden/reference_vectors.npz,
checked by tests/test_reference_vectors.py): classification, distances, Morton
codes, the cell BVH and the substep kernels bit for bit; contact records equal,
contact gradients, positions and velocities to float32 rounding.  Known-answer
and brute-force checks in tests/ cover the rest.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

P = C.c_void_p
I = C.c_int
F = C.c_float

_SIGS = {
    "or_predict": [I, P, P, P, P, F, F, F, F, I],
    "or_spring_sweep": [I, I, I, P, P, P, P, P, P, P, P, F, F, I, P, P, I],
    "or_spring_sweep_gather": [I, P, P, P, P, P, P, F, F, I, P, I],
    "or_velocity_update": [I, P, P, P, P, F, F, I],
    "or_face_aabbs": [I, P, P, F, P, P],
    "or_scene_aabb": [I, P, F, P],
    "or_morton3d": [I, P, P],
    "or_face_morton": [I, P, P, P, P, P],
    "or_radix_sort": [I, P, P, I],
    "or_karras": [I, P, I, P, P, P, P, P],
    "or_cell_bvh_init": [P, P, P, P, P, P, P],
    "or_cell_bvh_build": [I, P, P, P, P, P, P, P, P, P, P, P, P],
    "or_cell_bvh_traverse": [I, P, P, P, P, P, P, P, P, P, P, P, P, P, I, P, P, P],
    "or_face_bvh_refit": [I, P, P, P, P, P, P, P, P],
    "or_face_bvh_traverse": [I, I, P, P, P, P, P, P, P, I, P, P, P],
    "or_residual": [I, P, P, P, P],
    "or_sewing_step": [I, P, P, P, P, P, F],
    "or_velocity_contacts": [I, I, P, P, I, P, P, P, P, P, P, P, P, P, F, P],
    "or_warm_features": [I, P, P, P, P, P, P, P, F, F, F, F, P],
    "or_collision_sweep": [I, I, P, P, P, P, P, P, F, F, F, I, P, P, P, P, P, P, P, P, P, P, P, P, P, I, I],
    "or_edge_edge_classify": [I, P, F, P, P, P],
    "or_point_triangles": [I, P, P, P, P],
    "or_contact_cull": [I, P, F, P],
    "or_edge_edge_sweep": [I, P, P, P, P, P, P, P, P, F, F, I, P, P, P, P, P, P, P, P, P, P, P, I],
    "or_point_triangle": [P, P, P],
    "or_color_edges": [I, I, P, I, P, P, P],
    "or_gs_sweep": [I, P, P, P, F, F],
    "or_version": [],
}


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


NUM_CELLS = 32 * 32 * 32


# ---- cloth ------------------------------------------------------------------
def predict(x4, v4, fixed, dt, g, nthreads=1):
    y4 = np.empty_like(x4)
    lib().or_predict(x4.shape[0], _p(x4), _p(v4), _p(fixed), _p(y4), dt, g[0], g[1], g[2], nthreads)
    return y4


def spring_sweep(x4, y4, fixed, m_inv, edges, l0, bend, bl0, k_spring, k_bend, nthreads=1, bend_on_y=0):
    """One Jacobi sweep; updates y4 in place."""
    V = x4.shape[0]
    dx = np.empty(3 * V, np.float32)
    nc = np.empty(V, np.float32)
    lib().or_spring_sweep(V, edges.shape[0], bend.shape[0], _p(x4), _p(y4), _p(fixed), _p(m_inv), _p(edges),
                          _p(l0), _p(bend), _p(bl0), k_spring, k_bend, int(bend_on_y), _p(dx), _p(nc), nthreads)
    return y4


def spring_sweep_gather(x4, y4, fixed, m_inv, ptr, adj, k_spring, k_bend, nthreads=1, bend_on_y=0):
    """spring_sweep as a per-vertex gather over adjacency(): the serial sweep's
    result bit for bit at any thread count.  Updates y4 in place."""
    V = x4.shape[0]
    scratch = np.empty((V, 4), np.float32)
    lib().or_spring_sweep_gather(V, _p(x4), _p(y4), _p(fixed), _p(m_inv), _p(i32(ptr)), _p(i32(adj)), k_spring,
                                 k_bend, int(bend_on_y), _p(scratch), nthreads)
    return y4


def velocity_update(x4, y4, v4, fixed, damping, dt, nthreads=1):
    lib().or_velocity_update(x4.shape[0], _p(x4), _p(y4), _p(v4), _p(fixed), damping, dt, nthreads)


def face_aabbs(p4, faces, padding):
    F_ = faces.shape[0]
    mn = np.empty((F_, 4), np.float32)
    mx = np.empty((F_, 4), np.float32)
    lib().or_face_aabbs(F_, _p(p4), _p(i32(faces)), padding, _p(mn), _p(mx))
    return mn, mx


def scene_aabb(p4, padding):
    out = np.empty(6, np.float32)
    lib().or_scene_aabb(p4.shape[0], _p(p4), padding, _p(out))
    return out


# ---- LBVH -------------------------------------------------------------------
def morton3d(xyz):
    xyz = f32(xyz, (-1, 3))
    out = np.empty(xyz.shape[0], np.int32)
    lib().or_morton3d(xyz.shape[0], _p(xyz), _p(out))
    return out


def face_morton(mn4, mx4, box6):
    n = mn4.shape[0]
    codes = np.empty(n, np.int32)
    ids = np.empty(n, np.int32)
    lib().or_face_morton(n, _p(mn4), _p(mx4), _p(f32(box6)), _p(codes), _p(ids))
    return codes, ids


def radix_sort(keys, vals, bits):
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    v = i32(vals).copy()
    lib().or_radix_sort(k.shape[0], _p(k), _p(v), bits)
    return k, v


def karras(codes, tie=0):
    codes = i32(codes)
    n = codes.shape[0]
    ca = np.zeros(max(n - 1, 1), np.int32)
    cb = np.zeros_like(ca)
    rl = np.zeros_like(ca)
    rr = np.zeros_like(ca)
    par = np.zeros(2 * n - 1, np.int32)
    lib().or_karras(n, _p(codes), tie, _p(ca), _p(cb), _p(rl), _p(rr), _p(par))
    return ca[: n - 1], cb[: n - 1], rl[: n - 1], rr[: n - 1], par


class CellBVH:
    """Oracle of LBVH_CELL (lbvh_cell.py:16-714)."""

    def __init__(self):
        n = NUM_CELLS
        self.codes = np.empty(n, np.int32)
        self.ids = np.empty(n, np.int32)
        self.child_a = np.empty(n - 1, np.int32)
        self.child_b = np.empty(n - 1, np.int32)
        self.range_l = np.empty(n - 1, np.int32)
        self.range_r = np.empty(n - 1, np.int32)
        self.parent = np.empty(2 * n - 1, np.int32)
        lib().or_cell_bvh_init(_p(self.codes), _p(self.ids), _p(self.child_a), _p(self.child_b), _p(self.range_l),
                               _p(self.range_r), _p(self.parent))

    def build(self, fmn4, fmx4, box6):
        F_ = fmn4.shape[0]
        N = 2 * NUM_CELLS - 1
        self.box6 = f32(box6).copy()
        self.fmn4, self.fmx4 = fmn4, fmx4
        self.sorted_face_ids = np.empty(max(F_, 1), np.int32)
        self.prefix = np.empty(NUM_CELLS, np.int32)
        self.num_faces = np.empty(N, np.int32)
        self.nmin4 = np.zeros((N, 4), np.float32)
        self.nmax4 = np.zeros((N, 4), np.float32)
        self.cell_size = np.empty(3, np.float32)
        lib().or_cell_bvh_build(F_, _p(fmn4), _p(fmx4), _p(self.box6), _p(self.child_a), _p(self.child_b),
                                _p(self.parent), _p(self.sorted_face_ids), _p(self.prefix), _p(self.num_faces),
                                _p(self.nmin4), _p(self.nmax4), _p(self.cell_size))
        self.sorted_face_ids = self.sorted_face_ids[:F_]

    def traverse(self, qmin4, qmax4, cap):
        Q = qmin4.shape[0]
        cand = np.full((Q, cap), -1, np.int32)
        num = np.zeros(Q, np.int32)
        status = np.zeros(1, np.int32)
        sfi = self.sorted_face_ids if self.sorted_face_ids.size else np.zeros(1, np.int32)
        lib().or_cell_bvh_traverse(Q, _p(qmin4), _p(qmax4), _p(self.cell_size), _p(self.box6), _p(self.child_a),
                                   _p(self.child_b), _p(self.num_faces), _p(self.nmin4), _p(self.nmax4),
                                   _p(self.prefix), _p(sfi), _p(self.fmn4), _p(self.fmx4), cap, _p(cand), _p(num),
                                   _p(status))
        return cand, num, int(status[0])


def query_boxes(p4, padding):
    p = f32(p4)[:, :3]
    pad = np.float32(padding)
    mn = np.zeros((p.shape[0], 4), np.float32)
    mx = np.zeros((p.shape[0], 4), np.float32)
    mn[:, :3] = p - pad
    mx[:, :3] = p + pad
    return mn, mx


class FaceBVH:
    """Oracle of the face-level LBVH (Morton -> radix sort -> Karras -> refit)."""

    def __init__(self, fmn4, fmx4, box6, tie=1):
        n = fmn4.shape[0]
        self.n = n
        codes, ids = face_morton(fmn4, fmx4, box6)
        self.codes_unsorted = codes
        k, v = radix_sort(codes.view(np.uint32), ids, 32)
        self.sorted_codes = k.view(np.int32)
        self.sorted_ids = v
        self.child_a, self.child_b, self.range_l, self.range_r, self.parent = karras(self.sorted_codes, tie)
        self.nmin4 = np.zeros((2 * n - 1, 4), np.float32)
        self.nmax4 = np.zeros((2 * n - 1, 4), np.float32)
        ca = self.child_a if n > 1 else np.zeros(1, np.int32)
        cb = self.child_b if n > 1 else np.zeros(1, np.int32)
        lib().or_face_bvh_refit(n, _p(self.sorted_ids), _p(fmn4), _p(fmx4), _p(ca), _p(cb), _p(self.parent),
                                _p(self.nmin4), _p(self.nmax4))

    def traverse(self, qmin4, qmax4, cap):
        Q = qmin4.shape[0]
        cand = np.full((Q, cap), -1, np.int32)
        num = np.zeros(Q, np.int32)
        status = np.zeros(1, np.int32)
        ca = self.child_a if self.n > 1 else np.zeros(1, np.int32)
        cb = self.child_b if self.n > 1 else np.zeros(1, np.int32)
        lib().or_face_bvh_traverse(self.n, Q, _p(qmin4), _p(qmax4), _p(ca), _p(cb), _p(self.sorted_ids),
                                   _p(self.nmin4), _p(self.nmax4), cap, _p(cand), _p(num), _p(status))
        return cand, num, int(status[0])


# ---- narrow phase -----------------------------------------------------------
def point_triangle(p, t0, t1, t2):
    buf = f32(np.concatenate([p, t0, t1, t2]))
    d = np.zeros(1, np.float32)
    g = np.zeros(12, np.float32)
    dt = lib().or_point_triangle(_p(buf), _p(d), _p(g))
    return dt, float(d[0]), g.reshape(4, 3)


def point_triangles(p12):
    """point_triangle over rows of 12 floats (p, t0, t1, t2): dtype, d, g[n, 4, 3]."""
    p12 = np.ascontiguousarray(f32(p12).reshape(-1, 12))
    n = p12.shape[0]
    dt = np.zeros(n, np.int32)
    d = np.zeros(n, np.float32)
    g = np.zeros((n, 12), np.float32)
    lib().or_point_triangles(n, _p(p12), _p(dt), _p(d), _p(g))
    return dt, d, g.reshape(n, 4, 3)


def collision_sweep(faces_dy, faces_st, y4, xs4, fixed, m_inv, dHat, compliance, cap, vt_st, vt_dy, tv_st,
                    want_pairs=False, nthreads=1, cull_d2=0.0, acc=None):
    """Narrow phase + update_dx; updates y4 in place.  vt_st etc. = (cand, num).
    cull_d2 > 0 skips pairs whose point-to-triangle-box squared distance
    exceeds it (the CUDA pair-list sweep's cull).  acc = (dx, nc) from
    :func:`edge_edge_sweep` of the same iteration, added to before update_dx."""
    Vd = y4.shape[0]
    Vs = xs4.shape[0] if xs4 is not None else 0
    if acc is None:
        dx = np.zeros(3 * Vd, np.int64)
        nc = np.zeros(Vd, np.int32)
    else:
        dx, nc = acc
    status = np.zeros(1, np.int32)
    pair = pair_g = pair_schur = pair_num = None
    if want_pairs:
        Q = 2 * Vd + Vs
        pair = np.zeros((Q, cap, 2), np.int32)
        pair_g = np.zeros((Q, cap, 4, 4), np.float32)
        pair_schur = np.zeros((Q, cap), np.float32)
        pair_num = np.zeros(Q, np.int32)
    fs = i32(faces_st) if faces_st is not None else np.zeros(3, np.int32)
    xs = xs4 if xs4 is not None else np.zeros((1, 4), np.float32)
    lib().or_collision_sweep(Vd, Vs, _p(i32(faces_dy)), _p(fs), _p(y4), _p(xs), _p(fixed), _p(m_inv), dHat,
                             compliance, cull_d2, cap, _p(vt_st[0]), _p(vt_st[1]), _p(vt_dy[0]), _p(vt_dy[1]),
                             _p(tv_st[0]), _p(tv_st[1]), _p(dx), _p(nc), _p(pair), _p(pair_g), _p(pair_schur),
                             _p(pair_num), _p(status), nthreads, 0 if acc is None else 1)
    out = {"status": int(status[0])}
    if want_pairs:
        out.update(pair=pair, pair_g=pair_g, pair_schur=pair_schur, pair_num=pair_num)
    return out


def edge_query_boxes(p4, edges, padding):
    """Edge boxes of the edge broad phase (XPBD.py:221-232): min / max of the two
    endpoints, minus / plus padding."""
    p = f32(p4)[:, :3]
    e = i32(edges).reshape(-1, 2)
    pad = np.float32(padding)
    mn = np.zeros((e.shape[0], 4), np.float32)
    mx = np.zeros((e.shape[0], 4), np.float32)
    mn[:, :3] = np.minimum(p[e[:, 0]], p[e[:, 1]]) - pad
    mx[:, :3] = np.maximum(p[e[:, 0]], p[e[:, 1]]) + pad
    return mn, mx


def edge_edge_classify(p12, dHat):
    """d_type_EE, squared distance and gradient of n quadruples (x0, x1 = edge 0,
    x2, x3 = edge 1): d = dHat unless dtype 8 with |x01 x x23| > 1e-3."""
    p12 = f32(p12).reshape(-1, 12)
    n = p12.shape[0]
    dt = np.zeros(n, np.int32)
    d = np.zeros(n, np.float32)
    g = np.zeros((n, 12), np.float32)
    lib().or_edge_edge_classify(n, _p(np.ascontiguousarray(p12)), np.float32(dHat), _p(dt), _p(d), _p(g))
    return dt, d, g.reshape(n, 4, 3)


def edge_edge_sweep(edges_dy, edges_st, face_edges_dy, face_edges_st, y4, xs4, fixed, m_inv, dHat, compliance, cap,
                    ee_st, ee_dy, dx, nc, want_pairs=False, nthreads=1):
    """Edge-edge terms of one iteration added to (dx, nc); ee_st / ee_dy =
    (cand, num) of the edge broad phase (ee_st None: no static mesh)."""
    e_dy = i32(edges_dy).reshape(-1, 2)
    Ed = e_dy.shape[0]
    status = np.zeros(1, np.int32)
    pair = pair_g = pair_schur = pair_num = None
    if want_pairs:
        pair = np.zeros((2 * Ed, cap, 2), np.int32)
        pair_g = np.zeros((2 * Ed, cap, 4, 4), np.float32)
        pair_schur = np.zeros((2 * Ed, cap), np.float32)
        pair_num = np.zeros(2 * Ed, np.int32)
    has_st = ee_st is not None
    e_st = i32(edges_st) if has_st else np.zeros(2, np.int32)
    fe_st = i32(face_edges_st) if has_st else np.zeros(3, np.int32)
    xs = xs4 if has_st else np.zeros((1, 4), np.float32)
    lib().or_edge_edge_sweep(Ed, _p(e_dy), _p(e_st), _p(i32(face_edges_dy)), _p(fe_st), _p(y4), _p(xs), _p(fixed),
                             _p(m_inv), np.float32(dHat), np.float32(compliance), cap,
                             _p(ee_st[0]) if has_st else None, _p(ee_st[1]) if has_st else None, _p(ee_dy[0]),
                             _p(ee_dy[1]), _p(dx), _p(nc), _p(pair), _p(pair_g), _p(pair_schur), _p(pair_num),
                             _p(status), nthreads)
    out = {"status": int(status[0])}
    if want_pairs:
        out.update(pair=pair, pair_g=pair_g, pair_schur=pair_schur, pair_num=pair_num)
    return out


def adjacency(n_verts, edges, l0, bend, bl0):
    """Vertex-centric CSR of the constraints in ascending constraint index
    (springs 0..E-1, then bending pairs): entry = (neighbour | bit 31 for a
    bending pair, bits of the rest length).  The order in which a serial run of
    solve_spring_constraints_x (XPBD.py:141-184) meets a vertex's constraints."""
    edges = i32(edges).reshape(-1, 2)
    bend = i32(bend).reshape(-1, 2)
    E, B = edges.shape[0], bend.shape[0]
    a = np.concatenate([edges[:, 0], bend[:, 0], edges[:, 1], bend[:, 1]]).astype(np.int64)
    nb = np.concatenate([edges[:, 1], bend[:, 1], edges[:, 0], bend[:, 0]]).astype(np.int64)
    cid = np.concatenate([np.arange(E + B), np.arange(E + B)])
    rest = np.concatenate([f32(l0), f32(bl0)])
    order = np.lexsort((cid, a))
    a, nb, cid = a[order], nb[order], cid[order]
    ptr = np.zeros(n_verts + 1, np.int32)
    ptr[1:] = np.cumsum(np.bincount(a, minlength=n_verts))
    adj = np.empty((a.shape[0], 2), np.int32)
    adj[:, 0] = np.where(cid >= E, nb | 0x80000000, nb).astype(np.int64).astype(np.uint32).view(np.int32)
    adj[:, 1] = rest[cid].view(np.int32)
    return ptr, adj


def contact_cull(p12, cull_d2):
    """The pair-list sweep's two cull stages on n point-triangle quadruples
    (n x 12 floats: point, then the triangle): 1 = box distance, 2 =
    separating axes, 0 = kept."""
    p = f32(np.asarray(p12, np.float32).reshape(-1, 12))
    out = np.zeros(p.shape[0], np.int32)
    lib().or_contact_cull(p.shape[0], _p(p), float(cull_d2), _p(out))
    return out


def velocity_contacts(faces_dy, faces_st, cap, rec, v4, vs4, fixed, m_inv, m_inv_st, mu):
    """solve_constraints_v over pair records rec (the dict collision_sweep
    returns with want_pairs); updates v4 in place."""
    Vd = v4.shape[0]
    Vs = vs4.shape[0] if vs4 is not None else 0
    fs = i32(faces_st) if faces_st is not None else np.zeros(3, np.int32)
    vs = vs4 if vs4 is not None else np.zeros((1, 4), np.float32)
    ms = f32(m_inv_st) if m_inv_st is not None else np.zeros(1, np.float32)
    status = np.zeros(1, np.int32)
    lib().or_velocity_contacts(Vd, Vs, _p(i32(faces_dy)), _p(fs), cap, _p(rec["pair"]), _p(rec["pair_g"]),
                               _p(rec["pair_schur"]), _p(rec["pair_num"]), _p(v4), _p(vs), _p(f32(fixed)),
                               _p(f32(m_inv)), _p(ms), float(mu), _p(status))
    return int(status[0])


def sewing_step(y4, fixed, sewn, sptr, partner, k):
    """Sewing constraints + update_dx on y4 (in place)."""
    lib().or_sewing_step(int(len(sewn)), _p(i32(sewn)), _p(i32(sptr)), _p(i32(partner)), _p(y4), _p(f32(fixed)),
                         float(k))
    return y4


def residual(p4, ptr, adj):
    """The CUDA library's constraint residual {S, n, sqrt(S/n)} in its exact
    summation order (float per vertex and block, FP64 across blocks); the
    reference defines no residual."""
    out = np.zeros(3, np.float64)
    lib().or_residual(int(ptr.shape[0] - 1), _p(f32(p4)), _p(i32(ptr)), _p(i32(adj)), _p(out))
    return out


def constraint_residual(p4, edges, l0, bend, bl0):
    """residual() of positions p4 over the springs and bending pairs."""
    ptr, adj = adjacency(p4.shape[0], edges, l0, bend, bl0)
    return residual(p4, ptr, adj)


def system_energy(x4, v4, m_inv, ptr, adj, ks, kb, g):
    """Kinetic, gravitational and elastic energy in float64 (the library's
    sx_system_energy; no counterpart in the reference): masses 1/m_inv where
    m_inv > 0, elastic 1/2 k C^2 per constraint with every constraint seen from
    both adjacency endpoints (1/4 per entry), k = kb for bending entries (bit 31
    of the neighbour word) else ks."""
    x = x4[:, :3].astype(np.float64)
    v = v4[:, :3].astype(np.float64)
    mi = m_inv.astype(np.float32)
    has = mi > 0
    m = np.zeros(x.shape[0])
    m[has] = 1.0 / mi[has].astype(np.float64)
    ek = 0.5 * float((m * (v * v).sum(1)).sum())
    eg = -float((m * (x @ np.asarray(g, np.float32).astype(np.float64))).sum())  # g arrives as float32
    ptr = np.asarray(ptr, np.int64)
    a = np.asarray(adj, np.int32).reshape(-1, 2)
    owner = np.repeat(np.arange(x.shape[0]), np.diff(ptr))
    nbr = a[:, 0] & 0x7FFFFFFF
    rest = a[:, 1].view(np.float32).astype(np.float64)
    C = np.linalg.norm(x[owner] - x[nbr], axis=1) - rest
    k = np.where(a[:, 0] < 0, kb, ks)
    ee = float((0.25 * k * C * C).sum())
    return ek, eg, ee


# ---- learned warm start (no counterpart in the reference) --------------------
# Parameter blob (FP32, 6792): W1[64][32] | b1[64] | W2[64][64] | b2[64] |
# W3[8][64] | b3[8]; the BF16 copy holds the three weight matrices.
MLP_SHAPES = [("W1", (64, 32)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (8, 64)), ("b3", (8,))]
MLP_PARAMS = sum(int(np.prod(s)) for _, s in MLP_SHAPES)


def mlp_unpack(p, dtype=np.float32):
    out, o = {}, 0
    for name, shape in MLP_SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype).reshape(shape)
        o += n
    return out


def bf16_round(a):
    """float32 -> nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def bf16_to_f32(u16):
    return (np.asarray(u16, np.uint16).astype(np.uint32) << 16).view(np.float32)


def warm_features(x4, y4, c4, fixed, ptr, adj, Lref, g, dt):
    """BF16 feature rows [V, 32] (uint16) of the CUDA warm_features_kernel."""
    V = y4.shape[0]
    feat = np.zeros((V, 32), np.uint16)
    lib().or_warm_features(V, _p(f32(x4)), _p(f32(y4)), _p(f32(c4)), _p(f32(fixed)), _p(i32(ptr)), _p(i32(adj)),
                           _p(f32(Lref)), float(g[0]), float(g[1]), float(g[2]), float(dt), _p(feat))
    return feat


def _silu(z):
    return z / (np.float32(1) + np.exp(-z))


def _silu_grad(z):
    s = np.float32(1) / (np.float32(1) + np.exp(-z))
    return s + z * (s * (np.float32(1) - s))


def mlp_forward(feat_u16, params, keep=False):
    """BF16 operands, FP32 accumulation, BF16 hidden activations."""
    P = mlp_unpack(params)
    X = bf16_to_f32(feat_u16)
    W1, W2, W3 = (bf16_round(P[k]) for k in ("W1", "W2", "W3"))
    Z1 = (X @ W1.T + P["b1"]).astype(np.float32)
    H1 = bf16_round(_silu(Z1))
    Z2 = (H1 @ W2.T + P["b2"]).astype(np.float32)
    H2 = bf16_round(_silu(Z2))
    O = (H2 @ W3.T + P["b3"]).astype(np.float32)
    if keep:
        return O, (X, Z1, H1, Z2, H2, W1, W2, W3)
    return O


def mlp_gradients(feat_u16, target4, params):
    """Loss = sum over rows of mask * |O[:3] - t|^2 / n_valid and its gradient,
    with the CUDA kernels' rounding points (BF16 dO, dZ2, dZ1 operands)."""
    O, (X, Z1, H1, Z2, H2, W1, W2, W3) = mlp_forward(feat_u16, params, keep=True)
    T = np.asarray(target4, np.float32)
    mask = T[:, 3:4]
    n_valid = max(int(np.count_nonzero(mask)), 1)
    E = np.zeros_like(O)
    E[:, :3] = mask * (O[:, :3] - T[:, :3])
    loss = float(np.sum(E[:, :3] * (O[:, :3] - T[:, :3]), dtype=np.float64))
    dO = (np.float32(2.0) * np.float32(1.0 / n_valid)) * E
    dOb = bf16_round(dO)
    dZ2 = (dOb @ W3).astype(np.float32) * _silu_grad(Z2)
    dZ2b = bf16_round(dZ2)
    dZ1 = (dZ2b @ W2).astype(np.float32) * _silu_grad(Z1)
    dZ1b = bf16_round(dZ1)
    g = {"W1": dZ1b.T @ X, "b1": dZ1.sum(0), "W2": dZ2b.T @ H1, "b2": dZ2.sum(0), "W3": dOb.T @ H2,
         "b3": dO.sum(0)}
    g["W1"][:, 24:] = 0
    g["W3"][3:] = 0
    g["b3"][3:] = 0
    flat = np.concatenate([np.asarray(g[name], np.float32).ravel() for name, _ in MLP_SHAPES])
    return flat, loss, n_valid


def mlp_loss64(feat_u16, target4, params):
    """Float64 loss of the same network without any rounding (for finite
    differences of the gradient formulas)."""
    P = mlp_unpack(params, np.float64)
    X = bf16_to_f32(feat_u16).astype(np.float64)
    s = lambda z: z / (1.0 + np.exp(-z))  # noqa: E731
    O = s(s(X @ P["W1"].T + P["b1"]) @ P["W2"].T + P["b2"]) @ P["W3"].T + P["b3"]
    T = np.asarray(target4, np.float64)
    n_valid = max(int(np.count_nonzero(T[:, 3])), 1)
    return float(np.sum(T[:, 3:4] * (O[:, :3] - T[:, :3]) ** 2) / n_valid)


def mlp_gradients64(feat_u16, target4, params):
    """The backward formulas in float64 without rounding."""
    P = mlp_unpack(params, np.float64)
    X = bf16_to_f32(feat_u16).astype(np.float64)
    sig = lambda z: 1.0 / (1.0 + np.exp(-z))  # noqa: E731
    Z1 = X @ P["W1"].T + P["b1"]
    H1 = Z1 * sig(Z1)
    Z2 = H1 @ P["W2"].T + P["b2"]
    H2 = Z2 * sig(Z2)
    O = H2 @ P["W3"].T + P["b3"]
    T = np.asarray(target4, np.float64)
    n_valid = max(int(np.count_nonzero(T[:, 3])), 1)
    dO = np.zeros_like(O)
    dO[:, :3] = 2.0 * T[:, 3:4] * (O[:, :3] - T[:, :3]) / n_valid
    sg = lambda z: sig(z) + z * sig(z) * (1 - sig(z))  # noqa: E731
    dZ2 = (dO @ P["W3"]) * sg(Z2)
    dZ1 = (dZ2 @ P["W2"]) * sg(Z1)
    g = {"W1": dZ1.T @ X, "b1": dZ1.sum(0), "W2": dZ2.T @ H1, "b2": dZ2.sum(0), "W3": dO.T @ H2, "b3": dO.sum(0)}
    return np.concatenate([np.asarray(g[name]).ravel() for name, _ in MLP_SHAPES])


# ---- colouring --------------------------------------------------------------
def color_edges(n_verts, edges, max_colors=100):
    edges = i32(edges)
    E = edges.shape[0]
    color = np.empty(max(E, 1), np.int32)
    sorted_edges = np.empty(max(E, 1), np.int32)
    prefix = np.empty(max_colors, np.int32)
    lib().or_color_edges(n_verts, E, _p(edges), max_colors, _p(color), _p(sorted_edges), _p(prefix))
    return color[:E], sorted_edges[:E], prefix


def gs_constraints(n_verts, edges, l0, bend, bend_l0, max_colors=100):
    """Springs and bending pairs coloured together as one edge list (the
    reference's colouring, graph_coloring.py:131-201) and packed in colour
    order: cons[i] = (v0, v1 | bit 31 for a bending pair, bits(l0), id) for
    id = sorted[i]; colour_start = the n_colors + 1 offsets of the colours."""
    edges, bend = i32(edges).reshape(-1, 2), i32(bend).reshape(-1, 2)
    E = edges.shape[0]
    pairs = np.concatenate([edges, bend])
    rest = np.concatenate([f32(l0), f32(bend_l0)])
    color, order, prefix = color_edges(n_verts, pairs, max_colors)
    n_colors = int(color.max()) + 1 if color.size else 0
    cons = np.zeros((pairs.shape[0], 4), np.int32)
    cons[:, 0] = pairs[order, 0]
    cons[:, 1] = np.where(order >= E, pairs[order, 1] | np.int32(-2147483648), pairs[order, 1])
    cons[:, 2] = rest[order].view(np.int32)
    cons[:, 3] = order
    start = np.append(prefix[:n_colors], pairs.shape[0]).astype(np.int32)
    return cons, start


def gs_sweep(y4, cons, colour_start, k_spring, k_bend):
    """One colour-ordered Gauss-Seidel sweep over cons, in place on y4."""
    assert y4.dtype == np.float32 and y4.flags.c_contiguous
    start = i32(colour_start)
    lib().or_gs_sweep(start.shape[0] - 1, _p(start), _p(i32(cons)), _p(y4), np.float32(k_spring),
                      np.float32(k_bend))


# ---- whole-solver driver -----------------------------------------------------
class OracleSolver:
    """CPU restatement of ``Solver.forward`` (XPBD.py:443-469).

    Per frame: if collisions are on and ``rebuild == "frame"``, build both cell
    BVHs on ``x`` (XPBD.py:448-458).  Per substep: compute_y; ``n_iter`` times
    [spring sweep + update_dx; if collisions: (first iteration: broad phase on y)
    narrow phase + update_dx]; compute_velocity; update_x.  With
    ``rebuild == "substep"`` the BVHs are rebuilt on ``x`` at the start of every
    substep.  With n_iter = 1 this is exactly the reference's substep.
    """

    def __init__(self, mesh_dy, mesh_st=None, *, dt, g, k_stretch_stiffness, k_bend_stiffness, dHat=4e-3,
                 damping=0.001, padding=0.05, n_iter=1, collisions=False, rebuild="frame", cap=40,
                 compliance_collision=1e8, nthreads=1, bending_on="x", self_collision=True,
                 contact_cull=False, tol=None, check_every=4, tol_relative=False, sewing=None,
                 velocity_update=False, mu=0.8, edge_edge=False, scatter_atomics=False, gauss_seidel=False):
        self.d = mesh_dy
        # colour-ordered Gauss-Seidel sweeps instead of the Jacobi sweep (needs
        # bending on y; the reference's solver has only the Jacobi sweep)
        self.gauss_seidel = gauss_seidel
        if gauss_seidel and bending_on != "y":
            raise ValueError("Gauss-Seidel sweeps need bending_on='y'")
        # multithreaded spring sweeps: a deterministic per-vertex gather (equal
        # to the serial sweep bit for bit) unless scatter_atomics, which runs
        # the reference's scatter with float atomics (order dependent), the
        # way a parallel Taichi CPU build executes it
        self.scatter_atomics = scatter_atomics
        # edge-edge contacts (the reference's commented-out ee_st / ee_dy path)
        self.edge_edge = edge_edge
        # iterate to a residual (the CUDA solver's tol mode): every
        # check_every-th iteration measures the residual of the current y; once
        # it is <= tol, that block of check_every iterations completes and the
        # rest are skipped
        self.tol = tol
        self.tol_relative = tol_relative
        # sewing: (sewn, sptr, partner, stiffness) -- k = stiffness * dt^2 per iteration
        self.sewing = sewing
        # velocity-level contact + friction pass after compute_velocity (XPBD.py:467-468)
        self.velocity_update = velocity_update
        self.mu = mu
        self._records = None
        self.check_every = check_every
        self.checks = 0
        self.stop_sum = 0
        self.converged = 0
        self.last_residual = None
        # the CUDA solver's contact_cull threshold, rounded to float32 from the
        # same double product
        self.cull_d2 = float(dHat) * 1.0625 if contact_cull else 0.0
        self.self_collision = self_collision
        self.s = mesh_st
        self.dt = float(dt)
        self.g = np.asarray(g, np.float32)
        self.kss = k_stretch_stiffness
        self.kbs = k_bend_stiffness
        self.dHat = np.float32(dHat)
        self.damping = np.float32(damping)
        self.padding = np.float32(padding)
        self.n_iter = n_iter
        self.collisions = collisions
        self.rebuild = rebuild
        self.cap = cap
        self.compliance = np.float32(compliance_collision)
        self.nthreads = nthreads
        self.bend_on_y = 1 if bending_on == "y" else 0
        V = mesh_dy["x"].shape[0]
        self.x4 = np.zeros((V, 4), np.float32)
        self.x4[:, :3] = mesh_dy["x"]
        self.fixed = f32(mesh_dy["fixed"])
        self.m_inv = f32(mesh_dy["m_inv"])
        self.x4[:, 3] = self.fixed * self.m_inv
        self.v4 = np.zeros((V, 4), np.float32)
        self.edges = i32(mesh_dy["edges"])
        self.l0 = f32(mesh_dy["l0"])
        self.bend = i32(mesh_dy["bend"]).reshape(-1, 2)
        self.bl0 = f32(mesh_dy["bend_l0"])
        self.faces = i32(mesh_dy["faces"])
        self.adj_ptr, self.adj = adjacency(V, self.edges, self.l0, self.bend, self.bl0)
        if gauss_seidel:
            self.gs_cons, self.gs_start = gs_constraints(V, self.edges, self.l0, self.bend, self.bl0)
        if edge_edge:
            self.face_edges = i32(mesh_dy["face_edges"])
            if mesh_st is not None:
                self.edges_st = i32(mesh_st["edges"])
                self.face_edges_st = i32(mesh_st["face_edges"])
        if collisions:
            self.bvh_dy = CellBVH()
            if mesh_st is not None:
                self.bvh_st = CellBVH()
                self.xs4 = np.zeros((mesh_st["x"].shape[0], 4), np.float32)
                self.xs4[:, :3] = mesh_st["x"]
                self.faces_st = i32(mesh_st["faces"])
        self.last_status = 0

    def _build(self):
        mn, mx = face_aabbs(self.x4, self.faces, self.padding)
        self.bvh_dy.build(mn, mx, scene_aabb(self.x4, self.padding))
        if self.s is not None:
            mn, mx = face_aabbs(self.xs4, self.faces_st, self.padding)
            self.bvh_st.build(mn, mx, scene_aabb(self.xs4, self.padding))

    def _broad(self, y4):
        qmn, qmx = query_boxes(y4, self.padding)
        Vd = y4.shape[0]
        if self.s is not None:
            vt_st = self.bvh_st.traverse(qmn, qmx, self.cap)
            smn, smx = query_boxes(self.xs4, self.padding)
            tv_st = self.bvh_dy.traverse(smn, smx, self.cap)
        else:
            vt_st = (np.zeros((Vd, self.cap), np.int32), np.zeros(Vd, np.int32), 0)
            tv_st = (np.zeros((0, self.cap), np.int32), np.zeros(0, np.int32), 0)
        if self.self_collision:
            vt_dy = self.bvh_dy.traverse(qmn, qmx, self.cap)
        else:
            vt_dy = (np.zeros((Vd, self.cap), np.int32), np.zeros(Vd, np.int32), 0)
        self.last_status |= vt_st[2] | vt_dy[2] | tv_st[2]
        self._ee = None
        if self.edge_edge:
            emn, emx = edge_query_boxes(y4, self.edges, self.padding)
            ee_st = self.bvh_st.traverse(emn, emx, self.cap) if self.s is not None else None
            ee_dy = self.bvh_dy.traverse(emn, emx, self.cap)
            self.last_status |= ee_dy[2] | (ee_st[2] if ee_st is not None else 0)
            self._ee = (ee_st, ee_dy)
        return vt_st, vt_dy, tv_st

    def substep(self, dt_sub):
        # dt_sub and the stiffness products are Python doubles, rounded to float32
        # when passed to the kernels, as the reference's kernel arguments are.
        dt_sub = float(dt_sub)
        if self.collisions and self.rebuild == "substep":
            self._build()
        y4 = predict(self.x4, self.v4, self.fixed, dt_sub, self.g, self.nthreads)
        k_spring = float(self.kbs) * dt_sub * dt_sub   # XPBD.py:354 (names swapped)
        k_bend = float(self.kss) * dt_sub * dt_sub     # XPBD.py:355
        cands = None
        stop = -1
        ref = residual(y4, self.adj_ptr, self.adj) if self.tol is not None and self.tol_relative else None
        for it in range(self.n_iter):
            if self.tol is not None:
                if stop >= 0 and it >= stop + self.check_every:
                    break
                if it > 0 and it % self.check_every == 0:
                    r = residual(y4, self.adj_ptr, self.adj)
                    self.last_residual = r
                    self.checks += 1
                    if stop < 0 and r[0] <= (self.tol * self.tol) * (ref[0] if ref is not None else r[1]):
                        stop = it
                        self.stop_sum += it
                        self.converged += 1
            if self.gauss_seidel:
                gs_sweep(y4, self.gs_cons, self.gs_start, k_spring, k_bend)
            elif self.nthreads > 1 and not self.scatter_atomics:
                spring_sweep_gather(self.x4, y4, self.fixed, self.m_inv, self.adj_ptr, self.adj, k_spring, k_bend,
                                    self.nthreads, self.bend_on_y)
            else:
                spring_sweep(self.x4, y4, self.fixed, self.m_inv, self.edges, self.l0, self.bend, self.bl0, k_spring,
                             k_bend, self.nthreads, self.bend_on_y)
            if self.collisions:
                if it == 0:
                    cands = self._broad(y4)
                vt_st, vt_dy, tv_st = cands
                acc = None
                if self.edge_edge:
                    Vd = y4.shape[0]
                    acc = (np.zeros(3 * Vd, np.int64), np.zeros(Vd, np.int32))
                    ee_st, ee_dy = self._ee
                    has_st = self.s is not None
                    re = edge_edge_sweep(self.edges, self.edges_st if has_st else None, self.face_edges,
                                         self.face_edges_st if has_st else None, y4, self.xs4 if has_st else None,
                                         self.fixed, self.m_inv, self.dHat, self.compliance, self.cap,
                                         ee_st[:2] if ee_st is not None else None, ee_dy[:2], acc[0], acc[1],
                                         nthreads=self.nthreads)
                    self.last_status |= re["status"]
                r = collision_sweep(self.faces, self.faces_st if self.s is not None else None, y4,
                                    self.xs4 if self.s is not None else None, self.fixed, self.m_inv, self.dHat,
                                    self.compliance, self.cap, vt_st[:2], vt_dy[:2], tv_st[:2],
                                    nthreads=self.nthreads, cull_d2=self.cull_d2,
                                    want_pairs=self.velocity_update, acc=acc)
                self.last_status |= r["status"]
                if self.velocity_update:
                    self._records = r
            if self.sewing is not None:
                sewn, sptr, partner, stiff = self.sewing
                sewing_step(y4, self.fixed, sewn, sptr, partner, float(stiff) * dt_sub * dt_sub)
        if self.velocity_update and self._records is not None:
            # compute_velocity, solve_constraints_v, update_x (XPBD.py:465-469), float32 as the kernels
            dtf = np.float32(dt_sub)
            s_ = (np.float32(1.0) - np.float32(self.damping)) * self.fixed
            self.v4[:, :3] = (s_[:, None] * (y4[:, :3] - self.x4[:, :3])) / dtf
            self.v4[:, 3] = 0
            vs4 = np.zeros_like(self.xs4) if self.s is not None else None
            self.last_status |= velocity_contacts(self.faces, self.faces_st if self.s is not None else None,
                                                  self.cap, self._records, self.v4, vs4, self.fixed, self.m_inv,
                                                  f32(self.s["m_inv"]) if self.s is not None else None, self.mu)
            self.x4[:, :3] = self.x4[:, :3] + dtf * self.v4[:, :3]
        else:
            velocity_update(self.x4, y4, self.v4, self.fixed, self.damping, dt_sub, self.nthreads)
        self.y4 = y4

    def forward(self, n_substeps):
        dt_sub = self.dt / n_substeps
        if self.collisions and self.rebuild == "frame":
            self._build()
        for _ in range(n_substeps):
            self.substep(dt_sub)
