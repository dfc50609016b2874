"""Golden vectors from the reference's own source -- TEST INFRASTRUCTURE ONLY.

Runs functions of the reference (medialab-ku/starlab-physics, read from the
directory given as the first argument) through ``taichi_standin`` (a numpy
stand-in for the Taichi API: serial loops, IEEE float32 per operation) on
seeded inputs and writes ``reference_vectors.npz`` beside this script:

* ``pt_*``   distance.d_type_PT and the distance of the branch it selects
             (d_PP / d_PE / d_PT, as collision_constraints_x.py calls them),
             plus the reference's generated gradients (g_PP / g_PE / g_PT);
* ``ee_*``   distance.d_type_EE and d_EE;
* ``morton_*`` LBVH_CELL.morton_3d on points in and around the unit cube;
* ``sub_*``  XPBD.Solver.compute_y, init_variables +
             solve_spring_constraints_x + update_dx (one sweep per substep,
             bending on x, the reference's substep) and compute_velocity +
             update_x, for three substeps of a small pinned cloth;
* ``lbvh_*`` LBVH_CELL.__init__ / build / traverse_cell_bvh_single on a
             small drape (digests of the 32768-cell arrays, candidate lists);
* ``ct_*``   XPBD.Solver.solve_collision_constraints_x + update_dx, then
             solve_constraints_v (friction + update_dv) (the
             three vertex-triangle contact kinds, with the reference's own
             gradients) on two cloth layers over a box;
* ``col_*``  GraphColoring.initEdgeIndicesForColor / initAdjEdges /
             colorEdgesGreedy / colorCountingSort on the edges of two grid
             cloths and an icosphere (edge ids in this repository's canonical
             numbering: the reference's own ids come from meshtaichi_patcher);
* ``mi_*``   MeshTaichiWrapper.findTriNeighbors / getBendingPair /
             init_bengding_l0 and initEdgeIndices (rest lengths, inverse
             masses) on a jittered grid cloth and an icosphere;
* ``kd_*``   LBVH_CELL.assign_internal_nodes_Karras12 (delta / find_split /
             determine_range) on sorted face codes with many repeated codes,
             the reference's equal-code rule.

Usage: python tests/golden/make_reference_vectors.py <reference checkout>
The npz is committed; the tests read it without the reference.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def point_triangle_vectors(ti, di, rng):
    pts = []
    for scale in (0.05, 2.0):
        pts.append((rng.normal(size=(800, 12)) * scale).astype(np.float32))
    # points near the triangle's plane and edges: region boundaries
    tri = rng.normal(size=(1200, 9)).astype(np.float32)
    w = rng.uniform(-0.2, 1.2, size=(1200, 3)).astype(np.float32)
    w /= w.sum(1, keepdims=True)
    p = (w[:, :1] * tri[:, 0:3] + w[:, 1:2] * tri[:, 3:6] + w[:, 2:3] * tri[:, 6:9]).astype(np.float32)
    p += rng.normal(size=p.shape).astype(np.float32) * np.float32(1e-3)
    pts.append(np.concatenate([p, tri], axis=1).astype(np.float32))
    P = np.concatenate(pts)
    n = P.shape[0]
    dtype = np.zeros(n, np.int32)
    d = np.zeros(n, np.float32)
    g = np.zeros((n, 4, 3), np.float32)
    for i in range(n):
        x = [ti.math.vec3(P[i, 3 * k: 3 * k + 3]) for k in range(4)]
        t = di.d_type_PT(*x)
        dtype[i] = t
        pair = {0: (0, 1), 1: (0, 2), 2: (0, 3)}
        edge = {3: (0, 1, 2), 4: (0, 2, 3), 5: (0, 1, 3)}
        if t in pair:
            a, b = pair[t]
            d[i] = di.d_PP(x[a], x[b])
            ga, gb = di.g_PP(x[a], x[b])
            g[i, a], g[i, b] = ga.to_numpy(), gb.to_numpy()
        elif t in edge:
            a, b, c = edge[t]
            d[i] = di.d_PE(x[a], x[b], x[c])
            ga, gb, gc = di.g_PE(x[a], x[b], x[c])
            g[i, a], g[i, b], g[i, c] = ga.to_numpy(), gb.to_numpy(), gc.to_numpy()
        else:
            d[i] = di.d_PT(*x)
            gg = di.g_PT(*x)
            for k in range(4):
                g[i, k] = gg[k].to_numpy()
    return {"pt_points": P, "pt_dtype": dtype, "pt_d": d, "pt_g": g}


def edge_edge_vectors(ti, di, rng):
    P = np.concatenate([(rng.normal(size=(1000, 12)) * s).astype(np.float32) for s in (0.01, 0.1, 1.0)])
    n = P.shape[0]
    dtype = np.zeros(n, np.int32)
    d = np.zeros(n, np.float32)
    for i in range(n):
        x = [ti.math.vec3(P[i, 3 * k: 3 * k + 3]) for k in range(4)]
        dtype[i] = di.d_type_EE(*x)
        d[i] = di.d_EE(*x) if dtype[i] == 8 else np.float32(0.0)
    return {"ee_points": P, "ee_dtype": dtype, "ee_d": d}


def morton_vectors(ti, lbvh_mod, rng):
    L = object.__new__(lbvh_mod.LBVH_CELL)
    pts = rng.uniform(-0.1, 1.1, size=(2000, 3)).astype(np.float32)
    pts[:20] = np.array([[0, 0, 0], [1, 1, 1], [0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5], [0.999, 0.001, 0.5],
                         [1023 / 1024, 0, 0], [1 / 1024, 1 / 1024, 1 / 1024]] + [[0.25, 0.5, 0.75]] * 12,
                        np.float32)
    codes = np.array([int(L.morton_3d(np.float32(x), np.float32(y), np.float32(z))) for x, y, z in pts], np.int64)
    return {"morton_points": pts, "morton_codes": codes.astype(np.int32)}


def _digest(a):
    import hashlib

    a = np.ascontiguousarray(a)
    return np.frombuffer(hashlib.sha256(a.tobytes()).digest(), dtype=np.uint8).copy()


class _Faces:
    """mesh.faces: per-face AABB fields, struct-for over faces."""

    def __init__(self, ti, mn, mx):
        self.n = mn.shape[0]
        self.aabb_min = ti.Field(np.ascontiguousarray(mn[:, :3]).copy(), 3)
        self.aabb_max = ti.Field(np.ascontiguousarray(mx[:, :3]).copy(), 3)

    def __iter__(self):
        for i in range(self.n):
            yield types.SimpleNamespace(id=i, aabb_min=self.aabb_min[i], aabb_max=self.aabb_max[i])


def lbvh_vectors(ti, lbvh_mod, repo_pkg, po):
    """LBVH_CELL.__init__ (cell codes, radix sort, Karras), build (face cells,
    counting sort, leaves, refit) and traverse_cell_bvh_single for the vertex
    boxes of a small drape.  The 32768-cell arrays are stored as SHA-256
    digests of their bytes."""
    sc = repo_pkg.scenes.drape256(n=12, sphere_subdiv=1)
    x = sc.cloth_x.astype(np.float32)
    f = sc.cloth_faces.astype(np.int32)
    x4 = np.zeros((x.shape[0], 4), np.float32)
    x4[:, :3] = x
    pad = np.float32(0.01)
    mn, mx = po.face_aabbs(x4, f, pad)
    box6 = po.scene_aabb(x4, pad)
    ref = lbvh_mod.LBVH_CELL(f.shape[0])
    n = ref.cell_nodes
    out = {"lbvh_init_digest": np.stack([_digest(ref.cell_morton_codes.a), _digest(ref.cell_ids.a),
                                         _digest(n.child_a.a[:32767]), _digest(n.child_b.a[:32767]),
                                         _digest(n.parent.a[1:]), _digest(n.range_l.a[:32767]),
                                         _digest(n.range_r.a[:32767])])}
    mesh = types.SimpleNamespace(faces=_Faces(ti, mn, mx))
    ref.build(mesh, ti.math.vec3(box6[:3]), ti.math.vec3(box6[3:]))
    out["lbvh_build_digest"] = np.stack([_digest(ref.prefix_sum_cell.a), _digest(ref.sorted_face_ids.a),
                                         _digest(n.num_faces.a), _digest(n.aabb_min.a),
                                         _digest(n.aabb_max.a)])
    Q, cap = x.shape[0], 40
    cache = ti.Field(np.full((Q, cap), -1, np.int32))
    nums = ti.Field(np.zeros(Q, np.int32))
    qmn, qmx = po.query_boxes(x4, pad)
    for i in range(Q):
        ref.traverse_cell_bvh_single(ref.cell_size, ref.origin, ti.math.vec3(qmn[i, :3]), ti.math.vec3(qmx[i, :3]),
                                     i, cache, nums)
    out.update(lbvh_x4=x4, lbvh_faces=f, lbvh_pad=np.array([pad], np.float32), lbvh_cand=cache.a.copy(),
               lbvh_num=nums.a.copy(), lbvh_cell_size=np.array(ref.cell_size.c, np.float32))
    return out


class _Verts:
    """mesh.verts: named per-vertex fields, struct-for over vertices."""

    def __init__(self, ti, n, **arrays):
        self._n = n
        for k, a in arrays.items():
            a = np.ascontiguousarray(a)
            object.__setattr__(self, k, ti.Field(a.copy(), a.shape[1] if a.ndim == 2 else None))

    def __iter__(self):
        for i in range(self._n):
            yield _VRef(self, i)


class _VRef:
    def __init__(self, verts, i):
        object.__setattr__(self, "_v", verts)
        object.__setattr__(self, "id", i)

    def __getattr__(self, k):
        return getattr(self._v, k)[self.id]

    def __setattr__(self, k, val):
        getattr(self._v, k)[self.id] = val


def substep_vectors(ti, xpbd_mod, repo_pkg):
    mesh = repo_pkg.mesh
    x, f = mesh.grid_cloth(7, height=1.0)
    rng = np.random.default_rng(3)
    x = (x + rng.uniform(-1e-3, 1e-3, size=x.shape)).astype(np.float32)
    edges = mesh.edges_from_faces(f)
    bend = mesh.bending_pairs(f)
    l0 = mesh.rest_lengths(x, edges)
    bl0 = mesh.rest_lengths(x, bend)
    m_inv = mesh.inverse_masses(x.shape[0], edges, l0)
    V = x.shape[0]
    fixed = np.ones(V, np.float32)
    fixed[[V - 7, V - 1]] = 0.0
    v0 = (rng.normal(size=(V, 3)) * 0.05).astype(np.float32)
    m = types.SimpleNamespace()
    m.verts = _Verts(ti, V, x=x, y=x, v=v0, dx=np.zeros((V, 3), np.float32), nc=np.zeros(V, np.float32),
                     fixed=fixed, m_inv=m_inv)
    m.edges = types.SimpleNamespace(l0=ti.Field(l0.astype(np.float32).copy()))
    m.edge_indices = ti.Field(edges.reshape(-1).astype(np.int32).copy())
    m.bending_indices = ti.Field(bend.reshape(-1).astype(np.int32).copy())
    m.bending_l0 = ti.Field(bl0.astype(np.float32).copy())
    m.bending_constraint_count = bend.shape[0]
    S = xpbd_mod.Solver
    s = object.__new__(S)
    s.mesh_dy = m
    s.max_num_edges_dy = edges.shape[0]
    s.g = ti.math.vec3(0.0, 0.0, -9.81)
    stiff_stretch, stiff_bending = 1e5, 1e8   # reference arguments (springs use stiffness_bending)
    s.stiffness_stretch, s.stiffness_bending = stiff_stretch, stiff_bending
    dt_frame, n_sub, damping = 1.0 / 60.0, 3, 0.001
    dt = dt_frame / n_sub
    ys, xs, vs = [], [], []
    for _ in range(n_sub):
        S.compute_y(s, dt)
        S.init_variables(s)
        S.solve_spring_constraints_x(s, stiff_bending * dt * dt, stiff_stretch * dt * dt)
        S.update_dx(s)
        ys.append(m.verts.y.to_numpy())
        S.compute_velocity(s, damping, dt)
        S.update_x(s, dt)
        xs.append(m.verts.x.to_numpy())
        vs.append(m.verts.v.to_numpy())
    return {"sub_x0": x, "sub_v0": v0, "sub_faces": f.astype(np.int32), "sub_fixed": fixed,
            "sub_params": np.array([dt_frame, n_sub, damping, stiff_stretch, stiff_bending], np.float64),
            "sub_y": np.stack(ys), "sub_x": np.stack(xs), "sub_v": np.stack(vs)}


def contact_vectors(ti, xpbd_mod, repo_pkg, po):
    """XPBD.Solver.solve_collision_constraints_x (+ update_dx) on two coarse
    cloth layers 1 cm apart lying 5 mm above a box: vertex-vs-static,
    vertex-vs-own-cloth and static-vertex contacts, with the reference's
    generated gradients.  Candidates come from the oracle's cell BVHs (pinned
    above)."""
    sc = repo_pkg.scenes.crossed_layers()
    x = sc.cloth_x.astype(np.float32).copy()
    nA = x.shape[0] // 2
    x[:nA, 2] = np.float32(0.515)
    x[nA:, 2] = np.float32(0.505)
    rng = np.random.default_rng(7)
    x[:, 2] += (rng.normal(size=x.shape[0]) * 2e-3).astype(np.float32)
    f = sc.cloth_faces.astype(np.int32)
    xs, fs = sc.obstacle_x.astype(np.float32), sc.obstacle_faces.astype(np.int32)
    mesh = repo_pkg.mesh
    edges = mesh.edges_from_faces(f)
    l0 = mesh.rest_lengths(x, edges)
    m_inv = mesh.inverse_masses(x.shape[0], edges, l0)
    fixed = np.ones(x.shape[0], np.float32)
    fixed[[0, nA + 5]] = 0.0
    Vd, Vs, cap = x.shape[0], xs.shape[0], 40
    pad, dHat, comp = np.float32(sc.padding), np.float32(sc.dHat), np.float32(1e8)
    x4 = np.zeros((Vd, 4), np.float32)
    x4[:, :3] = x
    xs4 = np.zeros((Vs, 4), np.float32)
    xs4[:, :3] = xs
    bd, bs = po.CellBVH(), po.CellBVH()
    mn, mx = po.face_aabbs(x4, f, pad)
    bd.build(mn, mx, po.scene_aabb(x4, pad))
    mn, mx = po.face_aabbs(xs4, fs, pad)
    bs.build(mn, mx, po.scene_aabb(xs4, pad))
    qd = po.query_boxes(x4, pad)
    qs = po.query_boxes(xs4, pad)
    vt_st = bs.traverse(*qd, cap)
    vt_dy = bd.traverse(*qd, cap)
    tv_st = bd.traverse(*qs, cap)
    s = object.__new__(xpbd_mod.Solver)
    md = types.SimpleNamespace()
    v0 = (rng.normal(size=(Vd, 3)) * 0.3).astype(np.float32)
    vs0 = (rng.normal(size=(Vs, 3)) * 0.05).astype(np.float32)
    # the static mesh's inverse masses are read at a cloth vertex index in one
    # branch of __vt_st (collision_constraints_v.py:68); padded with zeros past
    # the static vertex count, the convention the oracle follows
    ms_m_inv = np.zeros(max(Vd, Vs), np.float32)
    ms_m_inv[:Vs] = 1.0
    md.verts = _Verts(ti, Vd, x=x, y=x, v=v0, dx=np.zeros((Vd, 3), np.float32), dv=np.zeros((Vd, 3), np.float32),
                      nc=np.zeros(Vd, np.float32), fixed=fixed, m_inv=m_inv)
    md.face_indices = ti.Field(f.reshape(-1).copy())
    ms = types.SimpleNamespace()
    ms.verts = _Verts(ti, Vs, x=xs, v=vs0, m_inv=ms_m_inv)
    ms.face_indices = ti.Field(fs.reshape(-1).copy())
    s.mesh_dy, s.mesh_st = md, ms
    s.max_num_verts_dy, s.max_num_verts_st = Vd, Vs
    s.dHat = dHat
    s.vt_st_pair_cache_size = s.tv_st_pair_cache_size = s.vt_dy_pair_cache_size = cap
    for name, (c, nm), Q in (("vt_st", vt_st[:2], Vd), ("vt_dy", vt_dy[:2], Vd), ("tv_st", tv_st[:2], Vs)):
        setattr(s, name + "_candidates", ti.Field(c.copy()))
        setattr(s, name + "_candidates_num", ti.Field(np.minimum(nm, cap).astype(np.int32)))
        setattr(s, name + "_pair", ti.Field(np.zeros((Q, cap, 2), np.int32)))
        setattr(s, name + "_pair_num", ti.Field(np.zeros(Q, np.int32)))
        setattr(s, name + "_pair_g", ti.Field(np.zeros((Q, cap, 4, 3), np.float32), 3))
        setattr(s, name + "_pair_schur", ti.Field(np.zeros((Q, cap), np.float32)))
    xpbd_mod.Solver.solve_collision_constraints_x(s, comp)
    dx = md.verts.dx.to_numpy()
    nc = md.verts.nc.to_numpy()
    xpbd_mod.Solver.update_dx(s)
    y = md.verts.y.to_numpy()
    # the velocity pass (solve_constraints_v: reset dv/nc, friction over the
    # pair records just made, update_dv)
    s.mu = np.float32(0.8)
    s.enable_collision_handling = True
    xpbd_mod.Solver.solve_constraints_v(s)
    out = {"ct_x4": x4, "ct_faces": f, "ct_xs4": xs4, "ct_faces_st": fs, "ct_fixed": fixed, "ct_m_inv": m_inv,
           "ct_params": np.array([pad, dHat, comp, cap], np.float32), "ct_dx": dx, "ct_nc": nc, "ct_y": y,
           "ct_v0": v0, "ct_vs0": vs0, "ct_mu": np.array([s.mu], np.float32), "ct_v": md.verts.v.to_numpy()}
    for name in ("vt_st", "vt_dy", "tv_st"):
        out["ct_%s_pair" % name] = getattr(s, name + "_pair").a.copy()
        out["ct_%s_pair_num" % name] = getattr(s, name + "_pair_num").a.copy()
        out["ct_%s_pair_g" % name] = getattr(s, name + "_pair_g").a.copy()
        out["ct_%s_pair_schur" % name] = getattr(s, name + "_pair_schur").a.copy()
    return out


class _ERef:
    """One mesh edge in a struct-for: .id, .verts (two vertex refs), .l0."""

    def __init__(self, l0_field, verts, i, a, b):
        object.__setattr__(self, "_l0", l0_field)
        object.__setattr__(self, "id", i)
        object.__setattr__(self, "verts", [_VRef(verts, a), _VRef(verts, b)])

    def __getattr__(self, k):
        if k == "l0":
            return self._l0[self.id]
        raise AttributeError(k)

    def __setattr__(self, k, val):
        if k != "l0":
            raise AttributeError(k)
        self._l0[self.id] = val


def coloring_vectors(ti, gc_mod, repo_pkg):
    """GraphColoring's greedy colouring and counting sort (graph_coloring.py:
    112-149, 172-201), run as the reference's constructor runs them when no
    precomputed colouring exists (:55-92), minus the phantom insertion (prints
    only) and the .npy export."""
    mesh = repo_pkg.mesh
    cases = [mesh.grid_cloth(9)[1], mesh.grid_cloth(14)[1], mesh.icosphere(2, 1.0)[1]]
    out = {}
    for k, f in enumerate(cases):
        e = mesh.edges_from_faces(f).astype(np.int32)
        E = e.shape[0]
        g = object.__new__(gc_mod.GraphColoring)
        g.num_edges = E
        g.num_verts = int(f.max()) + 1
        g.edges = [types.SimpleNamespace(id=i) for i in range(E)]
        g.eid_np = e
        g.eid_field = ti.Field(e.copy())
        g.edge_indices_sequence = ti.Field(np.zeros(E, np.int32))
        g.edges_color = ti.Field(np.full(E, -1, np.int32))
        g.adj_edges_list = ti.Field(np.zeros((E, E), np.int32))
        g.max_num_colors = 100
        g.available_colors = ti.Field(np.zeros(g.max_num_colors, np.int32))
        g.initEdgeIndicesForColor()
        g.edge_indices_sequence_np = g.edge_indices_sequence.to_numpy()
        g.initAdjEdges()
        g.edges_color_np = g.edges_color.to_numpy()
        g.adj_edges_list_np = g.adj_edges_list.to_numpy()
        g.available_colors_np = g.available_colors.to_numpy()
        g.colorEdgesGreedy()
        g.sorted_edges_sequence_np = g.edge_indices_sequence.to_numpy()
        g.sorted_edges_color_np = g.edges_color_np.copy()
        g.color_prefix_sum_np = np.zeros(g.max_num_colors, np.int32)
        g.colorCountingSort()
        out["col%d_edges" % k] = e
        out["col%d_color" % k] = g.edges_color_np.astype(np.int32)
        out["col%d_sorted" % k] = g.sorted_edges_sequence_np.astype(np.int32)
        out["col%d_prefix" % k] = g.color_prefix_sum_np.astype(np.int32)
    return out


class _Np126Array(np.ndarray):
    """numpy 1.26 (the reference's pinned version) let a size-1 array be
    assigned to a scalar element (getBendingPair's ``pairs[count, 0] =
    v[~np.isin(v, w)]``); numpy 2.x raises.  This array restores that one rule."""

    def __setitem__(self, key, value):
        if isinstance(value, np.ndarray) and value.ndim > 0 and value.size == 1 and np.ndim(self[key]) == 0:
            value = value.reshape(()).item()
        super().__setitem__(key, value)


class _Np126:
    """The numpy namespace with zeros() returning _Np126Array."""

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def zeros(*a, **k):
        return np.zeros(*a, **k).view(_Np126Array)


def mesh_init_vectors(ti, mtw_mod, repo_pkg):
    """findTriNeighbors / getBendingPair (meshTaichiWrapper.py:177-225) and the
    bending rest lengths of init_bengding_l0 (:142-145); initEdgeIndices
    (:244-256): rest lengths l0 and m_inv = 1 / sum of half the incident rest
    lengths, accumulated in edge order."""
    mesh = repo_pkg.mesh
    rng = np.random.default_rng(17)
    xg, fg = mesh.grid_cloth(11)
    xg = (xg + rng.uniform(-1e-3, 1e-3, xg.shape)).astype(np.float32)
    xi, fi = mesh.icosphere(2, 0.3, (0.5, 0.5, 0.5))
    out = {}
    for k, (x, f) in enumerate([(xg, fg), (xi.astype(np.float32), fi)]):
        m = object.__new__(mtw_mod.MeshTaichiWrapper)
        m.fid_np = np.asarray(f, np.int64)
        saved = mtw_mod.np
        mtw_mod.np = _Np126()
        try:
            count, nb = m.findTriNeighbors()
            pairs = np.asarray(m.getBendingPair(count, nb))
        finally:
            mtw_mod.np = saved
        V = x.shape[0]
        verts = _Verts(ti, V, x=x, m_inv=np.zeros(V, np.float32))
        e = mesh.edges_from_faces(f).astype(np.int32)
        E = e.shape[0]
        l0f = ti.Field(np.zeros(E, np.float32))
        m.mesh = types.SimpleNamespace(edges=[_ERef(l0f, verts, i, int(e[i, 0]), int(e[i, 1])) for i in range(E)],
                                       verts=verts)
        m.bending_constraint_count = count
        m.bending_indices = ti.Field(pairs.reshape(-1).astype(np.int32).copy())
        m.bending_l0 = ti.Field(np.zeros(count, np.float32))
        mtw_mod.MeshTaichiWrapper.init_bengding_l0(m)
        bl0 = m.bending_l0.to_numpy().astype(np.float32)
        m.edge_indices = ti.Field(np.zeros(2 * E, np.int32))
        mtw_mod.MeshTaichiWrapper.initEdgeIndices(m)
        out.update({"mi%d_x" % k: x, "mi%d_faces" % k: np.asarray(f, np.int32),
                    "mi%d_bend" % k: pairs.astype(np.int32), "mi%d_bend_l0" % k: bl0,
                    "mi%d_edges" % k: e, "mi%d_l0" % k: l0f.to_numpy().astype(np.float32),
                    "mi%d_m_inv" % k: verts.m_inv.to_numpy().astype(np.float32),
                    "mi%d_edge_indices" % k: m.edge_indices.to_numpy().astype(np.int32)})
    return out


def karras_dup_vectors(ti, lbvh_mod, rng):
    """assign_internal_nodes_Karras12 (lbvh_cell.py:384-405) over sorted 30-bit
    codes in which most codes repeat (runs of 1-40 equal codes, plus one long
    run), the case where delta returns 32 for equal neighbours (:256-264)."""
    out = {}
    for k, n in enumerate((600, 2500)):
        runs = []
        total = 0
        while total < n:
            r = int(rng.integers(1, 41)) if rng.random() > 0.02 else 200
            runs.append(min(r, n - total))
            total += runs[-1]
        vals = np.sort(rng.choice(1 << 30, size=len(runs), replace=False)).astype(np.int64)
        codes = np.repeat(vals, runs).astype(np.int32)
        L = object.__new__(lbvh_mod.LBVH_CELL)
        L.num_leafs = n
        L.leaf_offset = n - 1
        L.morton_codes = ti.Field(codes.copy())
        L.nodes = lbvh_mod.Node.field(shape=(2 * n - 1))
        L.assign_internal_nodes_Karras12()
        nd = L.nodes
        out.update({"kd%d_codes" % k: codes, "kd%d_child_a" % k: nd.child_a.a[: n - 1].copy(),
                    "kd%d_child_b" % k: nd.child_b.a[: n - 1].copy(),
                    "kd%d_range_l" % k: nd.range_l.a[: n - 1].copy(),
                    "kd%d_range_r" % k: nd.range_r.a[: n - 1].copy(), "kd%d_parent" % k: nd.parent.a.copy()})
    return out


def main(ref_dir):
    sys.path.insert(0, HERE)
    import taichi_standin

    ti = taichi_standin.install()
    sys.path.insert(0, ref_dir)
    import framework.collision.distance as di
    import framework.collision.lbvh_cell as lbvh_mod
    import framework.physics.XPBD as xpbd_mod

    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge

    pkg = ge.load_package()
    rng = np.random.default_rng(20240611)
    out = {}
    out.update(point_triangle_vectors(ti, di, rng))
    out.update(edge_edge_vectors(ti, di, rng))
    out.update(morton_vectors(ti, lbvh_mod, rng))
    out.update(substep_vectors(ti, xpbd_mod, pkg))
    from oracle import pyoracle as po

    out.update(lbvh_vectors(ti, lbvh_mod, pkg, po))
    out.update(contact_vectors(ti, xpbd_mod, pkg, po))
    import framework.utilities.graph_coloring as gc_mod

    # meshTaichiWrapper imports meshtaichi_patcher and igl at module level; the
    # functions used here touch neither
    for name in ("meshtaichi_patcher", "igl"):
        sys.modules.setdefault(name, types.ModuleType(name))
    import framework.meshio.meshTaichiWrapper as mtw_mod

    out.update(coloring_vectors(ti, gc_mod, pkg))
    out.update(mesh_init_vectors(ti, mtw_mod, pkg))
    out.update(karras_dup_vectors(ti, lbvh_mod, rng))
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STARLAB_REFERENCE", "."))
