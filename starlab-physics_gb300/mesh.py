"""Triangle-mesh state and topology for the XPBD cloth substep.

This module mirrors ``framework/meshio/meshTaichiWrapper.py`` (class
``MeshTaichiWrapper``): per-vertex state ``x, y, v, fixed, m_inv``, per-edge rest
lengths, face/edge index arrays, bending pairs and face AABBs.  Element numbering
is canonical and documented here (the reference takes its numbering from
meshtaichi_patcher, which relabels elements for patch locality):

* vertices: in the order the generator emits them;
* faces: in the order the generator emits them;
* edges: the unique undirected face edges, oriented ``(a, b)`` with ``a < b`` and
  sorted lexicographically by ``(a, b)``;
* bending pairs: exactly the rule of ``findTriNeighbors`` / ``getBendingPair``
  (``meshTaichiWrapper.py:152-225``) applied to the canonical face array.

Topology and rest-state set-up (rest lengths, masses, bending pairs, the
vertex-centric constraint adjacency) is host-side initialisation, as in the
reference, where it runs once in numpy/Taichi before the first frame.  All
per-substep work runs in the CUDA library.

Device layout (torch CUDA tensors, SoA, float4-padded):

* ``x4, y4, v4: float32[V, 4]`` -- xyz plus ``w``.  ``x4.w`` and ``y4.w`` hold
  ``wf = fixed * m_inv`` so a single 16-byte load gives a neighbour's position
  and its effective inverse mass; ``v4.w`` is 0.
* ``fixed, m_inv: float32[V]``.
* ``face_indices: int32[F*3]``, ``edge_indices: int32[E*2]``, ``l0: float32[E]``,
  ``bending_indices: int32[B*2]``, ``bending_l0: float32[B]``,
  ``face_edge_indices: int32[F*3]`` (edge ids of each face's sides, for the
  edge-edge contacts).
* ``adj_ptr: int32[V+1]`` and ``adj: int32[2*(E+B), 2]`` -- the vertex-centric
  list of incident constraints in ascending constraint index (springs
  ``0..E-1`` then bending pairs ``E..E+B-1``); each entry is
  ``(neighbour | BEND_FLAG, float_bits(rest_length))``.
"""
from __future__ import annotations

import numpy as np

from ._lib import ptr, stream_handle, sx

BEND_FLAG = np.int32(-2147483648)  # bit 31 marks a bending entry in the adjacency


# ----------------------------------------------------------------------------
# generators (canonical numbering)
# ----------------------------------------------------------------------------

def grid_cloth(n: int, *, origin=(0.0, 0.0), size=1.0, height=1.0):
    """Square cloth of ``n x n`` vertices in the plane ``z = height``.

    Vertex ``i * n + j`` sits at ``(origin_x + j*h, origin_y + i*h, height)`` with
    ``h = size / (n - 1)``.  Quad ``(i, j)`` is split along the diagonal
    ``v00-v11`` into faces ``(v00, v01, v11)`` and ``(v00, v11, v10)``.
    Returns ``(x: float32[V,3], faces: int32[F,3])``.
    """
    if n < 2:
        raise ValueError("grid side must be >= 2")
    h = np.float32(size) / np.float32(n - 1)
    jj, ii = np.meshgrid(np.arange(n, dtype=np.float32), np.arange(n, dtype=np.float32))
    x = np.empty((n * n, 3), dtype=np.float32)
    x[:, 0] = np.float32(origin[0]) + jj.ravel() * h
    x[:, 1] = np.float32(origin[1]) + ii.ravel() * h
    x[:, 2] = np.float32(height)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    v00 = (i * n + j).ravel()
    v01 = v00 + 1
    v10 = v00 + n
    v11 = v10 + 1
    faces = np.empty(((n - 1) * (n - 1) * 2, 3), dtype=np.int32)
    faces[0::2] = np.stack([v00, v01, v11], axis=1)
    faces[1::2] = np.stack([v00, v11, v10], axis=1)
    return x, faces


def box_mesh(side: float, center=(0.0, 0.0, 0.0)):
    """Axis-aligned closed box: 8 vertices, 12 outward-facing triangles."""
    c = np.asarray(center, dtype=np.float32)
    s = np.float32(side) * np.float32(0.5)
    corners = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float32)
    x = (c + corners * s).astype(np.float32)
    faces = np.array([[0, 2, 1], [0, 3, 2],   # bottom (-z)
                      [4, 5, 6], [4, 6, 7],   # top (+z)
                      [0, 1, 5], [0, 5, 4],   # -y
                      [2, 3, 7], [2, 7, 6],   # +y
                      [1, 2, 6], [1, 6, 5],   # +x
                      [3, 0, 4], [3, 4, 7]],  # -x
                     dtype=np.int32)
    return x, faces


def icosphere(subdivisions: int, radius: float, center=(0.0, 0.0, 0.0)):
    """Icosphere: 20 * 4**s faces, 10 * 4**s + 2 vertices (s=5: 20480 / 10242).

    Computed in float64 and rounded to float32 once.  Midpoint vertices are
    numbered in order of first appearance while faces are visited in order.
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    x = np.asarray(center, dtype=np.float64) + radius * np.stack(verts)
    return x.astype(np.float32), np.asarray(faces, dtype=np.int32)


# ----------------------------------------------------------------------------
# topology
# ----------------------------------------------------------------------------

def edges_from_faces(faces: np.ndarray) -> np.ndarray:
    """Unique undirected edges ``(a, b)``, ``a < b``, sorted by ``(a, b)``."""
    f = np.asarray(faces, dtype=np.int64)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    e.sort(axis=1)
    e = np.unique(e, axis=0)
    return e.astype(np.int32)


def face_edges(faces: np.ndarray, edges: np.ndarray) -> np.ndarray:
    """Edge ids of each face's sides ``(f0, f1), (f1, f2), (f2, f0)``
    (``face_edge_indices``, ``meshTaichiWrapper.py:115-119``), against the
    canonical edge table of :func:`edges_from_faces`."""
    f = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    if f.shape[0] == 0:
        return np.zeros((0, 3), np.int32)
    n = int(max(f.max(), e.max() if e.size else 0)) + 1
    keys = e[:, 0] * n + e[:, 1]
    out = np.empty(f.shape, dtype=np.int64)
    for k in range(3):
        a, b = f[:, k], f[:, (k + 1) % 3]
        q = np.minimum(a, b) * n + np.maximum(a, b)
        idx = np.searchsorted(keys, q)
        if (idx >= keys.shape[0]).any() or (keys[np.minimum(idx, keys.shape[0] - 1)] != q).any():
            raise ValueError("a face side is missing from the edge table")
        out[:, k] = idx
    return out.astype(np.int32)


def bending_pairs(faces: np.ndarray) -> np.ndarray:
    """Opposite-vertex pairs of adjacent triangles.

    Restates ``findTriNeighbors`` + ``getBendingPair``
    (``meshTaichiWrapper.py:152-225``): build the table ``(v1, v2, 3f+k)`` of each
    face's sorted-vertex edges ``(v1,v2), (v1,v3), (v2,v3)``; stable lexicographic
    sort by ``(v1, v2)``; pair up consecutive equal rows (advance by 2 on a match,
    else by 1); then visit faces in order and local edges ``k = 0..2`` and emit,
    for each not-yet-visited neighbour edge, ``(vertex of f not in g, vertex of g
    not in f)`` where ``g`` is the neighbour face.
    """
    f = np.asarray(faces, dtype=np.int64)
    nf = f.shape[0]
    fs = np.sort(f, axis=1)
    table = np.empty((3 * nf, 3), dtype=np.int64)
    table[0::3] = np.stack([fs[:, 0], fs[:, 1], 3 * np.arange(nf)], axis=1)
    table[1::3] = np.stack([fs[:, 0], fs[:, 2], 3 * np.arange(nf) + 1], axis=1)
    table[2::3] = np.stack([fs[:, 1], fs[:, 2], 3 * np.arange(nf) + 2], axis=1)
    order = np.lexsort((table[:, 1], table[:, 0]))  # stable
    table = table[order]
    n_rows = 3 * nf
    if n_rows < 2:
        return np.zeros((0, 2), np.int32)
    # The sequential scan pairs rows (r, r+1) and skips by two on a match, so
    # inside a run of equal keys starting at s it pairs (s, s+1), (s+2, s+3), ...
    key_change = np.ones(n_rows, dtype=bool)
    key_change[1:] = (table[1:, 0] != table[:-1, 0]) | (table[1:, 1] != table[:-1, 1])
    run_id = np.cumsum(key_change) - 1
    run_start = np.flatnonzero(key_change)
    pos_in_run = np.arange(n_rows) - run_start[run_id]
    run_len = np.diff(np.append(run_start, n_rows))[run_id]
    first = (pos_in_run % 2 == 0) & (pos_in_run + 1 < run_len)
    ra = table[first, 2]
    rb = table[np.flatnonzero(first) + 1, 2]
    # getBendingPair visits edge slots 3f+k in ascending order and emits each pair
    # once, at the smaller slot.
    lo = np.minimum(ra, rb)
    hi = np.maximum(ra, rb)
    o = np.argsort(lo, kind="stable")
    lo, hi = lo[o], hi[o]
    # local edge k of a sorted face (v1,v2,v3): 0=(v1,v2), 1=(v1,v3), 2=(v2,v3);
    # the vertex not on that edge is v3, v2, v1 respectively.
    opp_col = np.array([2, 1, 0])
    a = fs[lo // 3, opp_col[lo % 3]]
    b = fs[hi // 3, opp_col[hi % 3]]
    return np.stack([a, b], axis=1).astype(np.int32).reshape(-1, 2)


def rest_lengths(x: np.ndarray, pairs: np.ndarray) -> np.ndarray:
    """``|x[a] - x[b]|`` in float32, summed ``(dx*dx + dy*dy) + dz*dz``."""
    d = x[pairs[:, 0]].astype(np.float32) - x[pairs[:, 1]].astype(np.float32)
    s = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    return np.sqrt(s).astype(np.float32)


def inverse_masses(n_verts: int, edges: np.ndarray, l0: np.ndarray) -> np.ndarray:
    """``m_inv = 1 / sum(0.5 * l0)`` over incident edges (``initEdgeIndices``,
    ``meshTaichiWrapper.py:244-256``), accumulated per vertex in ascending edge
    index.  Vertices without edges get ``1/0 = inf`` as in the reference."""
    half = (np.float32(0.5) * l0).astype(np.float32)
    idx = edges.astype(np.int64).reshape(-1)           # a0, b0, a1, b1, ...
    vals = np.repeat(half, 2)
    m = np.zeros(n_verts, dtype=np.float32)
    np.add.at(m, idx, vals)                            # sequential, in index order
    with np.errstate(divide="ignore"):
        return (np.float32(1.0) / m).astype(np.float32)


def constraint_adjacency(n_verts: int, edges: np.ndarray, l0: np.ndarray,
                         bend: np.ndarray, bend_l0: np.ndarray):
    """Vertex-centric CSR of incident constraints, ascending constraint index.

    Entry ``(nbr | BEND_FLAG?, bits(l0))``; springs are ``0..E-1`` and bending
    pairs ``E..E+B-1``, so each vertex lists its springs first, then its bending
    pairs, each in ascending index -- the order in which a serial execution of
    ``solve_spring_constraints_x`` (``XPBD.py:141-184``) accumulates into ``dx``.
    """
    E = edges.shape[0]
    B = bend.shape[0]
    a = np.concatenate([edges[:, 0], bend[:, 0]]).astype(np.int64)
    b = np.concatenate([edges[:, 1], bend[:, 1]]).astype(np.int64)
    rl = np.concatenate([l0, bend_l0]).astype(np.float32)
    is_bend = np.concatenate([np.zeros(E, bool), np.ones(B, bool)])
    cid = np.arange(E + B, dtype=np.int64)
    owner = np.concatenate([a, b])
    nbr = np.concatenate([b, a])
    cc = np.concatenate([cid, cid])
    order = np.lexsort((cc, owner))
    owner, nbr, cc = owner[order], nbr[order], cc[order]
    counts = np.bincount(owner, minlength=n_verts)
    ptr = np.zeros(n_verts + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(counts)
    adj = np.empty((owner.shape[0], 2), dtype=np.int32)
    word = nbr.astype(np.int32)
    word = np.where(is_bend[cc], word | BEND_FLAG, word).astype(np.int32)
    adj[:, 0] = word
    adj[:, 1] = rl[cc].view(np.int32)
    return ptr, adj


def packed_adjacency(ptr: np.ndarray, adj: np.ndarray):
    """The packed form of :func:`constraint_adjacency` for ``sx_jacobi_sweep_packed``:
    ``nbr16[k] = neighbour - owner`` (int16) and ``rest32[k] = bits(l0)`` with
    bit 31 set for a bending pair, both padded with zeros to a multiple of 8
    entries plus 8 (the kernel reads whole 16-byte groups).  None when an
    offset does not fit in 16 bits (the int2 sweep then serves)."""
    ptr = np.asarray(ptr, np.int64)
    adj = np.asarray(adj, np.int32).reshape(-1, 2)
    n = adj.shape[0]
    owner = np.repeat(np.arange(ptr.shape[0] - 1, dtype=np.int64), np.diff(ptr))
    word = adj[:, 0].view(np.uint32)
    delta = (word & np.uint32(0x7FFFFFFF)).astype(np.int64) - owner
    if n and (delta.min() < -32768 or delta.max() > 32767):
        return None
    size = ((n + 7) // 8) * 8 + 8
    nbr16 = np.zeros(size, np.int16)
    rest32 = np.zeros(size, np.uint32)
    nbr16[:n] = delta.astype(np.int16)
    rest32[:n] = adj[:, 1].view(np.uint32) | (word & np.uint32(0x80000000))
    return nbr16, rest32.view(np.int32)


class _Verts:
    """Attribute bag mirroring ``mesh.verts.{x,y,v,fixed,m_inv}``."""


class TriMesh:
    """Mesh state on the GPU (mirrors ``MeshTaichiWrapper``).

    ``TriMesh(x, faces, device=...)``: ``x`` float32[V,3] rest positions, ``faces``
    int32[F,3].  Builds edges, rest lengths, masses (``initEdgeIndices``), bending
    pairs (``initBendingIndices``) and the vertex-centric adjacency, uploads
    everything as torch tensors and keeps ``x0`` for :meth:`reset`.
    """

    def __init__(self, x, faces, *, device="cuda", is_static=False, with_bending=True):
        import torch

        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, 3))
        faces = np.ascontiguousarray(np.asarray(faces, dtype=np.int32).reshape(-1, 3))
        self.device = torch.device(device)
        self.is_static = is_static
        self.num_verts = x.shape[0]
        self.num_faces = faces.shape[0]
        edges = edges_from_faces(faces)
        self.num_edges = edges.shape[0]
        l0 = rest_lengths(x, edges)
        m_inv = inverse_masses(self.num_verts, edges, l0)
        if with_bending:
            bend = bending_pairs(faces)
        else:
            bend = np.zeros((0, 2), np.int32)
        bend_l0 = rest_lengths(x, bend) if bend.shape[0] else np.zeros(0, np.float32)
        self.bending_constraint_count = bend.shape[0]
        ptr, adj = constraint_adjacency(self.num_verts, edges, l0, bend, bend_l0)

        # host copies (canonical topology; used by tests and the oracle)
        self.x0_np = x
        self.fid_np = faces
        self.eid_np = edges
        self.face_edge_np = face_edges(faces, edges)
        self.l0_np = l0
        self.m_inv_np = m_inv
        self.bending_np = bend
        self.bending_l0_np = bend_l0
        self.adj_ptr_np = ptr
        self.adj_np = adj

        dev = self.device
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.face_indices = t(faces.reshape(-1))
        self.edge_indices = t(edges.reshape(-1))
        self.face_edge_indices = t(self.face_edge_np.reshape(-1))
        self.l0 = t(l0)
        self.bending_indices = t(bend.reshape(-1))
        self.bending_l0 = t(bend_l0)
        self.adj_ptr = t(ptr)
        self.adj = t(adj)
        packed = packed_adjacency(ptr, adj)
        self.adj_nbr16, self.adj_rest32 = (t(packed[0]), t(packed[1])) if packed is not None else (None, None)

        V = self.num_verts
        self.x4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.y4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.v4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.fixed = torch.ones(V, dtype=torch.float32, device=dev)
        self.m_inv = t(m_inv)
        self.x0 = t(x)
        self.aabb_min4 = torch.zeros((self.num_faces, 4), dtype=torch.float32, device=dev)
        self.aabb_max4 = torch.zeros((self.num_faces, 4), dtype=torch.float32, device=dev)
        self.box6 = torch.zeros(6, dtype=torch.float32, device=dev)

        self.verts = _Verts()
        self.verts.x = self.x4[:, :3]
        self.verts.y = self.y4[:, :3]
        self.verts.v = self.v4[:, :3]
        self.verts.fixed = self.fixed
        self.verts.m_inv = self.m_inv
        self.verts.x0 = self.x0
        self._load_rest()

    # -- state ---------------------------------------------------------------
    def _load_rest(self):
        self.x4[:, :3] = self.x0
        self.v4.zero_()
        self.refresh_weights()

    def refresh_weights(self):
        """Recompute ``w = fixed * m_inv`` into ``x4.w`` and ``y4.w``."""
        wf = self.fixed * self.m_inv
        self.x4[:, 3] = wf
        self.y4[:, 3] = wf

    def reset(self):
        """``MeshTaichiWrapper.reset`` (``meshTaichiWrapper.py:230-233``):
        ``x = x0``, ``v = 0`` and ``fixed = 0`` (every vertex pinned until
        :meth:`Solver.set_fixed_vertices` is called again)."""
        self.x4[:, :3] = self.x0
        self.v4.zero_()
        self.fixed.zero_()
        self.refresh_weights()

    # -- AABBs (meshTaichiWrapper.py:335-365) -----------------------------------
    def computeAABB_faces(self, padding: float, positions4=None):
        """Face AABBs of ``positions4`` (default ``x``) +- padding into
        ``aabb_min4 / aabb_max4``."""
        p = self.x4 if positions4 is None else positions4
        sx.sx_face_aabbs(ptr(p), ptr(self.face_indices), self.num_faces, float(padding), ptr(self.aabb_min4),
                         ptr(self.aabb_max4), stream_handle())

    def computeAABB(self, padding: float, positions4=None):
        """Vertex AABB +- padding.  The reference returns it to the host; here it
        stays on the device in ``box6`` and views ``(box6[:3], box6[3:])`` are
        returned, so no host synchronisation happens."""
        p = self.x4 if positions4 is None else positions4
        sx.sx_scene_aabb(ptr(p), self.num_verts, float(padding), ptr(self.box6), stream_handle())
        return self.box6[:3], self.box6[3:]

    def positions(self):
        return self.x4[:, :3]

    def bbox_diagonal(self) -> float:
        p = self.x0_np.astype(np.float64)
        return float(np.linalg.norm(p.max(0) - p.min(0)))


def sewing_adjacency(n_verts: int, pairs: np.ndarray):
    """Sewn vertices and their partners for sx_sewing_sweep: sewn[i] has
    partners partner[sptr[i]:sptr[i+1]] in ascending pair index (a pair (a, b)
    lists b at a and a at b)."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    if pairs.size and (pairs.min() < 0 or pairs.max() >= n_verts):
        raise ValueError("sewing pair vertex out of range")
    P = pairs.shape[0]
    owner = np.concatenate([pairs[:, 0], pairs[:, 1]])
    other = np.concatenate([pairs[:, 1], pairs[:, 0]])
    pid = np.concatenate([np.arange(P), np.arange(P)])
    order = np.lexsort((pid, owner))
    owner, other = owner[order], other[order]
    sewn, counts = np.unique(owner, return_counts=True)
    sptr = np.zeros(sewn.shape[0] + 1, dtype=np.int32)
    sptr[1:] = np.cumsum(counts)
    return sewn.astype(np.int32), sptr, other.astype(np.int32)
