"""LBVH broad phase (mirrors framework/collision/lbvh_cell.py).

:class:`LBVH_CELL` keeps the reference's 32^3 cell-grid BVH: the Morton sort and
the Karras hierarchy over the cell centres run once at construction
(``lbvh_cell.py:78-80``); :meth:`LBVH_CELL.build` bins faces into cells and
refits (``lbvh_cell.py:637-653``); :meth:`LBVH_CELL.traverse` is
``traverse_cell_bvh_single`` (``lbvh_cell.py:662-714``) for a batch of points.

:class:`LBVH` is a face-level LBVH over a triangle soup: face-centre Morton
codes, stable radix sort, Karras hierarchy, bottom-up refit, stack traversal.

All work runs in the CUDA library; state lives in torch CUDA tensors.
"""
from __future__ import annotations

import torch

from ._lib import ptr, stream_handle, sx

NUM_CELLS = 32 * 32 * 32


def _as_box6(aabb_min, aabb_max, device):
    """Accept a device box6 tensor, or host/device (min, max) triples."""
    if aabb_max is None and torch.is_tensor(aabb_min) and aabb_min.numel() == 6:
        return aabb_min.to(device=device, dtype=torch.float32).contiguous()
    lo = torch.as_tensor(aabb_min, dtype=torch.float32).reshape(3)
    hi = torch.as_tensor(aabb_max, dtype=torch.float32).reshape(3)
    return torch.cat([lo.to(device), hi.to(device)]).contiguous()


class LBVH_CELL:
    """Cell-grid LBVH (``LBVH_CELL``, lbvh_cell.py:16-80)."""

    def __init__(self, num_leafs: int, device="cuda"):
        dev = torch.device(device)
        self.device = dev
        self.grid_res = (32, 32, 32)
        self.num_cells = NUM_CELLS
        self.num_leafs = int(num_leafs)
        n = NUM_CELLS
        i32 = dict(dtype=torch.int32, device=dev)
        self.cell_morton_codes = torch.empty(n, **i32)      # sorted
        self.cell_ids = torch.empty(n, **i32)               # sorted
        self.child_a = torch.empty(n - 1, **i32)
        self.child_b = torch.empty(n - 1, **i32)
        self.range_l = torch.empty(n - 1, **i32)
        self.range_r = torch.empty(n - 1, **i32)
        self.parent = torch.empty(2 * n - 1, **i32)
        self.sorted_face_ids = torch.empty(max(self.num_leafs, 1), **i32)
        self.prefix_sum_cell = torch.zeros(n, **i32)
        self.num_faces = torch.zeros(2 * n - 1, **i32)
        self.node_min4 = torch.zeros((2 * n - 1, 4), dtype=torch.float32, device=dev)
        self.node_max4 = torch.zeros((2 * n - 1, 4), dtype=torch.float32, device=dev)
        self.face_rec8 = torch.zeros((max(self.num_leafs, 1), 8), dtype=torch.float32, device=dev)
        # grid8 = cell size xyz, largest leaf overhang beyond its cell xyz, 0, 0,
        # then 1024 occupancy words (one bit per cell, a word per z-column)
        self.grid8 = torch.zeros(8 + 1024, dtype=torch.float32, device=dev)
        self.box6 = torch.zeros(6, dtype=torch.float32, device=dev)
        ws = int(sx.sx_cell_bvh_workspace_bytes(self.num_leafs))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=dev)
        self.face_aabb_min4 = None
        self.face_aabb_max4 = None
        sx.sx_cell_bvh_init(ptr(self.cell_morton_codes), ptr(self.cell_ids), ptr(self.child_a),
                            ptr(self.child_b), ptr(self.range_l), ptr(self.range_r), ptr(self.parent),
                            ptr(self.workspace), ws, stream_handle())

    @property
    def origin(self):
        """Grid origin (device tensor view of the build box's min corner)."""
        return self.box6[:3]

    @property
    def cell_size(self):
        """Cell size of the last build (device tensor view)."""
        return self.grid8[:3]

    def build(self, mesh, aabb_min_g=None, aabb_max_g=None, *, face_min4=None, face_max4=None):
        """``LBVH_CELL.build`` (lbvh_cell.py:637-653).

        ``mesh`` supplies the face AABBs (``mesh.aabb_min4 / aabb_max4`` filled by
        ``mesh.computeAABB_faces``) unless ``face_min4/face_max4`` are given; the
        grid box is ``(aabb_min_g, aabb_max_g)`` or a device box6 tensor passed as
        ``aabb_min_g``.  Nothing is read back to the host.
        """
        fmn = face_min4 if face_min4 is not None else mesh.aabb_min4
        fmx = face_max4 if face_max4 is not None else mesh.aabb_max4
        nf = fmn.shape[0]
        if nf != self.num_leafs:
            raise ValueError(f"LBVH_CELL built for {self.num_leafs} faces, got {nf}")
        self.box6.copy_(_as_box6(aabb_min_g, aabb_max_g, self.device))
        self.face_aabb_min4, self.face_aabb_max4 = fmn, fmx
        sx.sx_cell_bvh_build(ptr(fmn), ptr(fmx), nf, ptr(self.box6), ptr(self.child_a), ptr(self.child_b),
                             ptr(self.parent), ptr(self.sorted_face_ids), ptr(self.prefix_sum_cell),
                             ptr(self.num_faces), ptr(self.node_min4), ptr(self.node_max4), ptr(self.face_rec8),
                             ptr(self.grid8), ptr(self.workspace), self.workspace.numel(), stream_handle())

    def traverse(self, points4, padding: float, cap: int, cand, num, status, n_queries=None):
        """``traverse_cell_bvh_single`` for boxes ``points4[i] +- padding``."""
        q = points4.shape[0] if n_queries is None else n_queries
        sx.sx_cell_bvh_traverse(ptr(points4), q, float(padding), ptr(self.grid8), ptr(self.box6),
                                ptr(self.node_min4), ptr(self.node_max4), ptr(self.prefix_sum_cell),
                                ptr(self.face_rec8), int(cap), ptr(cand), ptr(num), ptr(status), stream_handle())

    def traverse_edges(self, edge_indices, n_edges: int, points4, padding: float, cap: int, cand, num, status):
        """``traverse_cell_bvh_single`` for edge boxes: min / max of each edge's
        endpoints in ``points4`` -/+ padding (XPBD.py:217-232)."""
        sx.sx_cell_bvh_traverse_edges(ptr(edge_indices), int(n_edges), ptr(points4), float(padding), ptr(self.grid8),
                                      ptr(self.box6), ptr(self.node_min4), ptr(self.node_max4),
                                      ptr(self.prefix_sum_cell), ptr(self.face_rec8), int(cap), ptr(cand), ptr(num),
                                      ptr(status), stream_handle())


class LBVH:
    """Face-level LBVH over ``n`` faces (one face per leaf).

    ``build(face_min4, face_max4, box6)``: Morton codes of face-AABB centres
    normalised by ``box6``, stable 32-bit radix sort, Karras hierarchy
    (``tie=1``: equal codes ordered by index, always a valid tree; ``tie=0``: the
    reference's rule), bottom-up refit.  ``query(points4, padding, cap)``: stack
    traversal for boxes ``points4[i] +- padding``.
    """

    def __init__(self, num_leafs: int, device="cuda", tie: int = 1, sort_bits: int = 32):
        dev = torch.device(device)
        n = int(num_leafs)
        if n < 1:
            raise ValueError("LBVH needs at least one face")
        self.n = n
        self.device = dev
        self.tie = tie
        self.sort_bits = sort_bits
        i32 = dict(dtype=torch.int32, device=dev)
        self.codes = torch.empty(n, **i32)
        self.sorted_ids = torch.empty(n, **i32)
        m = max(n - 1, 1)
        self.child_a = torch.empty(m, **i32)
        self.child_b = torch.empty(m, **i32)
        self.range_l = torch.empty(m, **i32)
        self.range_r = torch.empty(m, **i32)
        self.parent = torch.empty(2 * n - 1, **i32)
        self.flags = torch.zeros(m, **i32)
        self.status = torch.zeros(1, **i32)
        self.node_min4 = torch.zeros((2 * n - 1, 4), dtype=torch.float32, device=dev)
        self.node_max4 = torch.zeros((2 * n - 1, 4), dtype=torch.float32, device=dev)
        ws = int(sx.sx_radix_sort_workspace_bytes(n))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=dev)

    def morton(self, face_min4, face_max4, box6):
        sx.sx_face_morton(ptr(face_min4), ptr(face_max4), self.n, ptr(box6), ptr(self.codes), ptr(self.sorted_ids),
                          stream_handle())

    def sort(self):
        sx.sx_radix_sort_pairs(ptr(self.codes), ptr(self.sorted_ids), self.n, self.sort_bits, ptr(self.workspace),
                               self.workspace.numel(), stream_handle())

    def hierarchy(self):
        sx.sx_karras_build(ptr(self.codes), self.n, int(self.tie), ptr(self.child_a), ptr(self.child_b),
                           ptr(self.range_l), ptr(self.range_r), ptr(self.parent), stream_handle())

    def refit(self, face_min4, face_max4):
        if self.tie != 1:
            # the reference's tie rule can give a malformed hierarchy on repeated
            # codes: the plain one-thread-per-leaf climb handles that case
            sx.sx_face_bvh_refit(self.n, ptr(self.sorted_ids), ptr(face_min4), ptr(face_max4), ptr(self.child_a),
                                 ptr(self.child_b), ptr(self.parent), ptr(self.node_min4), ptr(self.node_max4),
                                 ptr(self.flags), ptr(self.status), stream_handle())
            return
        sx.sx_face_bvh_refit_tiled(self.n, ptr(self.sorted_ids), ptr(face_min4), ptr(face_max4), ptr(self.child_a),
                                   ptr(self.child_b), ptr(self.parent), ptr(self.range_l), ptr(self.range_r),
                                   ptr(self.node_min4), ptr(self.node_max4), ptr(self.flags), ptr(self.status),
                                   stream_handle())

    def build(self, face_min4, face_max4, box6):
        self.box6 = box6
        self.morton(face_min4, face_max4, box6)
        self.sort()
        self.hierarchy()
        self.refit(face_min4, face_max4)

    def query(self, points4, padding: float, cap: int, cand=None, num=None, status=None):
        q = points4.shape[0]
        if cand is None:
            cand = torch.empty((q, cap), dtype=torch.int32, device=self.device)
        if num is None:
            num = torch.empty(q, dtype=torch.int32, device=self.device)
        if status is None:
            status = self.status
        if q >= self.COHERENT_MIN_QUERIES and getattr(self, "box6", None) is not None:
            # visit the queries in Morton order of the points (normalised by the
            # build's box): a warp's threads then walk nearby parts of the tree
            order = self._query_order(points4, q)
            sx.sx_face_bvh_traverse_ordered(self.n, ptr(points4), q, float(padding), ptr(self.child_a),
                                            ptr(self.child_b), ptr(self.sorted_ids), ptr(self.node_min4),
                                            ptr(self.node_max4), int(cap), ptr(cand), ptr(num), ptr(status),
                                            ptr(order), stream_handle())
            return cand, num
        sx.sx_face_bvh_traverse(self.n, ptr(points4), q, float(padding), ptr(self.child_a), ptr(self.child_b),
                                ptr(self.sorted_ids), ptr(self.node_min4), ptr(self.node_max4), int(cap), ptr(cand),
                                ptr(num), ptr(status), stream_handle())
        return cand, num

    COHERENT_MIN_QUERIES = 1 << 14

    def _query_order(self, points4, q):
        if getattr(self, "_q_n", None) != q:
            i32 = dict(dtype=torch.int32, device=self.device)
            self._q_codes = torch.empty(q, **i32)
            self._q_order = torch.empty(q, **i32)
            self._q_ws = torch.empty(int(sx.sx_radix_sort_workspace_bytes(q)), dtype=torch.uint8, device=self.device)
            self._q_n = q
        sx.sx_face_morton(ptr(points4), ptr(points4), q, ptr(self.box6), ptr(self._q_codes), ptr(self._q_order),
                          stream_handle())
        sx.sx_radix_sort_pairs(ptr(self._q_codes), ptr(self._q_order), q, 30, ptr(self._q_ws), self._q_ws.numel(),
                               stream_handle())
        return self._q_order
