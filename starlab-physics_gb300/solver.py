"""XPBD cloth solver (mirrors ``framework/physics/XPBD.py`` class ``Solver``).

Same constructor arguments, attributes and methods as the reference
(``XPBD.py:9-106``): ``dt, dHat, damping, mu, padding,
enable_collision_handling, enable_velocity_update``; ``forward(n_substeps)``,
``reset()``, ``set_fixed_vertices(mask)``.  Each substep runs on the GPU through
the starxpbd C ABI on the current torch stream; nothing is read back to the
host inside :meth:`forward`.

Options beyond the reference (keyword-only, defaults reproduce the reference):

* ``n_iter`` -- Jacobi iterations per substep.  Each iteration is the
  reference's ``solve_constraints_jacobi_x`` (spring/bending sweep + update, and
  with collisions a contact sweep + update); the broad phase runs in the first
  iteration only and its candidate lists are reused by later iterations.
* ``rebuild`` -- ``"frame"`` builds both cell BVHs on ``x`` once per
  :meth:`forward` call (``XPBD.py:448-458``); ``"substep"`` rebuilds them on ``x``
  at the start of every substep.
* ``bending_on`` -- ``"x"`` evaluates bending pairs on the start-of-substep
  positions as the reference does (``XPBD.py:169``); ``"y"`` evaluates them on
  the current iterate.  With ``n_iter > 1``, ``"x"`` re-applies the same bending
  correction in every iteration, which diverges for stiff bending; iterated
  solves use ``"y"``.
* ``cap`` -- candidate / pair list capacity per query (the reference's 40,
  ``XPBD.py:51``).  Longer lists are truncated and flagged in :attr:`status`.
* ``tol`` / ``tol_relative`` / ``check_every`` (attributes; ``tol=None`` =
  fixed iteration count) -- iterate each substep until the constraint
  residual (RMS of C = |p0 - p1| - l0 over springs and bending pairs,
  :meth:`constraint_residual`) is at most ``tol`` (or, with ``tol_relative``,
  at most ``tol`` times the residual of the substep's predicted positions),
  with ``n_iter`` (even) as the cap.  Every
  ``check_every``-th sweep (even) measures the residual of its input on the GPU;
  once it is below ``tol`` the current pair of iterations completes and the
  remaining ones are skipped on the device, inside the captured graph, with no
  host synchronisation.  Needs ``bending_on="y"`` and the pair-list contacts.
  :meth:`convergence_stats` reads the counters.
* ``set_sewing_pairs(pairs, stiffness)`` -- zero-rest distance constraints
  between vertex pairs (``solve_sewing_constraints_x``, XPBD.py:425-441,
  commented out at XPBD.py:371-372 in the reference), solved after the contact
  update of every Jacobi iteration with k = stiffness * dt^2.
* ``enable_edge_edge`` (attribute, default off as in the reference, whose
  edge-edge calls are commented out) -- per substep an edge broad phase (each
  cloth edge's box against both cell BVHs, XPBD.py:217-232) and per iteration
  the edge-edge contacts __ee_st / __ee_dy (collision_constraints_x.py:313-588)
  over the three edges of every candidate face, added to the contact update.
* ``contact_cull`` (attribute, default on) -- the pair-list contact sweep skips
  a pair whose point-to-triangle-box squared distance exceeds ``dHat * 1.0625``
  before classifying its region.  The distance of every region is at least the
  box distance, so such a pair adds no correction; the skip only saves the
  classification.  Off, every pair is classified as the reference does.
* ``fast_math`` (attribute, default off) -- the sweep's fast arithmetic
  (``sx_jacobi_sweep_mode``: fused multiply-adds, the hardware reciprocal
  square root): within float rounding of the exact sweep, held to the
  substep's position and residual tolerance instead of bit-equality.
* ``gauss_seidel`` (attribute, default off) -- replace the Jacobi spring /
  bending sweep by a colour-ordered Gauss-Seidel sweep (``sx_gs_sweep``): the
  springs and bending pairs are coloured together once
  (``sx_color_edges_greedy``, the reference's colouring,
  ``graph_coloring.py:131-201``) and each colour is projected in place, one
  launch per colour.  This is the parallel Gauss-Seidel path the reference's
  colouring is meant for and which its README marks as work in progress;
  needs ``bending_on="y"`` and a fixed iteration count.

Reference quirks kept on purpose: the stretch springs use
``stiffness_bending * dt^2`` and the bending pairs ``stiffness_stretch * dt^2``
(``XPBD.py:354-355``); bending reads ``x`` not ``y`` (``XPBD.py:169``); ``dHat``
is compared with squared distances; the collision compliance is the constant
``1e8`` (``XPBD.py:367``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import load, ptr, stream_handle, sx
from .lbvh import LBVH_CELL


class Solver:
    def __init__(self, mesh_dy, mesh_st, dHat, stiffness_stretch, stiffness_bending, g, dt, *, n_iter: int = 1,
                 rebuild: str = "frame", cap: int = 40, record_pairs: bool = False, bending_on: str = "x"):
        if rebuild not in ("frame", "substep"):
            raise ValueError("rebuild must be 'frame' or 'substep'")
        if bending_on not in ("x", "y"):
            raise ValueError("bending_on must be 'x' or 'y'")
        if n_iter < 1:
            raise ValueError("n_iter must be >= 1")
        self.mesh_dy = mesh_dy
        self.mesh_st = mesh_st
        self.g = tuple(float(c) for c in g)
        self.dt = float(dt)
        self.dHat = float(dHat)
        self.stiffness_stretch = float(stiffness_stretch)
        self.stiffness_bending = float(stiffness_bending)
        self.damping = 0.001
        self.mu = 0.8
        self.padding = 0.05
        self.enable_velocity_update = False
        self.enable_collision_handling = False
        self.n_iter = int(n_iter)
        self.rebuild = rebuild
        self.compliance_collision = 1e8
        self.bending_on = bending_on
        # vertex-vs-own-triangle contacts (__vt_dy); the reference always runs them
        # when collisions are on
        self.self_collision = True
        self.contact_cull = True
        # the sweep's fast arithmetic (FMA, hardware reciprocal square root):
        # within float rounding of the exact sweep, held to the substep's
        # position and residual tolerance rather than bit-equality
        self.fast_math = False
        # colour-ordered Gauss-Seidel sweeps instead of the Jacobi sweep
        self.gauss_seidel = False
        self._gs = None  # (cons, colour_start as a host int array, n_colors)
        # edge-edge contacts (__ee_st / __ee_dy; commented out in the
        # reference's solver, so off by default)
        self.enable_edge_edge = False
        self._ee = None
        self._sewing = None  # (sewn, sptr, partner, scratch, stiffness)
        # launch configuration of the fixed-count sweep (autotune() picks one)
        self.sweep_variant = 0
        self._packed_sweep = False
        self.packed_form = 0  # the packed sweep staged per block (0) or read from global memory (1)
        # launch configuration of the contact-pair projection (None: the
        # library's default, sx_contact_pairs_project_variant_info lists all)
        self.pairs_variant = None
        # the broad phase on side streams: the per-substep BVH build beside
        # compute_y and the first sweep, the three query sets beside each other
        self.concurrent_broadphase = True
        self._bvh_join = None  # side stream of a BVH build the broad phase must wait for
        self._bp_streams = ((torch.cuda.Stream(device=mesh_dy.device), torch.cuda.Stream(device=mesh_dy.device))
                            if torch.device(mesh_dy.device).type == "cuda" else None)

        self.max_num_verts_dy = mesh_dy.num_verts
        self.max_num_edges_dy = mesh_dy.num_edges
        self.max_num_faces_dy = mesh_dy.num_faces
        self.max_num_verts_st = mesh_st.num_verts if mesh_st is not None else 0
        self.max_num_edges_st = mesh_st.num_edges if mesh_st is not None else 0
        self.max_num_faces_st = mesh_st.num_faces if mesh_st is not None else 0

        dev = mesh_dy.device
        self.device = dev
        self.lbvh_dy = LBVH_CELL(mesh_dy.num_faces, dev)
        self.lbvh_st = LBVH_CELL(mesh_st.num_faces, dev) if mesh_st is not None else None

        Vd, Vs = self.max_num_verts_dy, self.max_num_verts_st
        self.cache_size = int(cap)
        i32 = dict(dtype=torch.int32, device=dev)
        self.vt_st_candidates = torch.zeros((Vd, cap), **i32)
        self.vt_st_candidates_num = torch.zeros(Vd, **i32)
        self.vt_dy_candidates = torch.zeros((Vd, cap), **i32)
        self.vt_dy_candidates_num = torch.zeros(Vd, **i32)
        self.tv_st_candidates = torch.zeros((max(Vs, 1), cap), **i32)
        self.tv_st_candidates_num = torch.zeros(max(Vs, 1), **i32)
        self.status = torch.zeros(1, **i32)
        self._dx_fix = torch.zeros(3 * Vd, dtype=torch.int64, device=dev)
        self._nc = torch.zeros(Vd, **i32)
        self._y_other = torch.zeros_like(mesh_dy.y4)
        # dense contact-pair list (int4 per pair, worst case every candidate slot)
        self._pairs = torch.empty(((2 * Vd + Vs) * cap, 4), **i32)
        self._pairs_ws = torch.zeros(int(sx.sx_contact_pairs_workspace_bytes(Vd, Vs)), dtype=torch.uint8,
                                     device=dev)
        self._static_built_for = None
        self.use_graph = False
        self.tol = None
        self.tol_relative = False
        self.check_every = 4
        self._res_ref = torch.zeros(4, dtype=torch.float64, device=dev)
        self._conv = torch.zeros(8, dtype=torch.int32, device=dev)
        self._res3 = torch.zeros(4, dtype=torch.float64, device=dev)
        self._res_ws = torch.zeros(int(sx.sx_residual_workspace_bytes(Vd)), dtype=torch.uint8, device=dev)
        self._graphs = {}
        self.graph_kernel_launches = 0  # library kernels in the last captured frame
        self.record_pairs = record_pairs
        if record_pairs:
            Q = 2 * Vd + Vs
            self.pair = torch.zeros((Q, cap, 2), **i32)
            self.pair_g = torch.zeros((Q, cap, 4, 4), dtype=torch.float32, device=dev)
            self.pair_schur = torch.zeros((Q, cap), dtype=torch.float32, device=dev)
            self.pair_num = torch.zeros(Q, **i32)
        else:
            self.pair = self.pair_g = self.pair_schur = self.pair_num = None

    # -- reference surface ------------------------------------------------------
    def reset(self):
        """``Solver.reset`` (XPBD.py:108-112)."""
        self.mesh_dy.reset()
        if self.mesh_st is not None:
            self.mesh_st.reset()

    def set_fixed_vertices(self, fixed_vertices):
        """``Solver.set_fixed_vertices`` (XPBD.py:390-395): ``fixed = 0`` where the
        mask is >= 1 (pinned), else 1."""
        m = torch.as_tensor(fixed_vertices, device=self.device)
        self.mesh_dy.fixed.copy_(torch.where(m >= 1, 0.0, 1.0).to(torch.float32))
        self.mesh_dy.refresh_weights()

    def compute_y(self, dt):
        """XPBD.py:116-118."""
        m = self.mesh_dy
        g = self.g
        sx.sx_predict(ptr(m.x4), ptr(m.v4), ptr(m.fixed), ptr(m.y4), m.num_verts, float(dt), g[0], g[1], g[2],
                      stream_handle())

    def spring_sweep(self, dt, iteration: int = 0, loop: int = 0):
        """init_variables + solve_spring_constraints_x + update_dx
        (XPBD.py:345-348, :141-184, :384-387); ping-pongs ``y``.  In tolerance
        mode the sweep of every check_every-th iteration measures the residual;
        ``loop`` is the handle of a device-side loop whose body this is."""
        m = self.mesh_dy
        k_spring = self.stiffness_bending * dt * dt  # XPBD.py:354
        k_bend = self.stiffness_stretch * dt * dt    # XPBD.py:355
        fast = 1 if self.fast_math else 0
        if self.gauss_seidel:
            cons, start, n_colors = self.gs_setup()
            sx.sx_gs_sweep(ptr(m.y4), ptr(cons), start, n_colors, k_spring, k_bend, stream_handle())
            return
        if self.tol is None and self._packed_sweep:
            sx.sx_jacobi_sweep_packed_v(ptr(m.x4), ptr(m.y4), ptr(self._y_other), ptr(m.fixed), ptr(m.adj_ptr),
                                        ptr(m.adj_nbr16), ptr(m.adj_rest32), m.num_verts, k_spring, k_bend,
                                        1 if self.bending_on == "y" else 0, self.packed_form, fast, stream_handle())
        elif self.tol is None:
            sx.sx_jacobi_sweep_mode(ptr(m.x4), ptr(m.y4), ptr(self._y_other), ptr(m.fixed), ptr(m.adj_ptr),
                                    ptr(m.adj), m.num_verts, k_spring, k_bend, 1 if self.bending_on == "y" else 0,
                                    self.sweep_variant, fast, stream_handle())
        else:
            check = 1 if iteration > 0 and iteration % self.check_every == 0 else 0
            sx.sx_jacobi_sweep_checked_mode(ptr(m.x4), ptr(m.y4), ptr(self._y_other), ptr(m.fixed), ptr(m.adj_ptr),
                                            ptr(m.adj), m.num_verts, k_spring, k_bend, iteration, check,
                                            float(self.tol), ptr(self._res_ref) if self.tol_relative else None,
                                            ptr(self._conv), ptr(self._res3), ptr(self._res_ws), self._res_ws.numel(),
                                            loop, self.n_iter, fast, stream_handle())
        self._swap_y()

    def gs_setup(self):
        """Colour the springs and bending pairs together and pack them in
        colour order for the Gauss-Seidel sweep (once per mesh; synchronises
        the host to read the colour offsets, so it runs outside any graph
        capture).  Returns (cons, host colour offsets, number of colours)."""
        if self._gs is not None:
            return self._gs
        if self.bending_on != "y":
            raise ValueError("Gauss-Seidel sweeps need bending_on='y'")
        from .coloring import GraphColoring

        m = self.mesh_dy
        E, B = m.num_edges, m.bending_constraint_count
        pairs = torch.cat([m.edge_indices.view(-1, 2), m.bending_indices.view(-1, 2)]).to(torch.int32).contiguous()
        gc = GraphColoring(m.num_verts, pairs, device=self.device)
        cons = torch.empty((max(E + B, 1), 4), dtype=torch.int32, device=self.device)
        bad = torch.zeros(1, dtype=torch.int32, device=self.device)
        sx.sx_gs_pack(ptr(m.edge_indices), ptr(m.l0), E, ptr(m.bending_indices), ptr(m.bending_l0), B,
                      ptr(gc.sorted_edges_sequence_for_color), ptr(cons), ptr(bad), stream_handle())
        n_colors = int(gc.edges_color[:E + B].max().item()) + 1 if E + B else 0
        offs = gc.color_prefix_sum[:n_colors].cpu().tolist() + [E + B]
        if int(bad.item()):
            raise RuntimeError("sx_gs_pack: constraint id out of range")
        self._gs = (cons, (C.c_int * len(offs))(*offs), n_colors)
        self.gs_colouring = gc
        return self._gs

    def _swap_y(self):
        m = self.mesh_dy
        m.y4, self._y_other = self._y_other, m.y4
        m.verts.y = m.y4[:, :3]

    def build_bvhs(self):
        """XPBD.py:448-458: face AABBs and scene box on ``x``, then both builds.

        The static mesh does not move, so its build is the same every time: it
        runs on the first call and again only after :meth:`mark_static_moved`
        (or when ``padding`` changes)."""
        m = self.mesh_dy
        m.computeAABB_faces(self.padding)
        m.computeAABB(self.padding)
        self.lbvh_dy.build(m, m.box6)
        if self.mesh_st is not None and self._static_built_for != self.padding:
            s = self.mesh_st
            s.computeAABB_faces(self.padding)
            s.computeAABB(self.padding)
            self.lbvh_st.build(s, s.box6)
            self._static_built_for = self.padding

    def mark_static_moved(self):
        """The static mesh's positions changed: rebuild its BVH at the next build
        and drop captured graphs."""
        self._static_built_for = None
        self._graphs.clear()

    def broadphase_lbvh(self):
        """XPBD.py:187-215: three query sets.  They are independent (each
        writes its own candidate lists; the status word takes atomic ORs), so
        the two obstacle query sets run on side streams next to the self
        query set (parallel branches in a captured frame)."""
        m = self.mesh_dy
        cap = self.cache_size
        cur = torch.cuda.current_stream(self.device)
        side = self.concurrent_broadphase and self.mesh_st is not None and self._bp_streams is not None
        if side:
            s1, s2 = self._bp_streams
            s1.wait_stream(cur)
            s2.wait_stream(cur)
        if self.mesh_st is not None:
            with torch.cuda.stream(s1 if side else cur):
                self.lbvh_st.traverse(m.y4, self.padding, cap, self.vt_st_candidates, self.vt_st_candidates_num,
                                      self.status)
            with torch.cuda.stream(s2 if side else cur):
                self.lbvh_dy.traverse(self.mesh_st.x4, self.padding, cap, self.tv_st_candidates,
                                      self.tv_st_candidates_num, self.status)
        if self.self_collision:
            self.lbvh_dy.traverse(m.y4, self.padding, cap, self.vt_dy_candidates, self.vt_dy_candidates_num,
                                  self.status)
        else:
            self.vt_dy_candidates_num.zero_()
        if side:
            cur.wait_stream(s1)
            cur.wait_stream(s2)
        if self.enable_edge_edge:
            ee = self._ensure_ee()
            cap = self.cache_size
            if self.mesh_st is not None:
                self.lbvh_st.traverse_edges(m.edge_indices, m.num_edges, m.y4, self.padding, cap, ee["st_c"],
                                            ee["st_n"], self.status)
            self.lbvh_dy.traverse_edges(m.edge_indices, m.num_edges, m.y4, self.padding, cap, ee["dy_c"], ee["dy_n"],
                                        self.status)

    def _ensure_ee(self):
        """Edge-edge candidate lists (and records with record_pairs): blocks of
        num_edges x cap, allocated on first use."""
        if self._ee is None:
            E, cap, dev = self.mesh_dy.num_edges, self.cache_size, self.device
            i32 = dict(dtype=torch.int32, device=dev)
            ee = {"st_c": torch.zeros((E, cap), **i32), "st_n": torch.zeros(E, **i32),
                  "dy_c": torch.zeros((E, cap), **i32), "dy_n": torch.zeros(E, **i32)}
            if self.record_pairs:
                ee["pair"] = torch.zeros((2 * E, cap, 2), **i32)
                ee["pair_g"] = torch.zeros((2 * E, cap, 4, 4), dtype=torch.float32, device=dev)
                ee["pair_schur"] = torch.zeros((2 * E, cap), dtype=torch.float32, device=dev)
                ee["pair_num"] = torch.zeros(2 * E, **i32)
            self._ee = ee
        return self._ee

    def solve_edge_edge_constraints_x(self, compliance_col=None, iteration: int = 0, gated: bool = True):
        """The edge-edge half of solve_collision_constraints_x (the reference's
        commented-out loop, XPBD.py:266-281): terms added to the contact
        accumulators, applied by the vertex-triangle sweep that follows."""
        m, s = self.mesh_dy, self.mesh_st
        ee = self._ensure_ee()
        c = self.compliance_collision if compliance_col is None else compliance_col
        rec = self.record_pairs
        sx.sx_edge_edge_sweep(m.num_edges, ptr(m.edge_indices), ptr(s.edge_indices) if s is not None else None,
                              ptr(m.face_edge_indices), ptr(s.face_edge_indices) if s is not None else None, ptr(m.y4),
                              ptr(s.x4) if s is not None else None, ptr(m.fixed), ptr(m.m_inv), self.dHat, float(c),
                              self.cache_size, ptr(ee["st_c"]) if s is not None else None,
                              ptr(ee["st_n"]) if s is not None else None, ptr(ee["dy_c"]), ptr(ee["dy_n"]),
                              ptr(self._dx_fix), ptr(self._nc), ptr(ee["pair"]) if rec else None,
                              ptr(ee["pair_g"]) if rec else None, ptr(ee["pair_schur"]) if rec else None,
                              ptr(ee["pair_num"]) if rec else None, ptr(self.status),
                              ptr(self._conv) if self.tol is not None and gated else None, iteration,
                              stream_handle())

    def build_contact_pairs(self):
        """Flatten this substep's candidate lists into the dense pair list used by
        every iteration's contact sweep (not needed when pair records are kept)."""
        m = self.mesh_dy
        s = self.mesh_st
        sx.sx_contact_pairs_build(m.num_verts, s.num_verts if s is not None else 0, ptr(m.face_indices),
                                  ptr(s.face_indices) if s is not None else None, self.cache_size,
                                  ptr(self.vt_st_candidates), ptr(self.vt_st_candidates_num),
                                  ptr(self.vt_dy_candidates), ptr(self.vt_dy_candidates_num),
                                  ptr(self.tv_st_candidates), ptr(self.tv_st_candidates_num), ptr(self._pairs),
                                  self._pairs.shape[0], ptr(self._pairs_ws), self._pairs_ws.numel(),
                                  stream_handle())

    def solve_collision_constraints_x(self, compliance_col=None, iteration: int = 0, gated: bool = True):
        """XPBD.py:237-264 followed by update_dx (XPBD.py:384-387)."""
        m = self.mesh_dy
        s = self.mesh_st
        c = self.compliance_collision if compliance_col is None else compliance_col
        if self.enable_edge_edge:
            self.solve_edge_edge_constraints_x(c, iteration, gated)
        if not self.record_pairs:
            conv = ptr(self._conv) if self.tol is not None and gated else None
            if self.pairs_variant is None:
                sx.sx_contact_pairs_sweep(m.num_verts, s.num_verts if s is not None else 0, ptr(self._pairs),
                                          ptr(self._pairs_ws), ptr(m.y4), ptr(s.x4) if s is not None else None,
                                          ptr(m.fixed), ptr(m.m_inv), self.dHat, float(c), self.contact_cull_d2(),
                                          ptr(self._dx_fix), ptr(self._nc), ptr(self.status), conv, iteration,
                                          stream_handle())
            else:
                sx.sx_contact_pairs_project_v(m.num_verts, s.num_verts if s is not None else 0, ptr(self._pairs),
                                              ptr(self._pairs_ws), ptr(m.y4), ptr(s.x4) if s is not None else None,
                                              ptr(m.fixed), ptr(m.m_inv), self.dHat, float(c),
                                              self.contact_cull_d2(), ptr(self._dx_fix), ptr(self._nc),
                                              ptr(self.status), conv, iteration, int(self.pairs_variant),
                                              stream_handle())
                sx.sx_contact_apply(m.num_verts, ptr(m.y4), ptr(m.fixed), ptr(self._dx_fix), ptr(self._nc), conv,
                                    iteration, stream_handle())
            return
        sx.sx_collision_sweep(m.num_verts, s.num_verts if s is not None else 0, ptr(m.face_indices),
                              ptr(s.face_indices) if s is not None else None, ptr(m.y4),
                              ptr(s.x4) if s is not None else None, ptr(m.fixed), ptr(m.m_inv), self.dHat, float(c),
                              self.cache_size, ptr(self.vt_st_candidates), ptr(self.vt_st_candidates_num),
                              ptr(self.vt_dy_candidates), ptr(self.vt_dy_candidates_num),
                              ptr(self.tv_st_candidates), ptr(self.tv_st_candidates_num), ptr(self._dx_fix),
                              ptr(self._nc), ptr(self.pair), ptr(self.pair_g), ptr(self.pair_schur),
                              ptr(self.pair_num), ptr(self.status), stream_handle())

    def solve_constraints_jacobi_x(self, dt, first_iteration: bool = True, iteration: int = 0, loop: int = 0,
                                   in_loop: bool = False):
        """XPBD.py:350-369 (broad phase only in the first iteration of a substep).
        ``in_loop``: part of the body of a device-side loop (kernels not gated)."""
        self.spring_sweep(dt, iteration, loop)
        if self.enable_collision_handling:
            if self.mesh_st is None:
                # the reference always has a static mesh when collisions are on
                self.vt_st_candidates_num.zero_()
            if first_iteration:
                if self._bvh_join is not None:
                    torch.cuda.current_stream(self.device).wait_stream(self._bvh_join)
                    self._bvh_join = None
                self.broadphase_lbvh()
                if not self.record_pairs:
                    self.build_contact_pairs()
            self.solve_collision_constraints_x(iteration=iteration, gated=not in_loop)
        self.solve_sewing_constraints_x(dt)

    def set_sewing_pairs(self, pairs, stiffness: float):
        """Sew vertex pairs (an int array [P, 2]); None or an empty array removes
        the sewing."""
        from .mesh import sewing_adjacency

        if pairs is None or len(pairs) == 0:
            self._sewing = None
            self._graphs.clear()
            return
        sewn, sptr, partner = sewing_adjacency(self.mesh_dy.num_verts, np.asarray(pairs))
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.device)  # noqa: E731
        self._sewing = (t(sewn), t(sptr), t(partner),
                        torch.zeros((sewn.shape[0], 4), dtype=torch.float32, device=self.device), float(stiffness))
        self._graphs.clear()

    def solve_sewing_constraints_x(self, dt):
        """XPBD.py:425-441 followed by update_dx (no-op without sewing pairs)."""
        if self._sewing is None:
            return
        sewn, sptr, partner, scratch, stiff = self._sewing
        m = self.mesh_dy
        sx.sx_sewing_sweep(ptr(m.y4), ptr(m.fixed), sewn.shape[0], ptr(sewn), ptr(sptr), ptr(partner),
                           stiff * dt * dt, ptr(scratch), stream_handle())

    def compute_velocity_update_x(self, dt):
        """compute_velocity (XPBD.py:341-343) then update_x (XPBD.py:333-337)."""
        m = self.mesh_dy
        sx.sx_velocity_update(ptr(m.x4), ptr(m.y4), ptr(m.v4), ptr(m.fixed), m.num_verts, self.damping, float(dt),
                              stream_handle())

    def solve_constraints_v(self):
        """solve_constraints_v (XPBD.py:374-381): velocity-level contact and
        friction (mu) over the pair records of the last contact sweep, then
        update_dv.  Needs the records: ``record_pairs=True``."""
        if not self.record_pairs:
            raise ValueError("the velocity-level contact pass reads pair records: construct with record_pairs=True")
        m, s = self.mesh_dy, self.mesh_st
        sx.sx_velocity_contacts(m.num_verts, s.num_verts if s is not None else 0, ptr(m.face_indices),
                                ptr(s.face_indices) if s is not None else None, self.cache_size, ptr(self.pair),
                                ptr(self.pair_g), ptr(self.pair_schur), ptr(self.pair_num), ptr(m.v4),
                                ptr(s.v4) if s is not None else None, ptr(m.fixed), ptr(m.m_inv),
                                ptr(s.m_inv) if s is not None else None, float(self.mu), ptr(self._dx_fix),
                                ptr(self._nc), ptr(self.status), stream_handle())

    def substep(self, dt_sub):
        if self.enable_collision_handling and self.rebuild == "substep":
            if self.concurrent_broadphase and self._bp_streams is not None:
                # the build reads only x: it runs beside compute_y and the first
                # sweep, and the broad phase waits for it
                cur = torch.cuda.current_stream(self.device)
                side = self._bp_streams[0]
                side.wait_stream(cur)
                with torch.cuda.stream(side):
                    self.build_bvhs()
                self._bvh_join = side
            else:
                self.build_bvhs()
        self.compute_y(dt_sub)
        ce = self.check_every
        if self.tol is not None:
            self._check_tol_mode()
            sx.sx_convergence_begin(ptr(self._conv), ce, 0, stream_handle())
            if self.tol_relative:
                self.constraint_residual("y", out=self._res_ref)
        if self.tol is not None and self.n_iter > ce and torch.cuda.is_current_stream_capturing():
            # inside a graph: the first block of iterations, then the rest as a
            # device-side loop that stops once converged
            for it in range(ce):
                self.solve_constraints_jacobi_x(dt_sub, first_iteration=(it == 0), iteration=it)
            if getattr(self, "_body_stream", None) is None:
                self._body_stream = torch.cuda.Stream(device=self.device)
            h, ctx = C.c_ulonglong(0), C.c_void_p(None)
            sx.sx_loop_begin(stream_handle(), self._body_stream.cuda_stream, C.addressof(h), C.addressof(ctx))
            try:
                with torch.cuda.stream(self._body_stream):
                    for k in range(ce):
                        self.solve_constraints_jacobi_x(dt_sub, first_iteration=False, iteration=ce + k,
                                                        loop=h.value if k == 0 else 0, in_loop=True)
            finally:
                sx.sx_loop_end(ctx)
        else:
            for it in range(self.n_iter):
                self.solve_constraints_jacobi_x(dt_sub, first_iteration=(it == 0), iteration=it)
        if self.enable_velocity_update and self.enable_collision_handling:
            # compute_velocity, solve_constraints_v, update_x (XPBD.py:465-469)
            m = self.mesh_dy
            sx.sx_compute_velocity(ptr(m.x4), ptr(m.y4), ptr(m.v4), ptr(m.fixed), m.num_verts, self.damping,
                                   float(dt_sub), stream_handle())
            self.solve_constraints_v()
            sx.sx_update_x(ptr(m.x4), ptr(m.v4), m.num_verts, float(dt_sub), stream_handle())
        else:
            self.compute_velocity_update_x(dt_sub)

    def forward(self, n_substeps: int):
        """``Solver.forward`` (XPBD.py:443-469).

        With ``use_graph = True`` the whole frame is captured once into a CUDA
        graph (per set of parameters that the kernels receive by value) and
        replayed on later calls; results are identical to the eager path."""
        if self.enable_edge_edge and self.enable_collision_handling:
            self._ensure_ee()  # allocated outside any capture
        if self.gauss_seidel:
            self.gs_setup()  # colours read back outside any capture
        if not self.use_graph:
            self._forward_eager(n_substeps)
            return
        key = self._graph_key(n_substeps)
        g = self._graphs.get(key)
        if g is None:
            g = self._capture(n_substeps)
            self._graphs[key] = g
        g.replay()

    CULL_MARGIN = 1.0625

    def autotune(self, n_substeps: int | None = None, finalists: int = 4, reps: int = 3):
        """Time every launch configuration of the sweep on this mesh and keep
        the fastest (identical results).  With ``n_substeps``, the `finalists`
        fastest alone are timed again in whole frames (the state restored after
        each), which decides: on a small mesh the isolated times are within a
        few percent of each other and the frame's other launches change the
        ranking.  Returns (variant, isolated times in ms)."""
        from .autotune import tune_sweep, variants

        m = self.mesh_dy
        dt = self.dt / 10
        best, times = tune_sweep(m.x4, m.y4, m.fixed, m.adj_ptr, m.adj, m.num_verts, self.stiffness_bending * dt * dt,
                                 self.stiffness_stretch * dt * dt, 1 if self.bending_on == "y" else 0,
                                 packed=(m.adj_nbr16, m.adj_rest32), fast=self.fast_math)
        nv = len(variants())

        def choose(v):
            self._packed_sweep = v >= nv
            self.packed_form = v - nv if self._packed_sweep else 0
            self.sweep_variant = 0 if self._packed_sweep else v

        if n_substeps is not None and finalists > 1:
            x0, v0 = m.x4.clone(), m.v4.clone()
            frame_ms = {}
            for v in [int(i) for i in np.argsort(times)[:finalists]]:
                choose(v)
                self.forward(n_substeps)  # captures this variant's frame when use_graph is set
                t_best = None
                for _ in range(reps):
                    m.x4.copy_(x0)
                    m.v4.copy_(v0)
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record()
                    self.forward(n_substeps)
                    b.record()
                    torch.cuda.synchronize()
                    t = a.elapsed_time(b)
                    t_best = t if t_best is None else min(t_best, t)
                frame_ms[v] = t_best
                m.x4.copy_(x0)
                m.v4.copy_(v0)
            best = min(frame_ms, key=frame_ms.get)
        choose(best)
        return best, times

    def autotune_contacts(self, n_substeps: int, reps: int = 3):
        """Time whole frames with every launch configuration of the contact-pair
        projection (identical results) and keep the fastest: timed alone on one
        state the ranking differs from the frame's.  The state is restored after
        every frame.  Returns (variant, frame times in ms)."""
        if not (self.enable_collision_handling and not self.record_pairs):
            return self.pairs_variant, []
        m = self.mesh_dy
        x0, v0 = m.x4.clone(), m.v4.clone()
        times = []
        for v in range(int(sx.sx_contact_pairs_project_variants())):
            self.pairs_variant = v
            self.forward(n_substeps)  # captures the frame's graph for this variant when use_graph is set
            best = None
            for _ in range(reps):
                m.x4.copy_(x0)
                m.v4.copy_(v0)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self.forward(n_substeps)
                b.record()
                torch.cuda.synchronize()
                t = a.elapsed_time(b)
                best = t if best is None else min(best, t)
            times.append(best)
            m.x4.copy_(x0)
            m.v4.copy_(v0)
        self.pairs_variant = int(np.argmin(times))
        torch.cuda.synchronize()
        return self.pairs_variant, times

    @property
    def packed_sweep(self) -> bool:
        """The fixed-count sweep runs over the packed, shared-memory-staged
        adjacency (``sx_jacobi_sweep_packed``; identical results)."""
        return self._packed_sweep

    @packed_sweep.setter
    def packed_sweep(self, on: bool):
        if on and self.mesh_dy.adj_nbr16 is None:
            raise ValueError("the packed adjacency needs neighbour offsets within 16 bits")
        self._packed_sweep = bool(on)

    def _check_tol_mode(self):
        if self.gauss_seidel:
            raise ValueError("iterating to a tolerance runs the Jacobi sweep (gauss_seidel must be off)")
        if self._sewing is not None:
            raise ValueError("iterating to a tolerance does not support sewing pairs")
        if self.bending_on != "y":
            raise ValueError("iterating to a tolerance needs bending_on='y'")
        if self.record_pairs:
            raise ValueError("iterating to a tolerance needs the pair-list contacts (record_pairs=False)")
        if self.check_every < 2 or self.check_every % 2 or self.n_iter % self.check_every:
            raise ValueError("iterating to a tolerance needs an even check_every and n_iter a multiple of it")

    def convergence_stats(self, reset: bool = False) -> dict:
        """Counters of the tolerance mode since the last reset (host sync):
        converged substeps, their mean stop iteration (the sweep whose input met
        the tolerance; two more iterations run after it) and the last residual
        checked."""
        c = self._conv.cpu().tolist()
        r = self._res3.cpu().tolist()
        out = {"converged_substeps": c[4], "mean_stop_iteration": c[3] / c[4] if c[4] else None,
               "last_residual": r[2]}
        if reset:
            sx.sx_convergence_begin(ptr(self._conv), self.check_every, 1, stream_handle())
        return out

    def contact_cull_d2(self) -> float:
        """Box-distance threshold of the pair-list sweep (0 = classify every pair)."""
        return self.dHat * self.CULL_MARGIN if self.contact_cull else 0.0

    def _forward_eager(self, n_substeps: int):
        dt_sub = self.dt / n_substeps
        if self.enable_collision_handling and self.rebuild == "frame":
            self.build_bvhs()
        for _ in range(n_substeps):
            self.substep(dt_sub)

    def _graph_key(self, n_substeps):
        return (n_substeps, self.dt, self.dHat, self.damping, self.padding, self.g, self.stiffness_stretch,
                self.stiffness_bending, self.enable_collision_handling, self.n_iter, self.bending_on, self.rebuild,
                self.compliance_collision, self.self_collision, self.contact_cull, self.fast_math,
                self.gauss_seidel, self.sweep_variant, self._packed_sweep, self.packed_form,
                self.pairs_variant, self.concurrent_broadphase, self.enable_edge_edge,
                self.enable_velocity_update, self.mu, self.tol,
                self.tol_relative,
                self.check_every,
                self.mesh_dy.y4.data_ptr())

    def _capture(self, n_substeps):
        m = self.mesh_dy
        y_start = m.y4
        if self.enable_collision_handling and self.mesh_st is not None and self._static_built_for != self.padding:
            self.build_bvhs()  # the static build happens once, outside the graph
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        lib = load()
        n0 = lib.sx_kernel_launches()
        with torch.cuda.graph(g, stream=side):
            self._forward_eager(n_substeps)
            if m.y4 is not y_start:
                # an odd number of sweeps left y in the other buffer: copy it back
                # so that every replay starts from the same buffer assignment
                y_start.copy_(m.y4)
                self._swap_y()
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph_kernel_launches = lib.sx_kernel_launches() - n0
        return g

    # -- diagnostics ---------------------------------------------------------------
    def constraint_residual(self, positions: str = "x", out=None):
        """RMS stretch/bending violation on the GPU (``sx_constraint_residual``):
        C = |p0 - p1| - l0 in float as the sweep evaluates it, summed in float
        per vertex and per block and in FP64 across blocks.

        ``positions`` is ``"x"`` or ``"y"``.  Returns a device tensor
        ``[sum C^2, count, rms]`` (float64) over the adjacency entries (each
        constraint counted from both endpoints); no host synchronisation unless
        the caller reads it."""
        m = self.mesh_dy
        p = m.x4 if positions == "x" else m.y4
        if out is None:
            out = torch.empty(3, dtype=torch.float64, device=self.device)
        sx.sx_constraint_residual(ptr(p), ptr(m.adj_ptr), ptr(m.adj), m.num_verts, ptr(out), ptr(self._res_ws),
                                  self._res_ws.numel(), stream_handle())
        return out

    def system_energy(self, out=None):
        """Kinetic, gravitational and elastic energy of the cloth in FP64
        (``sx_system_energy``; no counterpart in the reference): a device
        tensor of three doubles, from ``x`` and ``v``.  The elastic term uses the
        stiffnesses the sweep applies to each constraint type (springs
        ``stiffness_bending``, bending pairs ``stiffness_stretch``, the
        reference's pairing, XPBD.py:354-355)."""
        m = self.mesh_dy
        if out is None:
            out = torch.zeros(3, dtype=torch.float64, device=self.device)
        if getattr(self, "_energy_ws", None) is None:
            self._energy_ws = torch.zeros(int(sx.sx_energy_workspace_bytes(m.num_verts)), dtype=torch.uint8,
                                          device=self.device)
        sx.sx_system_energy(ptr(m.x4), ptr(m.v4), ptr(m.m_inv), ptr(m.adj_ptr), ptr(m.adj), m.num_verts,
                            float(self.stiffness_bending), float(self.stiffness_stretch), *self.g, ptr(out),
                            ptr(self._energy_ws), self._energy_ws.numel(), stream_handle())
        return out

    def contact_pair_count(self) -> int:
        """Pairs in the current contact pair list (host sync): the counts sit in
        the last 256 bytes of the pair-list workspace, {end of vertex-vs-static
        pairs, end of vertex-vs-cloth pairs, total}."""
        return int(self._pairs_ws[-256:].view(torch.int32)[2].item())

    def status_flags(self) -> int:
        """Accumulated device status bits (host sync)."""
        return int(self.status.item())
