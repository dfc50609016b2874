"""Many independent cloths, each with its own static obstacle, in one solver.

The reference batches by concatenating meshes into one (``concat.py:11-58``,
``Scenes/concat_test.py:20-41``), sharing one BVH.  Here instances are
concatenated with per-instance offset tables (vertices, faces, obstacle
vertices and faces) while every instance keeps the candidate semantics of its
own pair of cell BVHs.  One launch per kernel covers every instance:

* the Jacobi sweep runs over the concatenated vertex-centric adjacency (a
  vertex only has neighbours in its own instance);
* obstacle contacts (``__vt_st`` and ``__tv_st``) use per-instance grids and
  brute-force candidate tests, which give the candidate sets the reference's
  traversal gives (``sx_batched_obstacle_broadphase``);
* self contact between a cloth and itself (``__vt_dy``) is not part of the
  batched workload (obstacle contacts only).

Each instance's result equals that instance alone in :class:`Solver` with
``self_collision = False`` and ``rebuild = "substep"``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import load, ptr, stream_handle, sx
from .mesh import bending_pairs, box_mesh, constraint_adjacency, edges_from_faces, grid_cloth, inverse_masses, \
    packed_adjacency, rest_lengths


@dataclass
class Instance:
    x: np.ndarray          # float32[V,3] rest positions
    faces: np.ndarray      # int32[F,3]
    pinned: np.ndarray     # vertex ids (local) with fixed = 0
    obstacle_x: np.ndarray
    obstacle_faces: np.ndarray


def batched_scene(n_instances: int = 512, seed: int = 0, n_min: int = 16, n_max: int = 128, spacing: float = 1.5):
    """Seeded batch: instance i is an N_i x N_i cloth (N_i uniform in [n_min, n_max])
    on the unit square at height 1, jittered +-1e-4, corners at y = 1 pinned,
    over its own box (side 0.5, centre randomised around (0.5, 0.5, 0.3)); the
    instances sit on a grid of `spacing` so that they never touch."""
    rng = np.random.default_rng(seed)
    cols = int(np.ceil(np.sqrt(n_instances)))
    out = []
    for i in range(n_instances):
        n = int(rng.integers(n_min, n_max + 1))
        ox, oy = spacing * (i % cols), spacing * (i // cols)
        x, f = grid_cloth(n, origin=(ox, oy), height=1.0)
        x = (x + rng.uniform(-1e-4, 1e-4, size=x.shape).astype(np.float32)).astype(np.float32)
        c = (ox + 0.5 + rng.uniform(-0.2, 0.2), oy + 0.5 + rng.uniform(-0.2, 0.2), 0.3 + rng.uniform(0.0, 0.3))
        bx, bf = box_mesh(0.5, center=c)
        out.append(Instance(x, f, np.array([(n - 1) * n, n * n - 1]), bx, bf))
    return out


def shard_instances(instances, rank: int, world: int):
    """The instances rank `rank` of `world` simulates: a greedy split by
    weight V + constraints (springs and bending pairs, about 6 V for a grid
    cloth), largest first onto the lightest rank.  Instances are independent,
    so ranks exchange nothing per substep.  Returns the instance indices in
    ascending order."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    w = []
    for inst in instances:
        V = int(np.asarray(inst.x).shape[0])
        F = int(np.asarray(inst.faces).shape[0])
        w.append(V + 3 * F)  # V + springs (~1.5 F) + bending pairs (~1.5 F)
    load = [0] * world
    owner = [0] * len(instances)
    for i in sorted(range(len(instances)), key=lambda k: (-w[k], k)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += w[i]
    return [i for i in range(len(instances)) if owner[i] == rank]


class BatchedSolver:
    """XPBD substep for a batch of independent cloths with obstacles."""

    def __init__(self, instances, dHat, stiffness_stretch, stiffness_bending, g, dt, *, n_iter=20, cap=40,
                 bending_on="y", padding=8e-3, damping=0.001, device="cuda"):
        dev = torch.device(device)
        self.device = dev
        self.n_instances = len(instances)
        self.dHat = float(dHat)
        self.stiffness_stretch = float(stiffness_stretch)
        self.stiffness_bending = float(stiffness_bending)
        self.g = tuple(float(c) for c in g)
        self.dt = float(dt)
        self.n_iter = int(n_iter)
        self.cap = int(cap)
        self.bending_on = bending_on
        self.padding = float(padding)
        self.damping = float(damping)
        self.compliance_collision = 1e8
        self.use_graph = False
        self._graphs = {}
        self.graph_kernel_launches = 0

        xs, fs, es, l0s, bs, bl0s, minvs, fixeds = [], [], [], [], [], [], [], []
        oxs, ofs = [], []
        vptr, fptr, optr, ofptr = [0], [0], [0], [0]
        for inst in instances:
            x = np.asarray(inst.x, np.float32)
            f = np.asarray(inst.faces, np.int32)
            e = edges_from_faces(f)
            l0 = rest_lengths(x, e)
            b = bending_pairs(f)
            bl0 = rest_lengths(x, b) if b.shape[0] else np.zeros(0, np.float32)
            v0 = vptr[-1]
            xs.append(x)
            fs.append(f + v0)
            es.append(e + v0)
            l0s.append(l0)
            bs.append(b + v0)
            bl0s.append(bl0)
            minvs.append(inverse_masses(x.shape[0], e, l0))
            fx = np.ones(x.shape[0], np.float32)
            fx[np.asarray(inst.pinned, np.int64)] = 0.0
            fixeds.append(fx)
            vptr.append(v0 + x.shape[0])
            fptr.append(fptr[-1] + f.shape[0])
            ox = np.asarray(inst.obstacle_x, np.float32)
            of = np.asarray(inst.obstacle_faces, np.int32)
            if of.shape[0] > 32:
                raise ValueError("an obstacle may have at most 32 faces")
            ofs.append(of + optr[-1])
            oxs.append(ox)
            optr.append(optr[-1] + ox.shape[0])
            ofptr.append(ofptr[-1] + of.shape[0])
        x = np.concatenate(xs)
        faces = np.concatenate(fs)
        edges = np.concatenate(es)
        l0 = np.concatenate(l0s)
        bend = np.concatenate(bs)
        bl0 = np.concatenate(bl0s)
        m_inv = np.concatenate(minvs)
        fixed = np.concatenate(fixeds)
        V = x.shape[0]
        self.num_verts = V
        self.num_faces = faces.shape[0]
        adj_ptr, adj = constraint_adjacency(V, edges, l0, bend, bl0)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        self.vptr_np = np.asarray(vptr, np.int32)
        self.fptr_np = np.asarray(fptr, np.int32)
        self.vptr, self.fptr = t(self.vptr_np), t(self.fptr_np)
        self.vinst = t(np.repeat(np.arange(self.n_instances, dtype=np.int32), np.diff(self.vptr_np)))
        self.faces = t(faces.reshape(-1))
        self.adj_ptr, self.adj = t(adj_ptr), t(adj)
        packed = packed_adjacency(adj_ptr, adj)
        self.adj_nbr16, self.adj_rest32 = (t(packed[0]), t(packed[1])) if packed is not None else (None, None)
        self.fixed, self.m_inv = t(fixed), t(m_inv)
        self.x4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.x4[:, :3] = t(x)
        wf = self.fixed * self.m_inv
        self.x4[:, 3] = wf
        self.y4 = self.x4.clone()
        self._y_other = torch.zeros_like(self.x4)
        self.v4 = torch.zeros_like(self.x4)
        self.fmin4 = torch.zeros((self.num_faces, 4), dtype=torch.float32, device=dev)
        # boxes of 32-face chunks, for the obstacle broad phase
        self.cmin4 = torch.zeros(((self.num_faces + 31) // 32, 4), dtype=torch.float32, device=dev)
        self.cmax4 = torch.zeros_like(self.cmin4)
        self.fmax4 = torch.zeros_like(self.fmin4)
        self.cl_box6 = torch.zeros((self.n_instances, 6), dtype=torch.float32, device=dev)
        # obstacles: static; their face boxes and grids are computed once
        ox = np.concatenate(oxs)
        self.n_ob_verts = ox.shape[0]
        self.xs4 = torch.zeros((self.n_ob_verts, 4), dtype=torch.float32, device=dev)
        self.xs4[:, :3] = t(ox)
        self.ob_faces = t(np.concatenate(ofs).reshape(-1))
        self.optr = t(np.asarray(optr, np.int32))
        self.ob_fptr = t(np.asarray(ofptr, np.int32))
        self.svinst = t(np.repeat(np.arange(self.n_instances, dtype=np.int32), np.diff(np.asarray(optr))))
        self.ob_fmin4 = torch.zeros((int(ofptr[-1]), 4), dtype=torch.float32, device=dev)
        self.ob_fmax4 = torch.zeros_like(self.ob_fmin4)
        self.ob_box6 = torch.zeros((self.n_instances, 6), dtype=torch.float32, device=dev)
        self._ob_built_for = None
        self.vmask = torch.zeros(V, dtype=torch.int32, device=dev)
        self.tv_cand = torch.zeros((max(self.n_ob_verts, 1), cap), dtype=torch.int32, device=dev)
        self.tv_num = torch.zeros(max(self.n_ob_verts, 1), dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._dx_fix = torch.zeros(3 * V, dtype=torch.int64, device=dev)
        self._nc = torch.zeros(V, dtype=torch.int32, device=dev)
        # learned warm start (learned.WarmStart) run after each prediction
        self.warm = None
        # launch configuration of the fixed-count sweep (autotune() picks one)
        self.sweep_variant = 0
        # the sweep over the packed, shared-memory-staged adjacency
        # (sx_jacobi_sweep_packed; same results; autotune() decides)
        self._packed_sweep = False
        self.packed_form = 0  # the packed sweep staged per block (0) or read from global memory (1)
        # the sweep's fast arithmetic (Solver.fast_math)
        self.fast_math = False
        # one persistent launch per substep (sx_batched_substep) instead of a
        # graph of grid-wide launches; fixed iteration counts only (iterating
        # to a residual keeps the grid-wide form).  persistent_variant: its
        # launch configuration (autotune_persistent() picks one)
        self.persistent = False
        self.persistent_variant = 0
        self._pargs = None
        self._vsizes = np.diff(self.vptr_np)
        # iterate to a residual (Solver.tol): n_iter is then the cap
        self.tol = None
        self.tol_relative = False
        self.check_every = 4
        self._res_ref = torch.zeros(4, dtype=torch.float64, device=dev)
        self._conv = torch.zeros(8, dtype=torch.int32, device=dev)
        self._res3 = torch.zeros(4, dtype=torch.float64, device=dev)
        self._res_ws = torch.zeros(int(sx.sx_residual_workspace_bytes(V)), dtype=torch.uint8, device=dev)

    # -- pieces ------------------------------------------------------------------
    def _static_obstacles(self):
        s = stream_handle()
        sx.sx_face_aabbs(ptr(self.xs4), ptr(self.ob_faces), self.ob_fmin4.shape[0], self.padding, ptr(self.ob_fmin4),
                         ptr(self.ob_fmax4), s)
        sx.sx_segment_aabbs(ptr(self.xs4), ptr(self.optr), self.n_instances, self.padding, ptr(self.ob_box6), s)
        self._ob_built_for = self.padding

    def _swap_y(self):
        self.y4, self._y_other = self._y_other, self.y4

    def _persistent_buffers(self):
        """Instance order (largest first), per-instance chunk offsets, their
        chunk boxes and the work queue of the persistent substep."""
        if self._pargs is None:
            dev = self.device
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
            nf = np.diff(self.fptr_np)
            cptr = np.zeros(self.n_instances + 1, np.int32)
            cptr[1:] = np.cumsum((nf + 31) // 32)
            order = np.argsort(-self._vsizes, kind="stable").astype(np.int32)
            self._p_order, self._p_cptr = t(order), t(cptr)
            self._p_cmin4 = torch.zeros((max(int(cptr[-1]), 1), 4), dtype=torch.float32, device=dev)
            self._p_cmax4 = torch.zeros_like(self._p_cmin4)
            self._p_queue = torch.zeros(2, dtype=torch.int32, device=dev)
            self._pargs = True

    def _persistent_substep(self, dt, predict: bool):
        """One substep as a single persistent launch (sx_batched_substep)."""
        from ._lib import SxBatchedSubstep

        self._persistent_buffers()
        g = self.g
        a = SxBatchedSubstep()
        a.n_inst, a.n_iter, a.predict, a.cap = self.n_instances, self.n_iter, 1 if predict else 0, self.cap
        for name, tns in (("order", self._p_order), ("vptr", self.vptr), ("fptr", self.fptr), ("cptr", self._p_cptr),
                          ("optr", self.optr), ("ob_fptr", self.ob_fptr), ("x4", self.x4), ("y4", self.y4),
                          ("y_other4", self._y_other), ("v4", self.v4), ("fixed", self.fixed), ("m_inv", self.m_inv),
                          ("adj_ptr", self.adj_ptr), ("adj", self.adj), ("faces", self.faces),
                          ("ob_faces", self.ob_faces), ("xs4", self.xs4), ("fmin4", self.fmin4),
                          ("fmax4", self.fmax4), ("cmin4", self._p_cmin4), ("cmax4", self._p_cmax4),
                          ("cl_box6", self.cl_box6), ("ob_box6", self.ob_box6), ("ob_fmin4", self.ob_fmin4),
                          ("ob_fmax4", self.ob_fmax4), ("vmask", self.vmask), ("tv_cand", self.tv_cand),
                          ("tv_num", self.tv_num), ("dx_fix", self._dx_fix), ("nc", self._nc),
                          ("status", self.status), ("queue", self._p_queue)):
            setattr(a, name, ptr(tns))
        if self._packed_sweep:
            a.adj_nbr16, a.adj_rest32 = ptr(self.adj_nbr16), ptr(self.adj_rest32)
        a.padding, a.dt, a.gx, a.gy, a.gz = self.padding, float(dt), g[0], g[1], g[2]
        a.k_spring = self.stiffness_bending * dt * dt  # XPBD.py:354
        a.k_bend = self.stiffness_stretch * dt * dt    # XPBD.py:355
        a.dHat, a.compliance, a.damping = self.dHat, self.compliance_collision, self.damping
        sx.sx_batched_substep(C.addressof(a), int(self.persistent_variant), 1 if self.fast_math else 0,
                              stream_handle())
        if self.n_iter % 2:
            self._swap_y()

    def substep(self, dt):
        if self.persistent and self.tol is None:
            if self.bending_on != "y":
                raise ValueError("the persistent substep evaluates bending on y")
            if self.warm is None:
                self._persistent_substep(dt, predict=True)
                return
            g = self.g
            sx.sx_predict(ptr(self.x4), ptr(self.v4), ptr(self.fixed), ptr(self.y4), self.num_verts, float(dt), g[0],
                          g[1], g[2], stream_handle())
            self.warm.begin(self, dt)
            self._persistent_substep(dt, predict=False)
            self.warm.end(self)
            return
        s = stream_handle()
        # per-instance cloth grids and face boxes on x (the substep's BVH build)
        sx.sx_face_aabbs_chunked(ptr(self.x4), ptr(self.faces), self.num_faces, self.padding, ptr(self.fmin4),
                                 ptr(self.fmax4), ptr(self.cmin4), ptr(self.cmax4), s)
        sx.sx_segment_aabbs(ptr(self.x4), ptr(self.vptr), self.n_instances, self.padding, ptr(self.cl_box6), s)
        g = self.g
        sx.sx_predict(ptr(self.x4), ptr(self.v4), ptr(self.fixed), ptr(self.y4), self.num_verts, float(dt), g[0], g[1],
                      g[2], s)
        if self.warm is not None:
            self.warm.begin(self, dt)
        ref = None
        if self.tol is not None and self.tol_relative:
            # threshold relative to the residual of the predicted (cold) start
            if self.warm is not None and self.warm.mode == "apply":
                ref = ptr(self.warm.res_cold)
            else:
                self.constraint_residual("y", out=self._res_ref)
                ref = ptr(self._res_ref)
        k_spring = self.stiffness_bending * dt * dt  # XPBD.py:354
        k_bend = self.stiffness_stretch * dt * dt    # XPBD.py:355
        tol_mode = self.tol is not None
        ce = self.check_every
        if tol_mode:
            if self.bending_on != "y" or self.n_iter % ce or ce < 2 or ce % 2:
                raise ValueError("iterating to a tolerance needs bending_on='y', an even check_every and n_iter a "
                                 "multiple of it")
            sx.sx_convergence_begin(ptr(self._conv), ce, 0, s)
        conv = ptr(self._conv) if tol_mode else None
        if tol_mode and self.n_iter > ce and torch.cuda.is_current_stream_capturing():
            # inside a graph: the first block of iterations, then the rest as a
            # device-side loop that stops once converged
            for it in range(ce):
                self._iteration(it, s, k_spring, k_bend, conv, ref, False)
            body = self._loop_stream()
            h, ctx = C.c_ulonglong(0), C.c_void_p(None)
            sx.sx_loop_begin(s, body.cuda_stream, C.addressof(h), C.addressof(ctx))
            try:
                for k in range(ce):
                    self._iteration(ce + k, body.cuda_stream, k_spring, k_bend, conv, ref, k == 0,
                                    loop=h.value if k == 0 else 0, in_loop=True)
            finally:
                sx.sx_loop_end(ctx)
        else:
            for it in range(self.n_iter):
                check = tol_mode and it > 0 and it % ce == 0
                self._iteration(it, s, k_spring, k_bend, conv, ref, check)
        if self.warm is not None:
            self.warm.end(self)
        sx.sx_velocity_update(ptr(self.x4), ptr(self.y4), ptr(self.v4), ptr(self.fixed), self.num_verts, self.damping,
                              float(dt), s)

    def _loop_stream(self):
        if getattr(self, "_body_stream", None) is None:
            self._body_stream = torch.cuda.Stream(device=self.device)
        return self._body_stream

    def _iteration(self, it, s, k_spring, k_bend, conv, ref, check, loop=0, in_loop=False):
        """One Jacobi iteration: sweep (checked in tolerance mode), broad phase
        in the first iteration, obstacle contacts.  Inside a device-side loop
        (in_loop) the contact kernels are not gated; ``loop`` is the loop
        handle, given with the body's checked sweep."""
        fast = 1 if self.fast_math else 0
        if conv is not None:
            sx.sx_jacobi_sweep_checked_mode(ptr(self.x4), ptr(self.y4), ptr(self._y_other), ptr(self.fixed),
                                            ptr(self.adj_ptr), ptr(self.adj), self.num_verts, k_spring, k_bend, it,
                                            1 if check else 0, float(self.tol), ref, conv, ptr(self._res3),
                                            ptr(self._res_ws), self._res_ws.numel(), loop, self.n_iter, fast, s)
        elif self.packed_sweep:
            sx.sx_jacobi_sweep_packed_v(ptr(self.x4), ptr(self.y4), ptr(self._y_other), ptr(self.fixed),
                                        ptr(self.adj_ptr), ptr(self.adj_nbr16), ptr(self.adj_rest32), self.num_verts,
                                        k_spring, k_bend, 1 if self.bending_on == "y" else 0, self.packed_form, fast,
                                        s)
        else:
            sx.sx_jacobi_sweep_mode(ptr(self.x4), ptr(self.y4), ptr(self._y_other), ptr(self.fixed),
                                    ptr(self.adj_ptr), ptr(self.adj), self.num_verts, k_spring, k_bend,
                                    1 if self.bending_on == "y" else 0, self.sweep_variant, fast, s)
        self._swap_y()
        if it == 0:
            sx.sx_batched_obstacle_broadphase(
                self.num_verts, ptr(self.y4), ptr(self.vinst), ptr(self.ob_box6), ptr(self.ob_fptr),
                ptr(self.ob_fmin4), ptr(self.ob_fmax4), self.padding, ptr(self.vmask), self.n_ob_verts,
                ptr(self.xs4), ptr(self.svinst), ptr(self.cl_box6), ptr(self.fptr), ptr(self.fmin4),
                ptr(self.fmax4), ptr(self.cmin4), ptr(self.cmax4), self.cap, ptr(self.tv_cand), ptr(self.tv_num),
                ptr(self.status), s)
        sx.sx_batched_obstacle_contacts(
            self.num_verts, ptr(self.y4), ptr(self.fixed), ptr(self.m_inv), ptr(self.vinst), ptr(self.ob_fptr),
            ptr(self.ob_faces), ptr(self.xs4), ptr(self.vmask), self.n_ob_verts, ptr(self.tv_cand),
            ptr(self.tv_num), self.cap, ptr(self.faces), self.dHat, self.compliance_collision, ptr(self._dx_fix),
            ptr(self._nc), ptr(self.status), None if in_loop else conv, it, s)

    def _forward_eager(self, n_substeps):
        if self._ob_built_for != self.padding:
            self._static_obstacles()
        dt_sub = self.dt / n_substeps
        for _ in range(n_substeps):
            self.substep(dt_sub)

    def forward(self, n_substeps: int):
        """One frame for every instance (a CUDA graph per frame with
        ``use_graph``)."""
        if self.persistent:
            self._persistent_buffers()  # allocated and uploaded outside any capture
        if not self.use_graph:
            self._forward_eager(n_substeps)
            return
        key = (n_substeps, self.dt, self.dHat, self.damping, self.padding, self.g, self.stiffness_stretch,
               self.stiffness_bending, self.n_iter, self.bending_on, self.sweep_variant, self._packed_sweep, self.packed_form,
               self.fast_math, self.tol,
               self.tol_relative, self.persistent, self.persistent_variant,
               self.check_every,
               id(self.warm) if self.warm is not None else None,
               self.warm.mode if self.warm is not None else None, self.y4.data_ptr())
        gr = self._graphs.get(key)
        if gr is None:
            if self._ob_built_for != self.padding:
                self._static_obstacles()
            y_start = self.y4
            gr = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            lib = load()
            n0 = lib.sx_kernel_launches()
            with torch.cuda.graph(gr, stream=side):
                self._forward_eager(n_substeps)
                if self.y4 is not y_start:
                    y_start.copy_(self.y4)
                    self._swap_y()
            torch.cuda.current_stream(self.device).wait_stream(side)
            self.graph_kernel_launches = lib.sx_kernel_launches() - n0
            self._graphs[key] = gr
        gr.replay()

    @property
    def packed_sweep(self) -> bool:
        return self._packed_sweep

    @packed_sweep.setter
    def packed_sweep(self, on: bool):
        if on and self.adj_nbr16 is None:
            raise ValueError("the packed adjacency needs neighbour offsets within 16 bits")
        self._packed_sweep = bool(on)

    def autotune(self):
        """Solver.autotune for the concatenated instances."""
        from .autotune import tune_sweep

        dt = self.dt / 10
        best, times = tune_sweep(self.x4, self.y4, self.fixed, self.adj_ptr, self.adj, self.num_verts,
                                 self.stiffness_bending * dt * dt, self.stiffness_stretch * dt * dt,
                                 1 if self.bending_on == "y" else 0, packed=(self.adj_nbr16, self.adj_rest32),
                                 fast=self.fast_math)
        from .autotune import variants

        self._packed_sweep = best >= len(variants())
        self.packed_form = best - len(variants()) if self._packed_sweep else 0
        self.sweep_variant = 0 if self._packed_sweep else best
        return best, times

    def autotune_persistent(self, reps: int = 3):
        """Time every launch configuration of the persistent substep on this
        batch (from the current state, restored after each run) and keep the
        fastest; identical results.  Returns (variant, times in ms)."""
        if self._ob_built_for != self.padding:
            self._static_obstacles()
        n = int(sx.sx_batched_substep_variants())
        x0, v0, y0 = self.x4.clone(), self.v4.clone(), self.y4.clone()
        dt = self.dt / 10
        times = []
        for v in range(n):
            self.persistent_variant = v
            self._persistent_substep(dt, predict=True)
            best = None
            for _ in range(reps):
                self.x4.copy_(x0)
                self.v4.copy_(v0)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self._persistent_substep(dt, predict=True)
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b)
                best = ms if best is None else min(best, ms)
            times.append(best)
        self.x4.copy_(x0)
        self.v4.copy_(v0)
        self.y4.copy_(y0)
        self.persistent_variant = int(np.argmin(times))
        self._graphs.clear()
        return self.persistent_variant, times

    def constraint_residual(self, positions: str = "x", out=None):
        """Solver.constraint_residual over every instance's constraints."""
        p = self.x4 if positions == "x" else self.y4
        if out is None:
            out = torch.empty(3, dtype=torch.float64, device=self.device)
        sx.sx_constraint_residual(ptr(p), ptr(self.adj_ptr), ptr(self.adj), self.num_verts, ptr(out),
                                  ptr(self._res_ws), self._res_ws.numel(), stream_handle())
        return out

    def convergence_stats(self, reset: bool = False) -> dict:
        """Solver.convergence_stats."""
        c = self._conv.cpu().tolist()
        r = self._res3.cpu().tolist()
        out = {"converged_substeps": c[4], "mean_stop_iteration": c[3] / c[4] if c[4] else None,
               "last_residual": r[2]}
        if reset:
            sx.sx_convergence_begin(ptr(self._conv), self.check_every, 1, stream_handle())
        return out

    def instance_positions(self, i):
        return self.x4[self.vptr_np[i]:self.vptr_np[i + 1], :3]
