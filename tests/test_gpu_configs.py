"""Parity on the benchmark configurations themselves, at full size.

Each test runs the CUDA solver and the CPU oracle on the same seeded inputs and
checks the acceptance criteria of the substep: positions bit for bit equal,
max |dx| <= 1e-4 x the cloth's bounding-box diagonal, and the constraint
residual (RMS of C = |p0 - p1| - l0, ``sx_constraint_residual``) within 1 % of
the oracle's.  Bit-equality implies the other two; they are asserted
separately so that a failure says which criterion broke.

* 64 x 64 cloth over a box, 10 substeps x 20 Jacobi iterations, 60 frames.
* 256 x 256 cloth draped over a 20480-face sphere with self contact, BVHs
  rebuilt every substep, 10 substeps x 30 iterations, 60 substeps (6 frames),
  replayed as a captured CUDA graph as the benchmark runs it.
* 512 batched cloths (grid side uniform in [16, 128]): the batch runs on the
  GPU; the smallest, the largest, the one whose box is nearest the cloth and
  five seeded picks are each run alone by the oracle.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1
POS_TOL = 1e-4   # x bounding-box diagonal
RES_TOL = 0.01   # relative


def _np(t):
    return t.detach().cpu().numpy()


def _oracle_for(pkg, po, scene, sim):
    return po.OracleSolver(pkg.scenes.oracle_inputs(sim.mesh_dy),
                           pkg.scenes.oracle_inputs(sim.mesh_st) if sim.mesh_st is not None else None,
                           dt=scene.dt, g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                           k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                           padding=scene.padding, n_iter=scene.n_iter, collisions=scene.collisions,
                           rebuild=scene.rebuild, cap=scene.cap, bending_on=sim.bending_on,
                           contact_cull=sim.contact_cull, nthreads=NTHREADS)


def _check(po, got4, orc_x4, adj_ptr, adj, diag, what):
    got = got4[:, :3]
    ref = orc_x4[:, :3]
    assert np.isfinite(got).all(), what
    dmax = float(np.abs(got.astype(np.float64) - ref).max())
    assert dmax <= POS_TOL * diag, f"{what}: max |dx| {dmax:.3e} > {POS_TOL} x diagonal {diag:.4f}"
    r_got = po.residual(np.ascontiguousarray(got4), adj_ptr, adj)
    r_ref = po.residual(np.ascontiguousarray(orc_x4), adj_ptr, adj)
    rms_got, rms_ref = np.sqrt(r_got[0] / r_got[1]), np.sqrt(r_ref[0] / r_ref[1])
    assert abs(rms_got - rms_ref) <= RES_TOL * rms_ref, f"{what}: residual {rms_got:.6e} vs {rms_ref:.6e}"
    assert np.array_equal(got, ref), f"{what}: not bit-exact (max |dx| {dmax:.3e})"
    return dmax, rms_ref


def test_plain64_box_60_frames(pkg, po):
    """64 x 64 cloth (4096 vertices, 7938 faces, 12033 springs, 11781 bending
    pairs), box obstacle, 10 substeps x 20 iterations, 60 frames."""
    scene = pkg.scenes.plain64()
    assert scene.n_substeps == 10 and scene.n_iter == 20
    sim = pkg.scenes.make_solver(scene, device="cuda")
    sim.bending_on = "y"
    sim.use_graph = True
    m = sim.mesh_dy
    assert (m.num_verts, m.num_faces, m.num_edges, m.bending_constraint_count) == (4096, 7938, 12033, 11781)
    orc = _oracle_for(pkg, po, scene, sim)
    for _ in range(60):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
    torch.cuda.synchronize()
    got = _np(m.x4)
    _check(po, got, orc.x4, orc.adj_ptr, orc.adj, m.bbox_diagonal(), "plain64 after 60 frames")
    # the cloth came down on the box: vertices rest on its top face (z = 0.55)
    # instead of falling past it
    on_top = (np.abs(got[:, 2] - 0.55) < 0.02) & (np.abs(got[:, 0] - 0.5) < 0.25) & (np.abs(got[:, 1] - 0.5) < 0.25)
    assert on_top.sum() > 100
    gpu_res = float(sim.constraint_residual("x")[2].item())
    r = po.residual(orc.x4, orc.adj_ptr, orc.adj)
    assert gpu_res == pytest.approx(np.sqrt(r[0] / r[1]), rel=RES_TOL)
    # candidate lists longer than the reference's 40 slots are truncated and
    # flagged by both (vertices on the box's top edges)
    assert sim.status_flags() & 1 == orc.last_status & 1
    assert sim.status_flags() & 4 == 0


def test_drape256_60_substeps(pkg, po):
    """256 x 256 cloth over the sphere with self contact, BVHs rebuilt every
    substep, 10 substeps x 30 iterations, 6 frames, as a replayed graph."""
    scene = pkg.scenes.drape256()
    assert scene.n_iter == 30 and scene.rebuild == "substep"
    sim = pkg.scenes.make_solver(scene, device="cuda")
    sim.bending_on = "y"
    sim.use_graph = True
    m = sim.mesh_dy
    assert (m.num_verts, m.num_faces) == (65536, 130050)
    orc = _oracle_for(pkg, po, scene, sim)
    for f in range(6):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
    torch.cuda.synchronize()
    _check(po, _np(m.x4), orc.x4, orc.adj_ptr, orc.adj, m.bbox_diagonal(), "drape256 after 60 substeps")
    assert np.array_equal(_np(m.v4)[:, :3], orc.v4[:, :3])
    # contacts were active: the pair list of the last substep is not empty and
    # the vertices over the sphere's cap are held above its top (z = 0.8)
    assert sim.contact_pair_count() > 100_000
    x = _np(m.x4)
    cap_ = (x[:, 0] - 0.5) ** 2 + (x[:, 1] - 0.5) ** 2 < 0.05 ** 2
    assert cap_.sum() > 100 and x[cap_, 2].min() > 0.8 - 2 * scene.meta["thickness"]
    gpu_res = float(sim.constraint_residual("x")[2].item())
    r = po.residual(orc.x4, orc.adj_ptr, orc.adj)
    assert gpu_res == pytest.approx(np.sqrt(r[0] / r[1]), rel=RES_TOL)
    assert sim.status_flags() & 1 == orc.last_status & 1
    assert sim.status_flags() & 4 == 0


def test_batched512_sampled_instances(pkg, po):
    """512 cloths in one BatchedSolver (graph per frame), 10 substeps x 20
    iterations, 10 frames; eight instances compared with the oracle run alone."""
    from starlab_physics_gb300 import mesh as M

    insts = pkg.batched_scene(512, seed=0)
    kw = dict(dt=1 / 60, g=(0.0, 0.0, -9.81), k_stretch_stiffness=1e5, k_bend_stiffness=1e8, dHat=(4e-3) ** 2,
              damping=0.001, padding=8e-3, n_iter=20, cap=40)
    sim = pkg.BatchedSolver(insts, dHat=kw["dHat"], stiffness_stretch=1e5, stiffness_bending=1e8, g=kw["g"],
                            dt=kw["dt"], n_iter=20, padding=8e-3)
    assert 3.0e6 < sim.num_verts < 3.4e6
    sim.use_graph = True
    frames = 10
    for _ in range(frames):
        sim.forward(10)
    torch.cuda.synchronize()
    sides = np.array([int(round(np.sqrt(i.x.shape[0]))) for i in insts])
    box_top = np.array([float(i.obstacle_x[:, 2].max()) for i in insts])
    picks = [int(np.argmin(sides)), int(np.argmax(sides)), int(np.argmax(box_top))]
    rng = np.random.default_rng(11)
    for k in rng.permutation(len(insts)):
        if len(picks) == 8:
            break
        if int(k) not in picks:
            picks.append(int(k))
    touched = 0
    for i in picks:
        inst = insts[i]
        cl = M.TriMesh(inst.x, inst.faces, device="cpu")
        cl.fixed[np.asarray(inst.pinned)] = 0.0
        ob = M.TriMesh(inst.obstacle_x, inst.obstacle_faces, device="cpu")
        orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), collisions=True,
                              rebuild="substep", self_collision=False, bending_on="y", nthreads=NTHREADS, **kw)
        for _ in range(frames):
            orc.forward(10)
        got = np.zeros_like(orc.x4)
        got[:, :3] = _np(sim.instance_positions(i))
        got[:, 3] = orc.x4[:, 3]
        p = inst.x.astype(np.float64)
        diag = float(np.linalg.norm(p.max(0) - p.min(0)))
        _check(po, got, orc.x4, orc.adj_ptr, orc.adj, diag, f"instance {i} (side {sides[i]})")
        # the box holds part of the cloth above the free-fall height
        touched += int((orc.x4[:, 2] > 1.0 - 0.5 * 9.81 * (frames / 60) ** 2 + 0.01).sum() > 0)
    assert touched >= 1
    assert int(sim.status.item()) & 4 == 0


def _check_tol(po, got4, orc_x4, adj_ptr, adj, diag, what):
    """The tolerance criteria alone (for the fast arithmetic, which is not
    bit-identical): max |dx| <= 1e-4 x diagonal, residual within 1 %."""
    got, ref = got4[:, :3], orc_x4[:, :3]
    assert np.isfinite(got).all(), what
    dmax = float(np.abs(got.astype(np.float64) - ref).max())
    assert dmax <= POS_TOL * diag, f"{what}: max |dx| {dmax:.3e} > {POS_TOL} x diagonal {diag:.4f}"
    r_got = po.residual(np.ascontiguousarray(got4), adj_ptr, adj)
    r_ref = po.residual(np.ascontiguousarray(orc_x4), adj_ptr, adj)
    rms_got, rms_ref = np.sqrt(r_got[0] / r_got[1]), np.sqrt(r_ref[0] / r_ref[1])
    assert abs(rms_got - rms_ref) <= RES_TOL * rms_ref, f"{what}: residual {rms_got:.6e} vs {rms_ref:.6e}"
    return dmax


def test_fast_math_within_tolerance(pkg, po):
    """The sweep's fast arithmetic (fused multiply-adds, hardware reciprocal
    square root; not bit-identical) against the exact oracle over the stated
    horizon of 60 substeps: the 64 x 64 box scene after 10 exact frames
    (falling), the drape after 3 (on the sphere, self contact) and four batched
    instances after 8.  Positions stay within 1e-4 x the bounding-box diagonal
    and the residual within 1 %, and differ from the exact run (the fast
    kernels ran).

    Two regimes amplify any change of rounding far beyond that tolerance, the
    exact arithmetic's own included, and are judged against that amplification
    instead:
    * a query with more candidates than the reference's 40 slots (the box
      scene's contact phase, instance 78 from its 14th frame): which candidates
      survive the truncation flips with the last bit of a position.  The
      windows here hold none (asserted through the oracle's status).
    * a cloth landing: instance 78 (the highest box) reaches its box within the
      window, and whether a vertex's contact is active in a given iteration
      flips with the last bit of its position.  There a one-ulp change of the
      frame-8 positions moves the exact oracle's result by about 1e-3 m; the
      fast run must stay within 4 times that (and the residual within 1 %)."""
    from starlab_physics_gb300 import mesh as M

    for scene, warm in ((pkg.scenes.plain64(), 10), (pkg.scenes.drape256(), 3)):
        sim = pkg.scenes.make_solver(scene, device="cuda")
        sim.bending_on = "y"
        sim.use_graph = True
        for _ in range(warm):
            sim.forward(scene.n_substeps)
        torch.cuda.synchronize()
        orc = _oracle_for(pkg, po, scene, sim)
        orc.x4[:] = _np(sim.mesh_dy.x4)
        orc.v4[:] = _np(sim.mesh_dy.v4)
        sim.fast_math = True
        for _ in range(6):
            sim.forward(scene.n_substeps)
            orc.forward(scene.n_substeps)
        torch.cuda.synchronize()
        d = _check_tol(po, _np(sim.mesh_dy.x4), orc.x4, orc.adj_ptr, orc.adj, sim.mesh_dy.bbox_diagonal(),
                       f"{scene.name} fast")
        assert d > 0.0
    insts = pkg.batched_scene(512, seed=0)
    kw = dict(dt=1 / 60, g=(0.0, 0.0, -9.81), k_stretch_stiffness=1e5, k_bend_stiffness=1e8, dHat=(4e-3) ** 2,
              damping=0.001, padding=8e-3, n_iter=20, cap=40)
    bs = pkg.BatchedSolver(insts, dHat=kw["dHat"], stiffness_stretch=1e5, stiffness_bending=1e8, g=kw["g"],
                           dt=kw["dt"], n_iter=20, padding=8e-3)
    bs.use_graph = True
    for _ in range(8):
        bs.forward(10)
    torch.cuda.synchronize()
    x8, v8 = _np(bs.x4).copy(), _np(bs.v4).copy()
    bs.fast_math = True
    for _ in range(6):
        bs.forward(10)
    torch.cuda.synchronize()
    sides = np.array([int(round(np.sqrt(i.x.shape[0]))) for i in insts])
    box_top = np.array([float(i.obstacle_x[:, 2].max()) for i in insts])
    assert int(np.argmax(box_top)) == 78
    for i in (int(np.argmin(sides)), int(np.argmax(sides)), 78, 100):
        inst = insts[i]
        cl = M.TriMesh(inst.x, inst.faces, device="cpu")
        cl.fixed[np.asarray(inst.pinned)] = 0.0
        ob = M.TriMesh(inst.obstacle_x, inst.obstacle_faces, device="cpu")
        o = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), collisions=True,
                            rebuild="substep", self_collision=False, bending_on="y", nthreads=NTHREADS, **kw)
        a, b = bs.vptr_np[i], bs.vptr_np[i + 1]
        o.x4[:] = x8[a:b]
        o.v4[:] = v8[a:b]
        o.last_status = 0
        for _ in range(6):
            o.forward(10)
        assert o.last_status & 1 == 0, f"instance {i}: a query overflowed the candidate slots"
        if i == 78:
            assert o.x4[:, 2].min() < box_top[i], "instance 78 reached its box"
        g4 = np.zeros_like(o.x4)
        g4[:, :3] = _np(bs.instance_positions(i))
        g4[:, 3] = o.x4[:, 3]
        p = inst.x.astype(np.float64)
        diag = float(np.linalg.norm(p.max(0) - p.min(0)))
        if i != 78:
            _check_tol(po, g4, o.x4, o.adj_ptr, o.adj, diag, f"instance {i} fast")
            continue
        # the landing instance: the exact oracle's own sensitivity to one ulp
        sens = 0.0
        for direction in (np.inf, -np.inf):
            q = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), collisions=True,
                                rebuild="substep", self_collision=False, bending_on="y", nthreads=NTHREADS, **kw)
            q.x4[:] = x8[a:b]
            q.x4[:, :3] = np.nextafter(x8[a:b, :3], np.float32(direction))
            q.v4[:] = v8[a:b]
            for _ in range(6):
                q.forward(10)
            sens = max(sens, float(np.abs(q.x4[:, :3].astype(np.float64) - o.x4[:, :3]).max()))
        assert sens > POS_TOL * diag, "the landing window is expected to amplify rounding changes"
        d = float(np.abs(g4[:, :3].astype(np.float64) - o.x4[:, :3]).max())
        assert d <= 4.0 * sens, f"instance 78 fast: max |dx| {d:.3e} > 4 x one-ulp sensitivity {sens:.3e}"
        r_got = po.residual(np.ascontiguousarray(g4), o.adj_ptr, o.adj)
        r_ref = po.residual(np.ascontiguousarray(o.x4), o.adj_ptr, o.adj)
        rms_got, rms_ref = np.sqrt(r_got[0] / r_got[1]), np.sqrt(r_ref[0] / r_ref[1])
        assert abs(rms_got - rms_ref) <= RES_TOL * rms_ref, f"instance 78 fast: residual {rms_got:.6e} vs {rms_ref:.6e}"
