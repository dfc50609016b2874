"""GPU parity of the edge-edge contacts (the reference's commented-out
__ee_st / __ee_dy path) against the CPU oracle, through the C ABI: the
classifier on every branch, the edge broad phase, one sweep's records and
accumulators, and whole frames of the solver -- all bit for bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda"


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _np(t):
    return t.detach().cpu().numpy()


def test_edge_edge_classify_bit_exact(pkg, po):
    from starlab_physics_gb300._lib import ptr, stream_handle, sx

    rng = np.random.default_rng(21)
    p = np.concatenate([(rng.normal(size=(4000, 12)) * s).astype(np.float32) for s in (0.01, 0.1, 1.0)])
    dHat = 1e-2
    dt, d, g = po.edge_edge_classify(p, dHat)
    assert set(dt.tolist()) == set(range(9)) and (d < dHat).sum() > 100
    P = _t(p)
    gdt = torch.zeros(p.shape[0], dtype=torch.int32, device=DEV)
    gd = torch.zeros(p.shape[0], dtype=torch.float32, device=DEV)
    gg = torch.zeros((p.shape[0], 12), dtype=torch.float32, device=DEV)
    assert sx.sx_edge_edge_classify(p.shape[0], ptr(P), dHat, ptr(gdt), ptr(gd), ptr(gg), stream_handle()) == 0
    torch.cuda.synchronize()
    assert np.array_equal(_np(gdt), dt)
    assert np.array_equal(_np(gd), d)
    assert np.array_equal(_np(gg).reshape(-1, 4, 3), g)


def _layers(pkg, **kw):
    sc = pkg.scenes.crossed_layers()
    sim = pkg.scenes.make_solver(sc, device=DEV)
    sim.bending_on = "y"
    sim.enable_edge_edge = True
    for k, v in kw.items():
        setattr(sim, k, v)
    return sc, sim


def _oracle(pkg, po, sc, sim, **kw):
    return po.OracleSolver(pkg.scenes.oracle_inputs(sim.mesh_dy), pkg.scenes.oracle_inputs(sim.mesh_st), dt=sc.dt,
                           g=sc.gravity, k_stretch_stiffness=sc.stiffness_stretch,
                           k_bend_stiffness=sc.stiffness_bending, dHat=sc.dHat, damping=sc.damping,
                           padding=sc.padding, n_iter=sc.n_iter, collisions=True, rebuild=sc.rebuild, cap=sc.cap,
                           bending_on="y", contact_cull=sim.contact_cull, edge_edge=True, **kw)


def test_edge_broad_phase_and_sweep_bit_exact(pkg, po):
    """Mid-fall state of the crossed layers: the edge candidate lists on both
    cell BVHs, then one edge-edge sweep's records and fixed-point accumulators,
    against the oracle on the same positions."""
    sc = pkg.scenes.crossed_layers()
    sim = pkg.scenes.make_solver(sc, device=DEV)
    sim.bending_on = "y"
    sim.enable_edge_edge = False
    for _ in range(3):
        sim.forward(sc.n_substeps)
    torch.cuda.synchronize()
    m, s = sim.mesh_dy, sim.mesh_st
    rec = pkg.Solver(m, s, dHat=sc.dHat, stiffness_stretch=sc.stiffness_stretch,
                     stiffness_bending=sc.stiffness_bending, g=sc.gravity, dt=sc.dt, n_iter=sc.n_iter,
                     rebuild=sc.rebuild, cap=sc.cap, record_pairs=True, bending_on="y")
    rec.padding = sc.padding
    rec.enable_collision_handling = True
    rec.enable_edge_edge = True
    dt_sub = sc.dt / sc.n_substeps
    rec.build_bvhs()
    rec.compute_y(dt_sub)
    rec.spring_sweep(dt_sub, 0)
    rec.broadphase_lbvh()
    y = _np(m.y4).copy()
    x = _np(m.x4).copy()
    rec.solve_edge_edge_constraints_x()
    torch.cuda.synchronize()
    ee = rec._ensure_ee()
    # oracle: BVHs on x, edge boxes on y
    bd, bs = po.CellBVH(), po.CellBVH()
    mn, mx = po.face_aabbs(x, m.fid_np, sc.padding)
    bd.build(mn, mx, po.scene_aabb(x, sc.padding))
    xs = _np(s.x4)
    mn, mx = po.face_aabbs(xs, s.fid_np, sc.padding)
    bs.build(mn, mx, po.scene_aabb(xs, sc.padding))
    emn, emx = po.edge_query_boxes(y, m.eid_np, sc.padding)
    st = bs.traverse(emn, emx, sc.cap)
    dy = bd.traverse(emn, emx, sc.cap)
    for (cand, num, _), gc, gn in ((st, ee["st_c"], ee["st_n"]), (dy, ee["dy_c"], ee["dy_n"])):
        gnum = _np(gn)
        assert np.array_equal(gnum, num)
        gcand = _np(gc)
        for q in range(num.shape[0]):
            k = min(num[q], sc.cap)
            assert np.array_equal(gcand[q, :k], cand[q, :k])
    V = m.num_verts
    dx = np.zeros(3 * V, np.int64)
    nc = np.zeros(V, np.int32)
    r = po.edge_edge_sweep(m.eid_np, s.eid_np, m.face_edge_np, s.face_edge_np, y, xs, _np(m.fixed), _np(m.m_inv),
                           sc.dHat, 1e8, sc.cap, st[:2], dy[:2], dx, nc, want_pairs=True)
    assert r["pair_num"].sum() > 20, "the state has edge-edge contacts"
    assert np.array_equal(_np(ee["pair_num"]), r["pair_num"])
    E = m.num_edges
    gp, gg, gs = _np(ee["pair"]), _np(ee["pair_g"]), _np(ee["pair_schur"])
    for q in range(2 * E):
        k = r["pair_num"][q]
        assert np.array_equal(gp[q, :k], r["pair"][q, :k])
        assert np.array_equal(gg[q, :k], r["pair_g"][q, :k])
        assert np.array_equal(gs[q, :k], r["pair_schur"][q, :k])
    assert np.array_equal(_np(rec._dx_fix), dx)
    assert np.array_equal(_np(rec._nc), nc)
    rec._dx_fix.zero_()
    rec._nc.zero_()


@pytest.mark.parametrize("record_pairs,use_graph", [(False, False), (False, True), (True, False)])
def test_edge_edge_solver_matches_oracle(pkg, po, record_pairs, use_graph):
    """Four frames of the crossed layers with edge-edge contacts: positions and
    velocities equal the oracle's; without the edge-edge terms they differ."""
    sc = pkg.scenes.crossed_layers()
    res = {}
    for ee in (True, False):
        sim = pkg.scenes.make_solver(sc, device=DEV) if not record_pairs else None
        if record_pairs:
            base = pkg.scenes.make_solver(sc, device=DEV)
            sim = pkg.Solver(base.mesh_dy, base.mesh_st, dHat=sc.dHat, stiffness_stretch=sc.stiffness_stretch,
                             stiffness_bending=sc.stiffness_bending, g=sc.gravity, dt=sc.dt, n_iter=sc.n_iter,
                             rebuild=sc.rebuild, cap=sc.cap, record_pairs=True)
            sim.padding, sim.damping = sc.padding, sc.damping
            sim.enable_collision_handling = True
        sim.bending_on = "y"
        sim.enable_edge_edge = ee
        sim.use_graph = use_graph
        for _ in range(4):
            sim.forward(sc.n_substeps)
        torch.cuda.synchronize()
        res[ee] = (_np(sim.mesh_dy.x4), _np(sim.mesh_dy.v4), sim)
    sim = res[True][2]
    orc = _oracle(pkg, po, sc, sim)
    for _ in range(4):
        orc.forward(sc.n_substeps)
    gx, gv = res[True][0], res[True][1]
    assert np.isfinite(gx).all()
    assert np.array_equal(gx[:, :3], orc.x4[:, :3])
    assert np.array_equal(gv[:, :3], orc.v4[:, :3])
    assert not np.array_equal(gx, res[False][0])
    assert (sim.status_flags() & ~1) == 0


def test_edge_edge_tolerance_mode_matches_oracle(pkg, po):
    """Iterating to a residual with the device-side loop: the edge-edge sweep is
    gated with the other kernels; stop decisions and positions equal the
    oracle's."""
    sc = pkg.scenes.crossed_layers()
    sc.n_iter = 16
    sim = pkg.scenes.make_solver(sc, device=DEV)
    sim.bending_on = "y"
    sim.enable_edge_edge = True
    sim.use_graph = True
    sim.tol = 1e9  # every substep stops at its first check
    for _ in range(4):
        sim.forward(sc.n_substeps)
    torch.cuda.synchronize()
    orc = _oracle(pkg, po, sc, sim, tol=1e9)
    for _ in range(4):
        orc.forward(sc.n_substeps)
    st = sim.convergence_stats()
    assert st["converged_substeps"] == orc.converged == 4 * sc.n_substeps
    assert np.array_equal(_np(sim.mesh_dy.x4)[:, :3], orc.x4[:, :3])
