"""GPU parity: every CUDA entry point against the CPU oracle, through the C ABI.

Integer outputs (Morton codes, sort order, BVH topology, candidate lists,
colourings) must match bit for bit.  Float outputs are compared bit for bit as
well: kernels and oracle evaluate the same expressions in the same order with
no FMA contraction, so any difference is a bug.  End-to-end solver runs are
additionally held to a tolerance of 1e-4 x the bounding-box diagonal.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda"


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def sxm(pkg):
    from starlab_physics_gb300 import _lib

    _lib.load()
    return _lib


def _cloth(pkg, n=16, seed=3, pinned=True):
    sc = pkg.scenes.plain64(n=n, seed=seed)
    m = pkg.TriMesh(sc.cloth_x, sc.cloth_faces, device=DEV)
    if pinned:
        m.fixed[sc.pinned] = 0.0
        m.refresh_weights()
    return sc, m


def _state(m, rng):
    V = m.num_verts
    x4 = _np(m.x4).copy()
    x4[:, :3] += rng.normal(0, 2e-3, (V, 3)).astype(np.float32)
    v4 = np.zeros((V, 4), np.float32)
    v4[:, :3] = rng.normal(0, 0.3, (V, 3)).astype(np.float32)
    return x4, v4


def test_predict_sweep_velocity_bit_exact(pkg, po, sxm):
    sc, m = _cloth(pkg)
    rng = np.random.default_rng(0)
    x4, v4 = _state(m, rng)
    fixed = _np(m.fixed)
    m_inv = _np(m.m_inv)
    dt = 1.0 / 600.0
    g = (0.0, 0.0, -9.81)
    s = torch.cuda.current_stream().cuda_stream
    X, Vv, Y, Y2 = _t(x4), _t(v4), torch.empty_like(m.x4), torch.empty_like(m.x4)
    sxm.sx.sx_predict(X.data_ptr(), Vv.data_ptr(), m.fixed.data_ptr(), Y.data_ptr(), m.num_verts, dt, *g, s)
    y_ref = po.predict(x4, v4, fixed, dt, g)
    assert np.array_equal(_np(Y), y_ref)
    for bend_on_y in (0, 1):
        yin = _t(y_ref)
        ks, kb = 1e8 * dt * dt, 1e5 * dt * dt
        sxm.sx.sx_jacobi_sweep(X.data_ptr(), yin.data_ptr(), Y2.data_ptr(), m.fixed.data_ptr(),
                               m.adj_ptr.data_ptr(), m.adj.data_ptr(), m.num_verts, ks, kb, bend_on_y, s)
        yo = y_ref.copy()
        po.spring_sweep(x4, yo, fixed, m_inv, m.eid_np, m.l0_np, m.bending_np, m.bending_l0_np, ks, kb,
                        bend_on_y=bend_on_y)
        got = _np(Y2)
        assert np.array_equal(got[:, :3], yo[:, :3]), f"bend_on_y={bend_on_y} max diff {np.abs(got - yo).max()}"
    xo, vo = x4.copy(), v4.copy()
    po.velocity_update(xo, yo, vo, fixed, 0.001, dt)
    Yt = _t(yo)
    sxm.sx.sx_velocity_update(X.data_ptr(), Yt.data_ptr(), Vv.data_ptr(), m.fixed.data_ptr(), m.num_verts, 0.001,
                              dt, s)
    assert np.array_equal(_np(X)[:, :3], xo[:, :3])
    assert np.array_equal(_np(Vv)[:, :3], vo[:, :3])


def test_sweep_variants_and_autotune(pkg, po, sxm):
    """Every launch configuration of the sweep gives the oracle's result bit for
    bit, and the autotuner picks one of them."""
    sc, m = _cloth(pkg)
    rng = np.random.default_rng(5)
    x4, v4 = _state(m, rng)
    fixed, m_inv = _np(m.fixed), _np(m.m_inv)
    dt = 1.0 / 600.0
    ks, kb = 1e8 * dt * dt, 1e5 * dt * dt
    y = po.predict(x4, v4, fixed, dt, (0.0, 0.0, -9.81))
    yo = y.copy()
    po.spring_sweep(x4, yo, fixed, m_inv, m.eid_np, m.l0_np, m.bending_np, m.bending_l0_np, ks, kb, bend_on_y=1)
    X, Yin, Yout = _t(x4), _t(y), torch.empty_like(m.x4)
    s = torch.cuda.current_stream().cuda_stream
    n_var = int(sxm.load().sx_jacobi_sweep_variants())
    assert n_var >= 4
    for v in range(n_var):
        Yout.fill_(float("nan"))
        sxm.sx.sx_jacobi_sweep_v(X.data_ptr(), Yin.data_ptr(), Yout.data_ptr(), m.fixed.data_ptr(),
                                 m.adj_ptr.data_ptr(), m.adj.data_ptr(), m.num_verts, ks, kb, 1, v, s)
        assert np.array_equal(_np(Yout)[:, :3], yo[:, :3]), v
    from starlab_physics_gb300 import autotune

    best, times = autotune.tune_sweep(X, Yin, m.fixed, m.adj_ptr, m.adj, m.num_verts, ks, kb, 1, reps=5, rounds=3)
    assert 0 <= best < n_var and len(times) == n_var and min(times) > 0


def test_aabbs(pkg, po, sxm):
    sc, m = _cloth(pkg, n=20)
    x4 = _np(m.x4)
    m.computeAABB_faces(0.01)
    mn, mx = po.face_aabbs(x4, m.fid_np, 0.01)
    assert np.array_equal(_np(m.aabb_min4), mn) and np.array_equal(_np(m.aabb_max4), mx)
    m.computeAABB(0.02)
    assert np.array_equal(_np(m.box6), po.scene_aabb(x4, 0.02))


@pytest.mark.parametrize("n,bits", [(1, 30), (7, 30), (2047, 30), (2048, 30), (2049, 15), (100003, 32),
                                    (65536, 8), (300000, 30)])
def test_radix_sort(pkg, sxm, n, bits):
    rng = np.random.default_rng(n)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    if n > 10:
        keys[: n // 3] = keys[n // 3: 2 * (n // 3)]  # many duplicates: stability matters
    vals = np.arange(n, dtype=np.int32)
    K, Vt = _t(keys.view(np.int32)), _t(vals)
    ws = torch.empty(int(sxm.load().sx_radix_sort_workspace_bytes(n)), dtype=torch.uint8, device=DEV)
    sxm.sx.sx_radix_sort_pairs(K.data_ptr(), Vt.data_ptr(), n, bits, ws.data_ptr(), ws.numel(),
                               torch.cuda.current_stream().cuda_stream)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(_np(Vt), order)
    assert np.array_equal(_np(K).view(np.uint32), keys[order])


def test_cell_bvh_init(pkg, po):
    bvh = pkg.LBVH_CELL(10, DEV)
    ref = po.CellBVH()
    assert np.array_equal(_np(bvh.cell_morton_codes), ref.codes)
    assert np.array_equal(_np(bvh.cell_ids), ref.ids)
    for a, b in [(bvh.child_a, ref.child_a), (bvh.child_b, ref.child_b), (bvh.range_l, ref.range_l),
                 (bvh.range_r, ref.range_r), (bvh.parent, ref.parent)]:
        assert np.array_equal(_np(a), b)


def _drape(pkg, n=48):
    sc = pkg.scenes.drape256(n=n, sphere_subdiv=3)
    cl = pkg.TriMesh(sc.cloth_x, sc.cloth_faces, device=DEV)
    sp = pkg.TriMesh(sc.obstacle_x, sc.obstacle_faces, device=DEV, is_static=True)
    return sc, cl, sp


def test_cell_bvh_build_and_traverse(pkg, po):
    sc, cl, sp = _drape(pkg)
    pad = 0.01
    for mesh in (cl, sp):
        mesh.computeAABB_faces(pad)
        mesh.computeAABB(pad)
        bvh = pkg.LBVH_CELL(mesh.num_faces, DEV)
        bvh.build(mesh, mesh.box6)
        ref = po.CellBVH()
        ref.build(_np(mesh.aabb_min4), _np(mesh.aabb_max4), _np(mesh.box6))
        assert np.array_equal(_np(bvh.prefix_sum_cell), ref.prefix)
        assert np.array_equal(_np(bvh.sorted_face_ids)[: mesh.num_faces], ref.sorted_face_ids)
        assert np.array_equal(_np(bvh.num_faces), ref.num_faces)
        assert np.array_equal(_np(bvh.node_min4), ref.nmin4)
        assert np.array_equal(_np(bvh.node_max4), ref.nmax4)
        assert np.array_equal(_np(bvh.cell_size), ref.cell_size)
        # queries: the cloth vertices
        pts = _np(cl.x4).copy()
        pts[:, :3] += np.random.default_rng(1).normal(0, 0.01, (pts.shape[0], 3)).astype(np.float32)
        P = _t(pts)
        cap = 40
        cand = torch.full((pts.shape[0], cap), -1, dtype=torch.int32, device=DEV)
        num = torch.zeros(pts.shape[0], dtype=torch.int32, device=DEV)
        status = torch.zeros(1, dtype=torch.int32, device=DEV)
        bvh.traverse(P, pad, cap, cand, num, status)
        qmn, qmx = po.query_boxes(pts, pad)
        rc, rn, rs = ref.traverse(qmn, qmx, cap)
        gn = _np(num)
        assert np.array_equal(gn, rn)
        gc = _np(cand)
        for q in range(pts.shape[0]):
            k = min(rn[q], cap)
            assert np.array_equal(gc[q, :k], rc[q, :k])
        assert int(status.item()) == rs


@pytest.mark.parametrize("size,seed", [(0.004, 1), (0.08, 2), (0.3, 3)])
def test_cell_traverse_adversarial(pkg, po, size, seed):
    """Faces that overhang many cells and queries inside, outside and on the edge
    of the grid: the cell walk must reproduce the reference's depth-first list."""
    rng = np.random.default_rng(seed)
    F = 20000
    c = rng.uniform(0, 1, (F, 3)).astype(np.float32)
    e = (rng.uniform(0, size, (F, 3)) * rng.uniform(0, 1, (F, 1)) ** 4).astype(np.float32)
    mn = np.zeros((F, 4), np.float32)
    mx = np.zeros((F, 4), np.float32)
    mn[:, :3], mx[:, :3] = c - e, c + e
    box = np.array([-0.05, -0.05, -0.05, 1.05, 1.05, 1.05], np.float32)
    bvh = pkg.LBVH_CELL(F, DEV)
    bvh.build(None, _t(box), face_min4=_t(mn), face_max4=_t(mx))
    ref = po.CellBVH()
    ref.build(mn, mx, box)
    assert np.array_equal(_np(bvh.node_min4), ref.nmin4) and np.array_equal(_np(bvh.node_max4), ref.nmax4)
    pts = np.zeros((30000, 4), np.float32)
    pts[:, :3] = rng.uniform(-0.2, 1.2, (30000, 3))
    pts[:100, :3] = np.array([1.05, 0.5, 0.5], np.float32)   # on the upper face of the grid
    cap = 64
    cand = torch.full((pts.shape[0], cap), -1, dtype=torch.int32, device=DEV)
    num = torch.zeros(pts.shape[0], dtype=torch.int32, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    for pad in (0.002, 0.05):
        bvh.traverse(_t(pts), pad, cap, cand, num, status)
        qmn, qmx = po.query_boxes(pts, pad)
        rc, rn, rs = ref.traverse(qmn, qmx, cap)
        assert np.array_equal(_np(num), rn)
        gc = _np(cand)
        for q in range(pts.shape[0]):
            k = min(rn[q], cap)
            assert np.array_equal(gc[q, :k], rc[q, :k]), q


@pytest.mark.parametrize("n", [1, 2, 3, 255, 257, 1000, 5000, 4800 * 256 + 7])
def test_face_lbvh_tiled_refit_ragged(pkg, po, n):
    """The shared-memory refit (tiles of 256 sorted leaves, a climb above
    them) at sizes that are not multiples of the tile: node boxes equal the
    oracle's bit for bit."""
    verts, faces, _ = pkg.scenes.triangle_soup(n, seed=n)
    V4 = np.zeros((verts.shape[0], 4), np.float32)
    V4[:, :3] = verts
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    box = po.scene_aabb(V4, 0.0)
    bvh = pkg.LBVH(n, DEV, tie=1)
    bvh.build(_t(mn), _t(mx), _t(box))
    ref = po.FaceBVH(mn, mx, box, tie=1)
    assert np.array_equal(_np(bvh.node_min4), ref.nmin4)
    assert np.array_equal(_np(bvh.node_max4), ref.nmax4)
    assert int(bvh.status.item()) == 0


def test_face_lbvh_small_soup(pkg, po):
    verts, faces, queries = pkg.scenes.triangle_soup(1 << 14, seed=5)
    V4 = np.zeros((verts.shape[0], 4), np.float32)
    V4[:, :3] = verts
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    box = po.scene_aabb(V4, 0.0)
    for tie in (0, 1):
        bvh = pkg.LBVH(faces.shape[0], DEV, tie=tie)
        bvh.build(_t(mn), _t(mx), _t(box))
        ref = po.FaceBVH(mn, mx, box, tie=tie)
        assert np.array_equal(_np(bvh.codes), ref.sorted_codes)
        assert np.array_equal(_np(bvh.sorted_ids), ref.sorted_ids)
        n = faces.shape[0]
        assert np.array_equal(_np(bvh.child_a)[: n - 1], ref.child_a)
        assert np.array_equal(_np(bvh.child_b)[: n - 1], ref.child_b)
        assert np.array_equal(_np(bvh.range_l)[: n - 1], ref.range_l)
        assert np.array_equal(_np(bvh.range_r)[: n - 1], ref.range_r)
        if tie == 1 or len(np.unique(ref.sorted_codes)) == n:
            assert np.array_equal(_np(bvh.parent), ref.parent)
            assert np.array_equal(_np(bvh.node_min4), ref.nmin4)
            assert np.array_equal(_np(bvh.node_max4), ref.nmax4)
            Q = np.zeros((queries.shape[0], 4), np.float32)
            Q[:, :3] = queries
            cand, num = bvh.query(_t(Q), 2e-3, 64)
            qmn, qmx = po.query_boxes(Q, 2e-3)
            rc, rn, _ = ref.traverse(qmn, qmx, 64)
            assert np.array_equal(_np(num), rn)
            gc = _np(cand)
            for q in range(0, Q.shape[0], 7):
                k = min(rn[q], 64)
                assert np.array_equal(gc[q, :k], rc[q, :k])


def test_collision_sweep_bit_exact(pkg, po):
    sc, cl, sp = _drape(pkg, n=40)
    sim = pkg.Solver(cl, sp, dHat=(4e-2) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8, g=(0, 0, -9.81),
                     dt=1 / 60, record_pairs=True)
    sim.padding = 0.04
    sim.enable_collision_handling = True
    # squash the cloth onto the sphere so that many contacts are active
    x = _np(cl.x4).copy()
    x[:, 2] = 0.5 + 0.3 + 0.01 * np.sin(13 * x[:, 0]) * np.cos(7 * x[:, 1])
    cl.x4.copy_(_t(x))
    sim.build_bvhs()
    sim.compute_y(1 / 600)
    sim.broadphase_lbvh()
    y_before = _np(cl.y4).copy()
    cap = sim.cache_size
    vt_st = (_np(sim.vt_st_candidates), _np(sim.vt_st_candidates_num))
    vt_dy = (_np(sim.vt_dy_candidates), _np(sim.vt_dy_candidates_num))
    tv_st = (_np(sim.tv_st_candidates), _np(sim.tv_st_candidates_num))
    sim.solve_collision_constraints_x()
    yo = y_before.copy()
    r = po.collision_sweep(cl.fid_np, sp.fid_np, yo, _np(sp.x4), _np(cl.fixed), _np(cl.m_inv), np.float32(sim.dHat),
                           np.float32(1e8), cap, vt_st, vt_dy, tv_st, want_pairs=True)
    got = _np(cl.y4)
    assert (r["pair_num"] > 0).sum() > 10, "test scene produced too few contacts"
    assert np.array_equal(got[:, :3], yo[:, :3]), f"max diff {np.abs(got[:, :3] - yo[:, :3]).max()}"
    assert np.array_equal(_np(sim.pair_num), r["pair_num"])
    pn = r["pair_num"]
    gp, gg, gs = _np(sim.pair), _np(sim.pair_g), _np(sim.pair_schur)
    for q in np.flatnonzero(pn):
        k = pn[q]
        assert np.array_equal(gp[q, :k], r["pair"][q, :k])
        assert np.array_equal(gg[q, :k], r["pair_g"][q, :k])
        assert np.array_equal(gs[q, :k], r["pair_schur"][q, :k])
    assert np.count_nonzero(_np(sim._dx_fix)) == 0 and np.count_nonzero(_np(sim._nc)) == 0


def _run_pair(pkg, po, scene, frames, **solver_kw):
    sim = pkg.scenes.make_solver(scene, device=DEV)
    for k, v in solver_kw.items():
        setattr(sim, k, v)
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(sim.mesh_dy),
                          pkg.scenes.oracle_inputs(sim.mesh_st) if sim.mesh_st is not None else None,
                          dt=scene.dt, g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                          k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                          padding=scene.padding, n_iter=scene.n_iter, collisions=scene.collisions,
                          rebuild=scene.rebuild, cap=scene.cap, bending_on=sim.bending_on,
                          contact_cull=sim.contact_cull)
    for _ in range(frames):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
    torch.cuda.synchronize()
    return sim, orc


@pytest.mark.parametrize("mode", ["reference", "iterated"])
def test_solver_end_to_end(pkg, po, mode):
    scene = pkg.scenes.plain64(n=24, seed=2)
    if mode == "reference":
        scene.n_iter, scene.rebuild, scene.padding = 1, "frame", 0.03
        sim_kw = {}
    else:
        scene.n_iter = 4
        sim_kw = {"bending_on": "y"}
    sim, orc = _run_pair(pkg, po, scene, 6, **sim_kw)
    gx = _np(sim.mesh_dy.x4)
    diag = sim.mesh_dy.bbox_diagonal()
    assert np.isfinite(gx).all()
    diff = np.abs(gx[:, :3] - orc.x4[:, :3]).max()
    assert diff <= 1e-4 * diag
    assert np.array_equal(gx[:, :3], orc.x4[:, :3]), f"not bit-exact: max diff {diff}"


def test_coloring(pkg, po):
    for n in (9, 33, 256):
        x, f = pkg.grid_cloth(n)
        e = pkg.mesh.edges_from_faces(f)
        gc = pkg.GraphColoring(n * n, e, device=DEV)
        color, sorted_e, prefix = po.color_edges(n * n, e)
        assert np.array_equal(_np(gc.edges_color)[: e.shape[0]], color)
        assert np.array_equal(_np(gc.sorted_edges_sequence_for_color)[: e.shape[0]], sorted_e)
        assert np.array_equal(_np(gc.color_prefix_sum), prefix)


@pytest.mark.parametrize("cull", [False, True])
def test_pair_list_sweep_equals_per_query_sweep(pkg, cull):
    """The compacted pair list, with or without the box-distance cull, gives the
    same positions as the per-query walk (which classifies every pair)."""
    outs = []
    for record in (True, False):
        sc, cl, sp = _drape(pkg, n=40)
        sim = pkg.Solver(cl, sp, dHat=(4e-2) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8, g=(0, 0, -9.81),
                         dt=1 / 60, record_pairs=record)
        sim.padding = 0.04
        sim.enable_collision_handling = True
        x = _np(cl.x4).copy()
        x[:, 2] = 0.5 + 0.3 + 0.01 * np.sin(13 * x[:, 0]) * np.cos(7 * x[:, 1])
        cl.x4.copy_(_t(x))
        sim.build_bvhs()
        sim.compute_y(1 / 600)
        sim.broadphase_lbvh()
        sim.contact_cull = cull
        if not record:
            sim.build_contact_pairs()
        for _ in range(3):
            sim.solve_collision_constraints_x()
        outs.append(_np(cl.y4).copy())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("cap", [40, 64, 80])
def test_contact_pair_list_layout(pkg, cap):
    """The flattened pair list equals a host restatement of its definition:
    queries in order (vertex vs obstacle, vertex vs cloth, obstacle vertex vs
    cloth), each query's candidates in list order, vertex-vs-cloth candidates
    incident to the query dropped, (query, triangle vertices) per pair; the
    kind boundaries in the workspace's last 256 bytes."""
    sc, cl, sp = _drape(pkg, n=40)
    sim = pkg.Solver(cl, sp, dHat=(4e-2) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8, g=(0, 0, -9.81),
                     dt=1 / 60, cap=cap)
    sim.padding = 0.06
    sim.enable_collision_handling = True
    x = _np(cl.x4).copy()
    x[:, 2] = 0.5 + 0.3 + 0.01 * np.sin(13 * x[:, 0]) * np.cos(7 * x[:, 1])
    cl.x4.copy_(_t(x))
    sim.build_bvhs()
    sim.compute_y(1 / 600)
    sim.broadphase_lbvh()
    sim.build_contact_pairs()
    torch.cuda.synchronize()
    fd, fs = cl.fid_np.reshape(-1, 3), sp.fid_np.reshape(-1, 3)
    Vd, Vs = cl.num_verts, sp.num_verts
    ref = []
    c, n = _np(sim.vt_st_candidates), _np(sim.vt_st_candidates_num)
    for q in range(Vd):
        for f in c[q, :min(n[q], cap)]:
            ref.append((q, *fs[f]))
    st_end = len(ref)
    c, n = _np(sim.vt_dy_candidates), _np(sim.vt_dy_candidates_num)
    for q in range(Vd):
        for f in c[q, :min(n[q], cap)]:
            if q not in fd[f]:
                ref.append((q, *fd[f]))
    dy_end = len(ref)
    c, n = _np(sim.tv_st_candidates), _np(sim.tv_st_candidates_num)
    for q in range(Vs):
        for f in c[q, :min(n[q], cap)]:
            ref.append((q, *fd[f]))
    ref = np.array(ref, np.int32).reshape(-1, 4)
    P = sim.contact_pair_count()
    meta = sim._pairs_ws[-256:].view(torch.int32)[:3].cpu().numpy()
    assert P == ref.shape[0] and tuple(meta) == (st_end, dy_end, P)
    assert st_end > 0 and dy_end > st_end and P > dy_end
    assert int(_np(sim.vt_dy_candidates_num).max()) > 0
    assert np.array_equal(_np(sim._pairs)[:P], ref)


@pytest.mark.parametrize("cull", [False, True])
def test_pair_projection_variants_agree(pkg, cull):
    """Every compiled launch configuration of the pair projection adds the same
    fixed-point corrections and counts as the default one."""
    from starlab_physics_gb300._lib import ptr, sx, stream_handle

    sc, cl, sp = _drape(pkg, n=40)
    sim = pkg.Solver(cl, sp, dHat=(4e-2) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8, g=(0, 0, -9.81),
                     dt=1 / 60, record_pairs=False)
    sim.padding = 0.04
    sim.enable_collision_handling = True
    x = _np(cl.x4).copy()
    x[:, 2] = 0.5 + 0.3 + 0.01 * np.sin(13 * x[:, 0]) * np.cos(7 * x[:, 1])
    cl.x4.copy_(_t(x))
    sim.build_bvhs()
    sim.compute_y(1 / 600)
    sim.broadphase_lbvh()
    sim.contact_cull = cull
    sim.build_contact_pairs()
    torch.cuda.synchronize()
    assert sim.contact_pair_count() > 1000
    V, Vs = cl.num_verts, sp.num_verts
    n_var = sx.sx_contact_pairs_project_variants()
    assert n_var >= 2
    outs = []
    for v in [None, *range(n_var)]:
        sim._dx_fix.zero_()
        sim._nc.zero_()
        args = (V, Vs, ptr(sim._pairs), ptr(sim._pairs_ws), ptr(cl.y4), ptr(sp.x4), ptr(cl.fixed), ptr(cl.m_inv),
                sim.dHat, float(sim.compliance_collision), sim.contact_cull_d2(), ptr(sim._dx_fix), ptr(sim._nc),
                ptr(sim.status), None, 0)
        if v is None:
            sx.sx_contact_pairs_project(*args, stream_handle())
        else:
            sx.sx_contact_pairs_project_v(*args, v, stream_handle())
        torch.cuda.synchronize()
        outs.append((_np(sim._dx_fix).copy(), _np(sim._nc).copy()))
    assert outs[0][1].sum() > 0
    for dxf, nc in outs[1:]:
        assert np.array_equal(dxf, outs[0][0]) and np.array_equal(nc, outs[0][1])
    assert int(sim.status.item()) & 4 == 0  # SX_STATUS_FIXED_RANGE
    sim._dx_fix.zero_()
    sim._nc.zero_()


@pytest.mark.parametrize("n_iter", [3, 4])
def test_graph_replay_equals_eager(pkg, n_iter):
    res = []
    for use_graph in (False, True):
        scene = pkg.scenes.plain64(n=20, seed=6)
        scene.n_iter = n_iter
        sim = pkg.scenes.make_solver(scene, device=DEV)
        sim.bending_on = "y"
        sim.use_graph = use_graph
        for _ in range(4):
            sim.forward(scene.n_substeps)
        torch.cuda.synchronize()
        res.append((_np(sim.mesh_dy.x4), _np(sim.mesh_dy.v4), _np(sim.mesh_dy.y4)))
    for a, b in zip(*res):
        assert np.array_equal(a, b)


def test_system_energy(pkg, po):
    """The FP64 energy reduction against the oracle's float64 sums (same
    terms, another summation order: agreement to 1e-12 relative)."""
    scene = pkg.scenes.drape256(n=48, seed=3, sphere_subdiv=3)
    sim = pkg.scenes.make_solver(scene, device=DEV)
    sim.bending_on = "y"
    for _ in range(2):
        sim.forward(scene.n_substeps)
    e = sim.system_energy().cpu().numpy()
    m = sim.mesh_dy
    ref = po.system_energy(_np(m.x4), _np(m.v4), _np(m.m_inv), _np(m.adj_ptr), _np(m.adj), sim.stiffness_bending,
                           sim.stiffness_stretch, sim.g)
    for got, want in zip(e, ref):
        assert abs(got - want) <= 1e-12 * max(abs(want), 1e-30), (got, want)
    assert e[0] > 0 and e[2] > 0
    # deterministic
    assert np.array_equal(sim.system_energy().cpu().numpy(), e)


def test_constraint_residual(pkg, po):
    """sx_constraint_residual equals the oracle's restatement of its summation
    order bit for bit, and the FP64 value agrees with a float64 evaluation."""
    scene = pkg.scenes.plain64(n=24, seed=2)
    scene.n_iter = 3
    sim = pkg.scenes.make_solver(scene, device=DEV)
    sim.bending_on = "y"
    for _ in range(2):
        sim.forward(scene.n_substeps)
    m = sim.mesh_dy
    for which in ("x", "y"):
        r = sim.constraint_residual(which).cpu().numpy()
        p = _np(m.x4 if which == "x" else m.y4)
        ref = po.constraint_residual(p, m.eid_np, m.l0_np, m.bending_np, m.bending_l0_np)
        assert int(r[1]) == 2 * (m.num_edges + m.bending_constraint_count)
        assert np.array_equal(r[:3], ref), (r, ref)
        # float64 evaluation of the same quantity
        pp = p[:, :3].astype(np.float64)
        prs = np.concatenate([m.eid_np.reshape(-1, 2), m.bending_np.reshape(-1, 2)])
        rest = np.concatenate([m.l0_np, m.bending_l0_np]).astype(np.float64)
        C = np.linalg.norm(pp[prs[:, 0]] - pp[prs[:, 1]], axis=1) - rest
        assert abs(r[2] - np.sqrt(np.mean(C * C))) <= 1e-4 * r[2]


def _tol_run(pkg, po, tol, frames=3, n_iter=16, use_graph=False, relative=False):
    scene = pkg.scenes.plain64(n=24, seed=4)
    scene.n_iter = n_iter
    sim = pkg.scenes.make_solver(scene, device=DEV)
    sim.bending_on = "y"
    sim.tol = tol
    sim.tol_relative = relative
    sim.use_graph = use_graph
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(sim.mesh_dy), pkg.scenes.oracle_inputs(sim.mesh_st),
                          dt=scene.dt, g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                          k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                          padding=scene.padding, n_iter=n_iter, collisions=scene.collisions, rebuild=scene.rebuild,
                          cap=scene.cap, bending_on="y", contact_cull=sim.contact_cull, tol=tol,
                          tol_relative=relative)
    for _ in range(frames):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
    torch.cuda.synchronize()
    return sim, orc


@pytest.mark.parametrize("use_graph", [False, True])
def test_tolerance_mode_matches_oracle(pkg, po, use_graph):
    """Iterating to a residual: the device-side stop decisions and the positions
    equal the oracle's, for a tolerance that is met at some checks and missed
    at others."""
    # the residual after the first check of a free run sets the tolerance
    probe_sim, probe = _tol_run(pkg, po, tol=0.0, frames=1)
    tol = float(probe.last_residual[2]) * 1.0000001
    sim, orc = _tol_run(pkg, po, tol=tol, use_graph=use_graph)
    st = sim.convergence_stats()
    assert st["converged_substeps"] == orc.converged
    assert 0 < orc.converged < 30, orc.converged
    assert st["mean_stop_iteration"] == orc.stop_sum / orc.converged
    assert np.array_equal(_np(sim.mesh_dy.x4)[:, :3], orc.x4[:, :3])


@pytest.mark.parametrize("rho", [0.999, 0.99])
def test_relative_tolerance_matches_oracle(pkg, po, rho):
    """Tolerance relative to each substep's cold-start residual."""
    sim, orc = _tol_run(pkg, po, tol=rho, relative=True)
    st = sim.convergence_stats()
    assert st["converged_substeps"] == orc.converged > 0
    assert st["mean_stop_iteration"] == orc.stop_sum / orc.converged
    assert np.array_equal(_np(sim.mesh_dy.x4)[:, :3], orc.x4[:, :3])


def test_tolerance_mode_extremes(pkg, po):
    """tol large: every substep stops at the first check, iteration 4, and its
    block (iterations 4..7) completes; tol 0: none stops.  Both equal
    fixed-count runs."""
    sim, orc = _tol_run(pkg, po, tol=1.0, frames=2)
    assert sim.convergence_stats()["converged_substeps"] == 20 == orc.converged
    fixed_sim, fixed_orc = _tol_run(pkg, po, tol=None, frames=2, n_iter=8)
    assert np.array_equal(_np(sim.mesh_dy.x4), _np(fixed_sim.mesh_dy.x4))
    sim0, _ = _tol_run(pkg, po, tol=0.0, frames=2)
    full, _ = _tol_run(pkg, po, tol=None, frames=2)
    assert sim0.convergence_stats()["converged_substeps"] == 0
    assert np.array_equal(_np(sim0.mesh_dy.x4), _np(full.mesh_dy.x4))
    # the device-side loop of a captured frame gives the same iterations
    g_big, _ = _tol_run(pkg, po, tol=1.0, frames=2, use_graph=True)
    assert np.array_equal(_np(g_big.mesh_dy.x4), _np(fixed_sim.mesh_dy.x4))
    g0, _ = _tol_run(pkg, po, tol=0.0, frames=2, use_graph=True)
    assert np.array_equal(_np(g0.mesh_dy.x4), _np(full.mesh_dy.x4))


def test_sewing_matches_oracle(pkg, po):
    """Sewing constraints (two edges of a cloth sewn together) through the
    solver, against the oracle, bit for bit; the sewn vertices approach."""
    scene = pkg.scenes.plain64(n=16, seed=5, collisions=False)
    scene.n_iter = 4
    sim = pkg.scenes.make_solver(scene, device=DEV)
    sim.bending_on = "y"
    n = 16
    pairs = np.array([[i, (n - 1) * n + i] for i in range(2, n - 2)], np.int32)  # first row to last row
    sim.set_sewing_pairs(pairs, 1e5)
    sewn, sptr, partner = pkg.mesh.sewing_adjacency(sim.mesh_dy.num_verts, pairs)
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(sim.mesh_dy), None, dt=scene.dt, g=scene.gravity,
                          k_stretch_stiffness=scene.stiffness_stretch, k_bend_stiffness=scene.stiffness_bending,
                          dHat=scene.dHat, damping=scene.damping, padding=scene.padding, n_iter=scene.n_iter,
                          collisions=False, rebuild=scene.rebuild, cap=scene.cap, bending_on="y",
                          sewing=(sewn, sptr, partner, 1e5))
    x0 = _np(sim.mesh_dy.x4).copy()
    for _ in range(3):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
    torch.cuda.synchronize()
    gx = _np(sim.mesh_dy.x4)
    assert np.array_equal(gx[:, :3], orc.x4[:, :3])
    d0 = np.linalg.norm(x0[pairs[:, 0], :3] - x0[pairs[:, 1], :3], axis=1)
    d1 = np.linalg.norm(gx[pairs[:, 0], :3] - gx[pairs[:, 1], :3], axis=1)
    assert np.all(d1 < d0)


def test_velocity_contacts_all_branches(pkg, po, sxm):
    """solve_constraints_v over synthetic pair records that exercise every
    region of every kind (random g, schur, velocities; half the records with
    Cv < 0): the kernel equals the oracle's branch-by-branch restatement."""
    rng = np.random.default_rng(21)
    Vd, Vs, cap = 300, 120, 6
    faces_dy = rng.integers(0, Vd, (200, 3)).astype(np.int32)
    faces_st = rng.integers(0, Vs, (80, 3)).astype(np.int32)
    Q = 2 * Vd + Vs
    num = rng.integers(0, cap + 1, Q).astype(np.int32)
    pair = np.zeros((Q, cap, 2), np.int32)
    pair[:Vd, :, 0] = rng.integers(0, 80, (Vd, cap))
    pair[Vd:, :, 0] = rng.integers(0, 200, (Vd + Vs, cap))
    pair[:, :, 1] = rng.integers(0, 7, (Q, cap))
    g = np.zeros((Q, cap, 4, 4), np.float32)
    g[..., :3] = rng.normal(0, 1, (Q, cap, 4, 3))
    schur = rng.uniform(0.5, 3.0, (Q, cap)).astype(np.float32)
    v4 = np.zeros((Vd, 4), np.float32)
    v4[:, :3] = rng.normal(0, 1, (Vd, 3))
    vs4 = np.zeros((Vs, 4), np.float32)
    vs4[:, :3] = rng.normal(0, 0.3, (Vs, 3))
    fixed = (rng.uniform(size=Vd) > 0.1).astype(np.float32)
    m_inv = rng.uniform(0.5, 2.0, Vd).astype(np.float32)
    m_inv[:5] = 0.0
    m_inv_st = rng.uniform(0.5, 2.0, Vs).astype(np.float32)
    rec = {"pair": pair, "pair_g": g, "pair_schur": schur, "pair_num": num}
    ref = v4.copy()
    po.velocity_contacts(faces_dy, faces_st, cap, rec, ref, vs4, fixed, m_inv, m_inv_st, 0.3)
    t = {k: _t(np.ascontiguousarray(a)) for k, a in
         dict(fd=faces_dy, fs=faces_st, pair=pair, g=g, schur=schur, num=num, v=v4, vs=vs4, fixed=fixed,
              m=m_inv, ms=m_inv_st).items()}
    dv = torch.zeros(3 * Vd, dtype=torch.int64, device=DEV)
    nc = torch.zeros(Vd, dtype=torch.int32, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    sxm.sx.sx_velocity_contacts(Vd, Vs, t["fd"].data_ptr(), t["fs"].data_ptr(), cap, t["pair"].data_ptr(),
                                t["g"].data_ptr(), t["schur"].data_ptr(), t["num"].data_ptr(), t["v"].data_ptr(),
                                t["vs"].data_ptr(), t["fixed"].data_ptr(), t["m"].data_ptr(), t["ms"].data_ptr(), 0.3,
                                dv.data_ptr(), nc.data_ptr(), status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    got = _np(t["v"])
    assert not np.array_equal(ref, v4)
    assert np.array_equal(got[:, :3], ref[:, :3]), np.abs(got - ref).max()
    assert not _np(dv).any() and not _np(nc).any()


def test_velocity_pass_solver_matches_oracle(pkg, po):
    """enable_velocity_update through the solver (contacts on a box, pair
    records kept), against the oracle, bit for bit."""
    scene = pkg.scenes.plain64(n=24, seed=7)
    scene.n_iter = 3
    from starlab_physics_gb300 import mesh as M

    cl = M.TriMesh(scene.cloth_x, scene.cloth_faces, device=DEV)
    ob = M.TriMesh(scene.obstacle_x, scene.obstacle_faces, device=DEV, is_static=True)
    sim = pkg.Solver(cl, ob, dHat=scene.dHat, stiffness_stretch=scene.stiffness_stretch,
                     stiffness_bending=scene.stiffness_bending, g=scene.gravity, dt=scene.dt, n_iter=scene.n_iter,
                     rebuild=scene.rebuild, record_pairs=True, bending_on="y")
    mask = np.zeros(cl.num_verts, np.int32)
    mask[scene.pinned] = 1
    sim.set_fixed_vertices(torch.from_numpy(mask))
    sim.damping = scene.damping
    sim.padding = scene.padding
    sim.enable_collision_handling = True
    sim.enable_velocity_update = True
    sim.mu = 0.4
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), dt=scene.dt, g=scene.gravity,
                          k_stretch_stiffness=scene.stiffness_stretch, k_bend_stiffness=scene.stiffness_bending,
                          dHat=scene.dHat, damping=scene.damping, padding=scene.padding, n_iter=scene.n_iter,
                          collisions=True, rebuild=scene.rebuild, cap=scene.cap, bending_on="y", contact_cull=False,
                          velocity_update=True, mu=0.4)
    plain = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), dt=scene.dt,
                            g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                            k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                            padding=scene.padding, n_iter=scene.n_iter, collisions=True, rebuild=scene.rebuild,
                            cap=scene.cap, bending_on="y", contact_cull=False)
    for _ in range(30):
        sim.forward(scene.n_substeps)
        orc.forward(scene.n_substeps)
        plain.forward(scene.n_substeps)
    torch.cuda.synchronize()
    assert int(_np(sim.pair_num).sum()) > 0, "no contact records"
    assert not np.array_equal(orc.x4, plain.x4), "the velocity pass changed nothing"
    assert np.array_equal(_np(cl.x4)[:, :3], orc.x4[:, :3])
    assert np.array_equal(_np(cl.v4)[:, :3], orc.v4[:, :3])


@pytest.mark.parametrize("use_graph", [False, True])
def test_programmatic_launch_gives_the_same_frames(pkg, sxm, use_graph):
    """Kernels launched as programmatic dependents (the default) give the same
    frames as plain launches."""
    lib = sxm.load()
    res = []
    prev = lib.sx_set_programmatic_launch(1)
    try:
        for pdl in (0, 1):
            lib.sx_set_programmatic_launch(pdl)
            scene = pkg.scenes.plain64(n=24, seed=9)
            scene.n_iter = 6
            sim = pkg.scenes.make_solver(scene, device=DEV)
            sim.bending_on = "y"
            sim.use_graph = use_graph
            for _ in range(3):
                sim.forward(scene.n_substeps)
            torch.cuda.synchronize()
            res.append((_np(sim.mesh_dy.x4), _np(sim.mesh_dy.v4)))
    finally:
        lib.sx_set_programmatic_launch(prev)
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
