"""The CPU oracle against golden vectors produced by the reference's own source
(tests/golden/make_reference_vectors.py runs distance.py, lbvh_cell.py,
XPBD.py, graph_coloring.py and meshTaichiWrapper.py of the reference through a
numpy stand-in for the Taichi API: serial loops, IEEE float32 per operation).
No reference checkout needed; the tests marked gpu hold the CUDA library to the
same vectors."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def R():
    return np.load(GOLDEN)


def test_point_triangle_matches_reference(po, R):
    """d_type_PT and the branch distance bit for bit; our closed-form gradients
    against the reference's generated ones within float32 rounding."""
    dt, d, g = po.point_triangles(R["pt_points"])
    assert np.array_equal(dt, R["pt_dtype"])
    assert np.array_equal(d, R["pt_d"])
    assert set(dt.tolist()) == set(range(7))
    sc = np.abs(R["pt_g"]).reshape(-1, 12).max(1)
    ok = sc > 0
    errs = np.abs(g - R["pt_g"]).reshape(-1, 12).max(1)[ok] / sc[ok]
    assert np.median(errs) < 1e-6 and errs.max() < 2e-2


def test_edge_edge_matches_reference(po, R):
    E = R["ee_points"]
    dt, d, _ = po.edge_edge_classify(E, np.float32(1e30))
    assert np.array_equal(dt, R["ee_dtype"])
    assert set(dt.tolist()) == set(range(9))
    x = E.reshape(-1, 4, 3).astype(np.float32)
    c = np.cross(x[:, 0] - x[:, 1], x[:, 2] - x[:, 3]).astype(np.float32)
    projected = (dt == 8) & (np.sqrt((c * c).sum(1)) > 1e-3)
    assert projected.sum() > 100
    assert np.array_equal(d[projected], R["ee_d"][projected])


def test_morton_matches_reference(po, R):
    assert np.array_equal(po.morton3d(R["morton_points"]), R["morton_codes"])


def test_substeps_match_reference(pkg, po, R):
    """Three reference substeps of a pinned 7 x 7 cloth (compute_y, one
    spring + bending sweep with update_dx, bending on x, compute_velocity,
    update_x), bit for bit."""
    x0, v0, f, fixed = R["sub_x0"], R["sub_v0"], R["sub_faces"], R["sub_fixed"]
    dt_frame, n_sub, damping, kss, kbs = R["sub_params"]
    n_sub = int(n_sub)
    dt = float(dt_frame) / n_sub
    m = pkg.TriMesh(x0, f, device="cpu")
    V = x0.shape[0]
    x4 = np.zeros((V, 4), np.float32)
    x4[:, :3] = x0
    x4[:, 3] = fixed * m.m_inv_np
    v4 = np.zeros((V, 4), np.float32)
    v4[:, :3] = v0
    for s in range(n_sub):
        y4 = po.predict(x4, v4, fixed, dt, np.array([0.0, 0.0, -9.81], np.float32))
        po.spring_sweep(x4, y4, fixed, m.m_inv_np, m.eid_np, m.l0_np, m.bending_np, m.bending_l0_np,
                        float(kbs) * dt * dt, float(kss) * dt * dt, bend_on_y=0)
        assert np.array_equal(y4[:, :3], R["sub_y"][s]), s
        po.velocity_update(x4, y4, v4, fixed, float(damping), dt)
        assert np.array_equal(x4[:, :3], R["sub_x"][s]), s
        assert np.array_equal(v4[:, :3], R["sub_v"][s]), s


def _digest(a):
    import hashlib

    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), dtype=np.uint8)


def test_cell_bvh_matches_reference(po, R):
    """LBVH_CELL: the cell codes and Karras topology of __init__, the build's
    prefix sums, sorted faces, leaf/node boxes and face counts, and the
    candidate lists of traverse_cell_bvh_single (order included)."""
    b = po.CellBVH()
    init = [b.codes, b.ids, b.child_a, b.child_b, b.parent[1:], b.range_l, b.range_r]
    for k, a in enumerate(init):
        assert np.array_equal(_digest(a.astype(np.int32)), R["lbvh_init_digest"][k]), k
    x4, f, pad = R["lbvh_x4"], R["lbvh_faces"], R["lbvh_pad"][0]
    mn, mx = po.face_aabbs(x4, f, pad)
    b.build(mn, mx, po.scene_aabb(x4, pad))
    assert np.array_equal(b.cell_size, R["lbvh_cell_size"])
    built = [b.prefix, b.sorted_face_ids, b.num_faces, np.ascontiguousarray(b.nmin4[:, :3]),
             np.ascontiguousarray(b.nmax4[:, :3])]
    for k, a in enumerate(built):
        assert np.array_equal(_digest(a), R["lbvh_build_digest"][k]), k
    qmn, qmx = po.query_boxes(x4, pad)
    cand, num, _ = b.traverse(qmn, qmx, R["lbvh_cand"].shape[1])
    assert np.array_equal(num, R["lbvh_num"]) and num.sum() > 100
    for q in range(num.shape[0]):
        k = min(num[q], cand.shape[1])
        assert np.array_equal(cand[q, :k], R["lbvh_cand"][q, :k]), q


def test_contacts_match_reference(po, R):
    """solve_collision_constraints_x + update_dx of the reference on two cloth
    layers over a box: the pair records of all three contact kinds (face and
    region) equal the oracle's; gradients, Schur complements and the updated
    positions agree to float32 rounding (the reference's generated gradient
    expressions and our closed forms round differently; the reference sums
    corrections in float, the oracle in fixed point)."""
    x4, f, xs4, fs = R["ct_x4"], R["ct_faces"], R["ct_xs4"], R["ct_faces_st"]
    pad, dHat, comp, cap = R["ct_params"]
    cap = int(cap)
    Vd, Vs = x4.shape[0], xs4.shape[0]
    bd, bs = po.CellBVH(), po.CellBVH()
    mn, mx = po.face_aabbs(x4, f, pad)
    bd.build(mn, mx, po.scene_aabb(x4, pad))
    mn, mx = po.face_aabbs(xs4, fs, pad)
    bs.build(mn, mx, po.scene_aabb(xs4, pad))
    qd, qs = po.query_boxes(x4, pad), po.query_boxes(xs4, pad)
    vt_st, vt_dy, tv_st = bs.traverse(*qd, cap), bd.traverse(*qd, cap), bd.traverse(*qs, cap)
    y4 = x4.copy()
    r = po.collision_sweep(f, fs, y4, xs4, R["ct_fixed"], R["ct_m_inv"], np.float32(dHat), np.float32(comp), cap,
                           vt_st[:2], vt_dy[:2], tv_st[:2], want_pairs=True)
    blocks = {"vt_st": (0, Vd), "vt_dy": (Vd, 2 * Vd), "tv_st": (2 * Vd, 2 * Vd + Vs)}
    for name, (a, b) in blocks.items():
        pn = r["pair_num"][a:b]
        assert np.array_equal(pn, R["ct_%s_pair_num" % name]), name
        assert pn.sum() > 20, name
        mask = np.arange(cap)[None, :] < pn[:, None]
        assert np.array_equal(r["pair"][a:b][mask], R["ct_%s_pair" % name][mask]), name
        g, rg = r["pair_g"][a:b, :, :, :3][mask], R["ct_%s_pair_g" % name][mask]
        assert np.abs(g - rg).max() <= 1e-5 * np.abs(rg).max(), name
        s, rs = r["pair_schur"][a:b][mask], R["ct_%s_pair_schur" % name][mask]
        assert np.abs(s - rs).max() <= 1e-5 * np.abs(rs).max(), name
    moved = np.abs(R["ct_y"] - x4[:, :3]).max()
    assert moved > 1e-3
    assert np.abs(y4[:, :3] - R["ct_y"]).max() <= 1e-5 * moved


def test_velocity_pass_matches_reference(po, R):
    """solve_constraints_v of the reference (friction over the pair records of
    the position pass, then update_dv) on the same scene: the oracle's
    velocity pass over its own records gives the same velocities to float32
    rounding (the gradients and Schur complements it reads differ from the
    reference's in the last bits, see the test above)."""
    x4, f, xs4, fs = R["ct_x4"], R["ct_faces"], R["ct_xs4"], R["ct_faces_st"]
    pad, dHat, comp, cap = R["ct_params"]
    cap = int(cap)
    Vd, Vs = x4.shape[0], xs4.shape[0]
    bd, bs = po.CellBVH(), po.CellBVH()
    mn, mx = po.face_aabbs(x4, f, pad)
    bd.build(mn, mx, po.scene_aabb(x4, pad))
    mn, mx = po.face_aabbs(xs4, fs, pad)
    bs.build(mn, mx, po.scene_aabb(xs4, pad))
    qd, qs = po.query_boxes(x4, pad), po.query_boxes(xs4, pad)
    vt_st, vt_dy, tv_st = bs.traverse(*qd, cap), bd.traverse(*qd, cap), bd.traverse(*qs, cap)
    y4 = x4.copy()
    r = po.collision_sweep(f, fs, y4, xs4, R["ct_fixed"], R["ct_m_inv"], np.float32(dHat), np.float32(comp), cap,
                           vt_st[:2], vt_dy[:2], tv_st[:2], want_pairs=True)
    v4 = np.zeros((Vd, 4), np.float32)
    v4[:, :3] = R["ct_v0"]
    vs4 = np.zeros((Vs, 4), np.float32)
    vs4[:, :3] = R["ct_vs0"]
    status = po.velocity_contacts(f, fs, cap, r, v4, vs4, R["ct_fixed"], R["ct_m_inv"], np.ones(Vs, np.float32),
                                  float(R["ct_mu"][0]))
    assert status == 0
    changed = np.abs(R["ct_v"] - R["ct_v0"]).max(1) > 0
    assert changed.sum() > 10
    dv = np.abs(R["ct_v"] - R["ct_v0"]).max()
    assert np.array_equal(np.abs(v4[:, :3] - R["ct_v0"]).max(1) > 0, changed)
    assert np.abs(v4[:, :3] - R["ct_v"]).max() <= 1e-5 * max(dv, np.abs(R["ct_v"]).max())


@pytest.mark.parametrize("k", [0, 1, 2])
def test_coloring_matches_reference(po, R, k):
    """GraphColoring.colorEdgesGreedy + colorCountingSort (graph_coloring.py:
    131-149, 172-201) on two grid cloths and an icosphere: colours, colour-sorted
    edge sequence and start offsets bit for bit."""
    e = R["col%d_edges" % k]
    color, sorted_e, prefix = po.color_edges(int(e.max()) + 1, e)
    assert np.array_equal(color, R["col%d_color" % k])
    assert np.array_equal(sorted_e, R["col%d_sorted" % k])
    assert np.array_equal(prefix, R["col%d_prefix" % k])


@pytest.mark.parametrize("k", [0, 1])
def test_mesh_init_matches_reference(pkg, R, k):
    """findTriNeighbors / getBendingPair / init_bengding_l0 and initEdgeIndices
    (meshTaichiWrapper.py:142-145, 177-225, 244-256): bending pairs in the
    reference's order, their rest lengths, spring rest lengths and the inverse
    masses 1 / sum(l0 / 2), bit for bit, through the product's mesh set-up."""
    x, f = R["mi%d_x" % k], R["mi%d_faces" % k]
    m = pkg.TriMesh(x, f, device="cpu")
    assert np.array_equal(m.eid_np.reshape(-1), R["mi%d_edge_indices" % k])
    assert np.array_equal(m.bending_np.reshape(-1, 2), R["mi%d_bend" % k])
    assert np.array_equal(m.bending_l0_np, R["mi%d_bend_l0" % k])
    assert np.array_equal(m.l0_np, R["mi%d_l0" % k])
    assert np.array_equal(m.m_inv_np, R["mi%d_m_inv" % k])


@pytest.mark.parametrize("k", [0, 1])
def test_karras_repeated_codes_match_reference(po, R, k):
    """assign_internal_nodes_Karras12 with delta/find_split/determine_range
    (lbvh_cell.py:256-336, 384-405) on sorted codes with long runs of equal
    codes (the reference's equal-code rule, oracle tie = 0): children and ranges
    bit for bit; parents equal wherever the reference writes one (nodes its
    malformed tree never claims keep the field's initial 0 there and -1 here)."""
    codes = R["kd%d_codes" % k]
    ca, cb, rl, rr, par = po.karras(codes, tie=0)
    assert np.array_equal(ca, R["kd%d_child_a" % k]) and np.array_equal(cb, R["kd%d_child_b" % k])
    assert np.array_equal(rl, R["kd%d_range_l" % k]) and np.array_equal(rr, R["kd%d_range_r" % k])
    written = par >= 0
    assert np.array_equal(par[written], R["kd%d_parent" % k][written])
    assert np.all(R["kd%d_parent" % k][~written] == 0)
    assert (~written).sum() > 1   # duplicates leave nodes unclaimed besides the root


@pytest.mark.gpu
def test_gpu_coloring_and_karras_match_reference(pkg, R):
    """The CUDA colouring (sx_color_edges_greedy) and Karras build
    (sx_karras_build, tie = 0) against the same reference vectors."""
    import torch
    from starlab_physics_gb300._lib import ptr, stream_handle, sx

    for k in range(3):
        e = R["col%d_edges" % k]
        gc = pkg.GraphColoring(int(e.max()) + 1, e, device="cuda")
        E = e.shape[0]
        assert np.array_equal(gc.edges_color.cpu().numpy()[:E], R["col%d_color" % k])
        assert np.array_equal(gc.sorted_edges_sequence_for_color.cpu().numpy()[:E], R["col%d_sorted" % k])
        assert np.array_equal(gc.color_prefix_sum.cpu().numpy(), R["col%d_prefix" % k])
    for k in range(2):
        codes = R["kd%d_codes" % k]
        n = codes.shape[0]
        c = torch.from_numpy(codes).cuda()
        i32 = dict(dtype=torch.int32, device="cuda")
        ca, cb, rl, rr = (torch.full((n - 1,), -7, **i32) for _ in range(4))
        par = torch.full((2 * n - 1,), -7, **i32)
        assert sx.sx_karras_build(ptr(c), n, 0, ptr(ca), ptr(cb), ptr(rl), ptr(rr), ptr(par), stream_handle()) == 0
        torch.cuda.synchronize()
        for got, name in ((ca, "child_a"), (cb, "child_b"), (rl, "range_l"), (rr, "range_r")):
            assert np.array_equal(got.cpu().numpy(), R["kd%d_%s" % (k, name)]), name
        kids = np.concatenate([R["kd%d_child_a" % k], R["kd%d_child_b" % k]])
        once = np.bincount(kids, minlength=2 * n - 1) == 1
        assert np.array_equal(par.cpu().numpy()[once], R["kd%d_parent" % k][once])
