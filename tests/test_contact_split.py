"""The contact-pair split by motion (sx_contact_pairs_split /
sx_contact_pairs_project_moved), checked on the CPU through the oracle's
restatement of it (or_split_far / or_split_skip, the kernels' formulas).

A far pair is one whose distance at the reference positions exceeds the cull
distance plus twice the motion budget on a triangle that stays classifiable
under any move of its vertices below the budget; later iterations leave it out
while none of its dynamic vertices has moved by the budget.  These tests show
(1) that no far pair perturbed by less than the budget reaches a contact under
the reference's classifier and distances, on adversarial inputs, and (2) that
whole oracle runs with the split equal runs without it bit for bit while the
split leaves out most pairs."""
import numpy as np
import pytest


def _quads_scene(p, tri):
    """n point-triangle quadruples as a cloth of 4n vertices whose vertex 4i has
    the single vertex-vs-own-cloth candidate face i = (4i+1, 4i+2, 4i+3)."""
    n = p.shape[0]
    y4 = np.zeros((4 * n, 4), np.float32)
    y4[0::4, :3] = p
    y4[1::4, :3] = tri[:, 0]
    y4[2::4, :3] = tri[:, 1]
    y4[3::4, :3] = tri[:, 2]
    faces = (4 * np.arange(n)[:, None] + np.arange(1, 4)[None, :]).astype(np.int32)
    cap = 1
    c = np.zeros((4 * n, cap), np.int32)
    num = np.zeros(4 * n, np.int32)
    c[0::4, 0] = np.arange(n)
    num[0::4] = 1
    empty = (np.zeros((4 * n, cap), np.int32), np.zeros(4 * n, np.int32))
    none_st = (np.zeros((0, cap), np.int32), np.zeros(0, np.int32))
    return y4, faces, cap, empty, (c, num), none_st


def _closest_point(p, a, b, c):
    """Closest point of triangle abc to p (float64, Ericson's regions)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        return a
    bp = p - b
    d3, d4 = ab @ bp, ac @ bp
    if d3 >= 0 and d4 <= d3:
        return b
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        return a + d1 / (d1 - d3) * ab
    cp = p - c
    d5, d6 = ab @ cp, ac @ cp
    if d6 >= 0 and d5 <= d6:
        return c
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        return a + d2 / (d2 - d6) * ac
    va = d3 * d6 - d5 * d4
    if va <= 0 and d4 - d3 >= 0 and d5 - d6 >= 0:
        return b + (d4 - d3) / ((d4 - d3) + (d5 - d6)) * (c - b)
    den = 1.0 / (va + vb + vc)
    return a + ab * (vb * den) + ac * (vc * den)


@pytest.mark.parametrize("budget_rel", [0.05, 0.5])
def test_far_pairs_moved_below_budget_stay_out_of_contact(po, budget_rel):
    """Sheets of triangles at 1.2-3 contact distances with points beside them,
    random triangles (slivers and tiny ones among them) with points at 0.8-1.6
    contact distances plus twice the budget; every far pair is then moved by
    just under the budget per vertex -- the point towards the triangle, the
    triangle towards the point, and random directions -- and classified by the
    oracle's restatement of d_type_PT / d_PP / d_PE / d_PT: none reaches
    d < dHat, and the skip test leaves every such pair out."""
    rng = np.random.default_rng(21)
    dHat = np.float32(2e-3) ** 2
    cull = np.float32(dHat * np.float32(1.0625))
    r = float(np.sqrt(np.float64(cull)))
    beta = np.float32(budget_rel * r)
    P, T = [], []
    for _ in range(6000):
        size = 10 ** rng.uniform(-4, -1.5)
        tri = rng.normal(0, size, (3, 3))
        if rng.random() < 0.3:
            tri[2] = tri[0] + (tri[1] - tri[0]) * rng.uniform(0, 1) + rng.normal(0, size * 1e-3, 3)
        tri += 0.6
        w = rng.dirichlet(np.ones(3))
        q = w @ tri
        dirn = rng.normal(size=3)
        if rng.random() < 0.5:  # in the plane of the triangle
            nrm = np.cross(tri[1] - tri[0], tri[2] - tri[0])
            nrm /= np.linalg.norm(nrm) + 1e-300
            dirn -= (dirn @ nrm) * nrm
        dirn /= np.linalg.norm(dirn) + 1e-300
        P.append(q + dirn * (r + 2 * float(beta)) * rng.uniform(0.8, 1.6))
        T.append(tri)
    # flat and bent sheets: each vertex against nearby triangles not containing it
    for h_over_r, bend in ((1.2, 0.0), (2.0, 0.3), (3.0, 1.0)):
        n = 8
        h = h_over_r * r
        u, v = np.meshgrid(np.arange(n) * h, np.arange(n) * h, indexing="ij")
        z = bend * h * np.sin(u / (3 * h)) * np.cos(v / (2 * h))
        X = np.stack([u, v, z], -1).reshape(-1, 3) + rng.normal(0, 0.05 * h, (n * n, 3)) + 0.5
        for i in range(n - 1):
            for j in range(n - 1):
                a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
                for f in ((a, b, c), (a, c, d)):
                    for qv in range(n * n):
                        if qv not in f and np.abs(X[list(f)].mean(0) - X[qv]).max() < 3 * h:
                            P.append(X[qv])
                            T.append(X[list(f)])
    p = np.asarray(P, np.float32)
    tri = np.asarray(T, np.float32)
    y4, faces, cap, vt_st, vt_dy, tv_st = _quads_scene(p, tri)
    far = po.split_far(faces, None, y4, None, cap, vt_st, vt_dy, tv_st, cull, beta)
    Vd = y4.shape[0]
    # the vertex-vs-own-cloth block of the slots: rows Vd .. 2 Vd, query 4i
    far_q = far.reshape(-1, cap)[Vd:2 * Vd:4, 0].astype(bool)
    # a large budget excludes small triangles (every edge must be 4 budgets long)
    min_far = 1000 if budget_rel < 0.1 else 50
    assert far_q.sum() > min_far and (~far_q).sum() > 100
    checked = 0
    for mode in ("towards", "random"):
        y = y4.copy()
        for i in np.flatnonzero(far_q):
            pp, a, b, c = (y4[4 * i + k, :3].astype(np.float64) for k in range(4))
            if mode == "towards":
                cp = _closest_point(pp, a, b, c)
                dvec = cp - pp
                # just under the budget in the L1 norm the motion test uses
                dvec /= np.abs(dvec).sum() + 1e-300
                step = 0.999 * float(beta)
                moves = [dvec * step, -dvec * step, -dvec * step, -dvec * step]
            else:
                moves = [rng.normal(size=3) for _ in range(4)]
                moves = [m / (np.abs(m).sum() + 1e-300) * 0.999 * float(beta) * rng.uniform(0.5, 1) for m in moves]
            for k in range(4):
                y[4 * i + k, :3] = (y4[4 * i + k, :3].astype(np.float64) + moves[k]).astype(np.float32)
        skip = po.split_skip(faces, None, y, y4, None, cap, vt_st, vt_dy, tv_st, beta, far)
        skip_q = skip.reshape(-1, cap)[Vd:2 * Vd:4, 0].astype(bool)
        idx = np.flatnonzero(far_q & skip_q)
        assert len(idx) > 0.95 * far_q.sum()
        p12 = np.concatenate([y[4 * idx + k, :3] for k in range(4)], axis=1).astype(np.float32)
        dt, d, _ = po.point_triangles(p12)
        assert not np.any(d < dHat), (mode, idx[d < dHat][:5], d[d < dHat][:5])
        checked += len(idx)
    assert checked > 2 * min_far


def _solver_pair(pkg, po, scene, budget, frames):
    from starlab_physics_gb300 import mesh as M

    cl = M.TriMesh(scene.cloth_x, scene.cloth_faces, device="cpu")
    ob = M.TriMesh(scene.obstacle_x, scene.obstacle_faces, device="cpu")
    if len(scene.pinned):
        cl.fixed[scene.pinned] = 0.0
    runs = []
    for mb in (None, budget):
        orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), dt=scene.dt,
                              g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                              k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                              padding=scene.padding, n_iter=scene.n_iter, collisions=True, rebuild=scene.rebuild,
                              cap=scene.cap, bending_on="y", contact_cull=True, nthreads=4,
                              motion_budget=None if mb is None else mb * np.sqrt(scene.dHat * 1.0625))
        for _ in range(frames):
            orc.forward(scene.n_substeps)
        runs.append(orc)
    return runs


@pytest.mark.parametrize("budget", [0.05, 0.3])
def test_split_keeps_solver_result(pkg, po, budget):
    """Oracle runs with the split equal runs without it bit for bit: a cloth
    over a box (10 substeps x 6 iterations) and a cloth draped over a sphere
    with self contact; the split leaves out pairs in later iterations."""
    sc = pkg.scenes.plain64(n=20, seed=3)
    sc.n_iter = 6
    sc.cloth_x[:, 2] = (sc.cloth_x[:, 2] - np.float32(0.43)).astype(np.float32)  # start just above the box top
    a, b = _solver_pair(pkg, po, sc, budget, 4)
    assert np.array_equal(a.x4, b.x4) and np.array_equal(a.v4, b.v4)
    assert b.split_skipped > 0
    sc = pkg.scenes.drape256(n=28, sphere_subdiv=3)
    sc.n_iter = 5
    sc.n_substeps = 4
    a, b = _solver_pair(pkg, po, sc, budget, 5)
    assert np.array_equal(a.x4, b.x4) and np.array_equal(a.v4, b.v4)
    assert b.split_skipped > 0
