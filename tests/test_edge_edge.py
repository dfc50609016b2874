"""Edge-edge contacts on the CPU: the oracle's classifier against a literal
restatement of d_type_EE (distance.py:50-99), its gradient against finite
differences, the face-edge table, and the sweep's rules on crafted crossings
(no GPU)."""
import numpy as np
import pytest

f32 = np.float32


def _sub(a, b):
    return [f32(a[i] - b[i]) for i in range(3)]


def _dot(a, b):
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def _cross(a, b):
    return [f32(f32(a[1] * b[2]) - f32(a[2] * b[1])), f32(f32(a[2] * b[0]) - f32(a[0] * b[2])),
            f32(f32(a[0] * b[1]) - f32(a[1] * b[0]))]


def d_type_ee_literal(v0, v1, v2, v3):
    """distance.py:50-99 line by line, in float32."""
    u, v, w = _sub(v1, v0), _sub(v3, v2), _sub(v0, v2)
    a, b, c, d, e = _dot(u, u), _dot(u, v), _dot(v, v), _dot(u, w), _dot(v, w)
    D = f32(f32(a * c) - f32(b * b))
    tD = D
    tN = f32(0.0)
    default_case = 8
    sN = f32(f32(b * e) - f32(c * d))
    if sN <= 0.0:
        tN, tD, default_case = e, c, 2
    elif sN >= D:
        tN, tD, default_case = f32(e + b), c, 5
    else:
        tN = f32(f32(a * e) - f32(b * d))
        uv = _cross(u, v)
        if tN > 0.0 and tN < tD and (_dot(uv, w) < f32(1e-4) or _dot(uv, uv) < f32(f32(f32(1.0e-20) * a) * c)):
            if sN < f32(D / f32(2.0)):
                tN, tD, default_case = e, c, 2
            else:
                tN, tD, default_case = f32(e + b), c, 5
    if tN <= 0.0:
        if -d <= 0.0:
            default_case = 0
        elif -d >= a:
            default_case = 3
        else:
            default_case = 6
    elif tN >= tD:
        if f32(-d + b) <= 0.0:
            default_case = 1
        elif f32(-d + b) >= a:
            default_case = 4
        else:
            default_case = 7
    return default_case


def test_d_type_ee_literal(po):
    rng = np.random.default_rng(11)
    seen = set()
    for scale in (0.01, 0.1, 1.0):
        p = (rng.normal(size=(1500, 12)) * scale).astype(np.float32)
        dt, d, g = po.edge_edge_classify(p, 1e-2)
        for i in range(p.shape[0]):
            q = p[i].reshape(4, 3)
            assert dt[i] == d_type_ee_literal(q[0], q[1], q[2], q[3]), (scale, i)
        seen |= set(dt.tolist())
    assert seen == set(range(9))


def _d_ee64(x0, x1, x2, x3):
    n = np.cross(x1 - x0, x3 - x2)
    s = np.dot(x2 - x0, n)
    return s * s / np.dot(n, n)


def test_edge_edge_gradient_finite_difference(po):
    """The closed-form gradient of the squared line-line distance (float32 in
    the oracle) against central differences of the float64 distance."""
    rng = np.random.default_rng(3)
    checked = 0
    while checked < 20:
        p = rng.normal(size=(1, 12)).astype(np.float32) * 0.3
        dt, d, g = po.edge_edge_classify(p, 10.0)
        if dt[0] != 8 or d[0] >= 10.0:
            continue
        X = p.reshape(4, 3).astype(np.float64)
        assert abs(d[0] - _d_ee64(*X)) <= 1e-4 * max(1e-6, _d_ee64(*X)) + 1e-7
        h = 1e-6
        for k in range(4):
            fd = np.zeros(3)
            for c in range(3):
                Xp, Xm = X.copy(), X.copy()
                Xp[k, c] += h
                Xm[k, c] -= h
                fd[c] = (_d_ee64(*Xp) - _d_ee64(*Xm)) / (2 * h)
            np.testing.assert_allclose(g[0, k], fd, rtol=2e-3, atol=2e-5 * max(1.0, np.abs(fd).max()))
        np.testing.assert_allclose(g[0].sum(axis=0), 0.0, atol=1e-5 * np.abs(g[0]).max())
        checked += 1


def test_edge_edge_projection_rules(pkg, po):
    """Edge-edge terms are gated by dtype 8 and |x01 x x23| > 1e-3; ee_dy skips
    edges that share a vertex; ee_st moves only the cloth edge; each term adds
    one count to every vertex it moves."""
    # cloth: two triangles, (0,1,2) and (3,4,5); edge (0,1) along x at z = 0,
    # edge (3,4) along y at z = 0.01 crossing it in the middle
    y4 = np.zeros((6, 4), np.float32)
    y4[:, :3] = [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, -1.0, 0.0],
                 [0.5, -0.5, 0.01], [0.5, 0.5, 0.01], [1.5, 0.0, 0.01]]
    faces = np.array([[0, 1, 2], [3, 4, 5]], np.int32)
    edges_from_faces, face_edges = pkg.mesh.edges_from_faces, pkg.mesh.face_edges
    edges = edges_from_faces(faces)
    fe = face_edges(faces, edges)
    for f in range(2):
        for k in range(3):
            a, b = faces[f, k], faces[f, (k + 1) % 3]
            assert sorted(edges[fe[f, k]]) == sorted([a, b])
    E = edges.shape[0]
    cap = 4
    # every edge sees both faces
    cand = np.tile(np.array([[0, 1, 0, 0]], np.int32), (E, 1))
    num = np.full(E, 2, np.int32)
    fixed = np.ones(6, np.float32)
    m_inv = np.ones(6, np.float32)
    e01 = int(np.nonzero((edges == [0, 1]).all(1))[0][0])
    e34 = int(np.nonzero((edges == [3, 4]).all(1))[0][0])
    for sign in (1.0, -1.0):
        # the interior case needs a triple product above 1e-4: the sign of the
        # offset decides whether crossing pairs project
        y = y4.copy()
        y[3:, 2] = sign * 0.01
        dx = np.zeros(18, np.int64)
        nc = np.zeros(6, np.int32)
        r = po.edge_edge_sweep(edges, None, fe, None, y, None, fixed, m_inv, 4e-4, 1e8, cap, None, (cand, num), dx,
                               nc, want_pairs=True)
        # brute force: every edge against the three edges of both faces, in
        # order, vertex-sharing pairs skipped
        exp_nc = np.zeros(6, np.int32)
        for e in range(E):
            want = []
            for f in (0, 1):
                for k in range(3):
                    e2 = fe[f, k]
                    if set(edges[e]) & set(edges[e2]):
                        continue
                    q = y[[*edges[e], *edges[e2]], :3].ravel()[None]
                    dt, d, _ = po.edge_edge_classify(q, 4e-4)
                    if d[0] < 4e-4:
                        assert dt[0] == 8
                        want.append(e2)
                        exp_nc[[*edges[e], *edges[e2]]] += 1
            got = r["pair"][E + e, : r["pair_num"][E + e], 0].tolist()
            assert got == want, (sign, e)
        assert np.array_equal(nc, exp_nc)
        if sign < 0:
            assert e34 in r["pair"][E + e01, : r["pair_num"][E + e01], 0]
            # pushed apart along z: edge (0,1) up, away from the other below
            assert dx[3 * 0 + 2] > 0 and dx[3 * 3 + 2] < 0
        else:
            assert r["pair_num"].sum() == 0
    # ee_st: the crossings against a static copy of the second triangle (below
    # the cloth) move the cloth edge only
    xs4 = y4[3:].copy()
    xs4[:, 2] = -0.01
    st_faces = np.array([[0, 1, 2]], np.int32)
    st_edges = edges_from_faces(st_faces)
    st_fe = face_edges(st_faces, st_edges)
    dx = np.zeros(18, np.int64)
    nc = np.zeros(6, np.int32)
    st_cand = np.zeros((E, cap), np.int32)
    st_num = np.ones(E, np.int32)
    r = po.edge_edge_sweep(edges, st_edges, fe, st_fe, y4, xs4, fixed, m_inv, 4e-4, 1e8, cap, (st_cand, st_num),
                           (cand, np.zeros(E, np.int32)), dx, nc, want_pairs=True)
    exp_nc = np.zeros(6, np.int32)
    for e in range(E):
        want = []
        for k in range(3):
            e2 = st_fe[0, k]
            q = np.concatenate([y4[edges[e], :3].ravel(), xs4[st_edges[e2], :3].ravel()])[None]
            dt, d, _ = po.edge_edge_classify(q, 4e-4)
            if d[0] < 4e-4:
                want.append(e2)
                exp_nc[edges[e]] += 1
        assert r["pair"][e, : r["pair_num"][e], 0].tolist() == want
    assert r["pair_num"][:E].sum() >= 1 and r["pair_num"][E:].sum() == 0
    assert np.array_equal(nc, exp_nc)


def test_edge_edge_changes_the_oracle_solver(pkg, po):
    """On the crossed-layers scene the edge-edge terms change the motion."""
    sc = pkg.scenes.crossed_layers()
    TriMesh = pkg.TriMesh
    cl = TriMesh(sc.cloth_x, sc.cloth_faces, device="cpu")
    bo = TriMesh(sc.obstacle_x, sc.obstacle_faces, device="cpu", is_static=True)
    outs = []
    for ee in (False, True):
        o = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(bo), dt=sc.dt, g=sc.gravity,
                            k_stretch_stiffness=sc.stiffness_stretch, k_bend_stiffness=sc.stiffness_bending,
                            dHat=sc.dHat, padding=sc.padding, n_iter=sc.n_iter, collisions=True, rebuild=sc.rebuild,
                            cap=sc.cap, bending_on="y", contact_cull=True, edge_edge=ee)
        for _ in range(4):
            o.forward(sc.n_substeps)
        outs.append(o.x4.copy())
    assert np.isfinite(outs[1]).all()
    assert not np.array_equal(outs[0], outs[1])
