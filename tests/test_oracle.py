"""CPU oracle against known answers, brute force and literal restatements of the
reference loops (no GPU).  These pin the oracle before it is used to judge the
CUDA kernels."""
import numpy as np
import pytest


# ---------------------------------------------------------------------------
# Morton codes (lbvh_cell.py:87-102)
# ---------------------------------------------------------------------------
def interleave3(x, y, z):
    r = 0
    for i in range(10):
        r |= ((x >> i) & 1) << (3 * i)
        r |= ((y >> i) & 1) << (3 * i + 1)
        r |= ((z >> i) & 1) << (3 * i + 2)
    return r


def test_morton_known_answers(po):
    pts = np.array([[0, 0, 0], [1, 1, 1], [0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5], [0.25, 0.5, 0.75],
                    [0.999, 0.001, 0.5]], np.float32)
    got = po.morton3d(pts)
    q = np.clip(np.floor(pts.astype(np.float64) * 1024), 0, 1023).astype(int)
    exp = [interleave3(*map(int, r)) for r in q]
    assert list(got) == exp
    assert got[1] == 0x3FFFFFFF
    assert got[2] == 1 << 27 and got[3] == 1 << 28 and got[4] == 1 << 29


def test_cell_codes_structure(po):
    """The 32^3 cell-centre codes are (interleave(i,j,k) << 15) | 0x7000, all
    distinct, and the Karras tree over them is a perfect depth-15 tree."""
    bvh = po.CellBVH()
    ids = np.arange(32768)
    x0, y0, z0 = ids // 1024, (ids % 1024) // 32, ids % 32
    exp = np.array([(interleave3(int(a), int(b), int(c)) << 15) | 0x7000 for a, b, c in zip(x0, y0, z0)])
    assert np.array_equal(np.sort(exp), bvh.codes)
    assert np.array_equal(exp[bvh.ids], bvh.codes)
    assert len(np.unique(bvh.codes)) == 32768
    # perfect tree: every internal range has a power-of-two size and splits in half
    size = bvh.range_r - bvh.range_l + 1
    assert np.all((size & (size - 1)) == 0)
    assert bvh.range_l[0] == 0 and bvh.range_r[0] == 32767


# ---------------------------------------------------------------------------
# radix sort (lbvh_cell.py:525-562)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n,bits", [(0, 30), (1, 30), (1000, 30), (4097, 12), (20000, 32)])
def test_radix_sort_stable(po, n, bits):
    rng = np.random.default_rng(n + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    if n > 3:
        keys[: n // 2] = keys[n // 2: 2 * (n // 2)]
    k, v = po.radix_sort(keys, np.arange(n, dtype=np.int32), bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v, order) and np.array_equal(k, keys[order])


# ---------------------------------------------------------------------------
# Karras hierarchy (lbvh_cell.py:256-336, :384-430)
# ---------------------------------------------------------------------------
def karras_literal(codes):
    """Literal transcription of delta / find_split / determine_range /
    assign_internal_nodes_Karras12 (reference rule, no tie-break)."""
    n = len(codes)

    def clz(v):
        v &= 0xFFFFFFFF
        return 32 if v == 0 else 32 - v.bit_length()

    def delta(i, j):
        ret = -1
        if 0 <= j <= n - 1:
            x = codes[i] ^ codes[j]
            ret = 32 if x == 0 else clz(x)
        return ret

    def find_split(l, r):
        first, last = codes[l], codes[r]
        if first == last:
            return (l + r) // 2
        common = clz(first ^ last)
        split, step = l, r - l
        while step > 1:
            step = (step + 1) // 2
            ns = split + step
            if ns < r and clz(first ^ codes[ns]) > common:
                split = ns
        return split

    def determine_range(i):
        dl, dr = delta(i, i - 1), delta(i, i + 1)
        d, dmin = 1, dl
        if dr < dl:
            d, dmin = -1, dr
        lmax = 2
        while delta(i, i + lmax * d) > dmin:
            lmax <<= 2
        l, t = 0, lmax // 2
        while t > 0:
            dd = -1
            if 0 <= i + (l + t) * d < n:
                dd = delta(i, i + (l + t) * d)
            if dd > dmin:
                l += t
            t //= 2
        s, e = i, i + l * d
        if d == -1:
            s, e = i + l * d, i
        return s, e

    out = []
    for i in range(n - 1):
        s, e = determine_range(i)
        sp = find_split(s, e)
        left = sp + (n - 1 if sp == s else 0)
        right = sp + 1 + (n - 1 if sp + 1 == e else 0)
        out.append((left, right, s, e))
    return np.array(out, np.int64).reshape(-1, 4)


def test_karras_paper_example(po):
    """The 8-key example of Karras (2012), Fig. 4: keys 00001 00010 00100 00101
    10011 11000 11001 11110.  Internal nodes (leaves are offset by n-1 = 7):
    I0->(I3,I4), I1->(L0,L1), I2->(L2,L3), I3->(I1,I2), I4->(L4,I5),
    I5->(I6,L7), I6->(L5,L6)."""
    codes = np.array([0b00001, 0b00010, 0b00100, 0b00101, 0b10011, 0b11000, 0b11001, 0b11110], np.int32)
    ca, cb, rl, rr, par = po.karras(codes, 0)
    L = lambda j: j + 7  # noqa: E731
    exp = {0: (3, 4), 1: (L(0), L(1)), 2: (L(2), L(3)), 3: (1, 2), 4: (L(4), 5), 5: (6, L(7)), 6: (L(5), L(6))}
    for i, (a, b) in exp.items():
        assert (ca[i], cb[i]) == (a, b), i
    assert (rl[0], rr[0]) == (0, 7)
    assert par[0] == -1 and par[3] == 0 and par[L(7)] == 5
    lit = karras_literal([int(c) for c in codes])
    assert np.array_equal(np.stack([ca, cb, rl, rr], 1), lit)


def _check_tree(ca, cb, rl, rr, n):
    seen = np.zeros(n, int)
    stack = [0]
    while stack:
        i = stack.pop()
        if i >= n - 1:
            seen[i - (n - 1)] += 1
            continue
        for c in (ca[i], cb[i]):
            stack.append(c)
        lo_a = rl[ca[i]] if ca[i] < n - 1 else ca[i] - (n - 1)
        hi_b = rr[cb[i]] if cb[i] < n - 1 else cb[i] - (n - 1)
        assert lo_a == rl[i] and hi_b == rr[i]
    assert np.all(seen == 1)


@pytest.mark.parametrize("n,dups", [(2, False), (3, False), (257, False), (2000, True)])
def test_karras_random(po, n, dups):
    rng = np.random.default_rng(n)
    if dups:
        codes = np.sort(rng.integers(0, 512, n)).astype(np.int32)  # many repeated codes
    else:
        codes = np.sort(rng.choice(1 << 30, n, replace=False)).astype(np.int32)
    lit = karras_literal([int(c) for c in codes])
    ca, cb, rl, rr, par = po.karras(codes, 0)
    assert np.array_equal(np.stack([ca, cb, rl, rr], 1), lit)
    if not dups:
        _check_tree(ca, cb, rl, rr, n)
    ca, cb, rl, rr, par = po.karras(codes, 1)   # index tie-break: always a valid tree
    _check_tree(ca, cb, rl, rr, n)


# ---------------------------------------------------------------------------
# cell BVH build + traversal vs brute force
# ---------------------------------------------------------------------------
def _random_faces(rng, F, lo=0.0, hi=1.0, size=0.03):
    c = rng.uniform(lo, hi, (F, 3)).astype(np.float32)
    e = rng.uniform(0.001, size, (F, 3)).astype(np.float32)
    mn = np.zeros((F, 4), np.float32)
    mx = np.zeros((F, 4), np.float32)
    mn[:, :3] = c - e
    mx[:, :3] = c + e
    return mn, mx


def _subtree(bvh, i, n=32768):
    """Reference rules (compute_cell_node_aabbs, lbvh_cell.py:491-522)."""
    if i >= n - 1:
        return bvh.num_faces[i], bvh.nmin4[i, :3], bvh.nmax4[i, :3]
    nl, a0, b0 = _subtree(bvh, bvh.child_a[i], n)
    nr, a1, b1 = _subtree(bvh, bvh.child_b[i], n)
    if nl > 0 and nr > 0:
        return nl + nr, np.minimum(a0, a1), np.maximum(b0, b1)
    if nl > 0:
        return nl, a0, b0
    if nr > 0:
        return nr, a1, b1
    c = np.float32(0.25) * (((a0 + b0) + a1) + b1)
    return 0, c, c


def test_cell_bvh_build_and_traverse_bruteforce(po):
    rng = np.random.default_rng(7)
    F = 3000
    mn, mx = _random_faces(rng, F, 0.1, 0.9)
    box = np.array([0.0, 0.0, 0.0, 1.0, 1.0, 1.0], np.float32)
    bvh = po.CellBVH()
    bvh.build(mn, mx, box)
    assert bvh.prefix[-1] == F
    # stable counting sort: ascending face ids inside each cell
    counts = np.diff(np.concatenate([[0], bvh.prefix]))
    starts = bvh.prefix - counts
    for c in np.flatnonzero(counts)[:200]:
        seg = bvh.sorted_face_ids[starts[c]: bvh.prefix[c]]
        assert np.all(np.diff(seg) > 0)
    # refit against a recursive evaluation of the reference rules (sampled nodes)
    for i in [0, 1, 2, 100, 1000, 16383, 32766]:
        nf, a, b = _subtree(bvh, i)
        assert nf == bvh.num_faces[i]
        assert np.array_equal(a, bvh.nmin4[i, :3]) and np.array_equal(b, bvh.nmax4[i, :3])
    # traversal finds exactly the faces whose AABB overlaps the query box
    pts = rng.uniform(0.05, 0.95, (400, 4)).astype(np.float32)
    pad = 0.02
    qmn, qmx = po.query_boxes(pts, pad)
    cand, num, status = bvh.traverse(qmn, qmx, 4096)
    assert status == 0
    for q in range(pts.shape[0]):
        ov = np.flatnonzero(np.all(qmn[q, :3] <= mx[:, :3], 1) & np.all(qmx[q, :3] >= mn[:, :3], 1))
        assert np.array_equal(np.sort(cand[q, : num[q]]), ov)


def test_cell_traverse_skip_rule(po):
    """Queries whose centre maps past the last cell are skipped
    (lbvh_cell.py:665); negative cell coordinates are not."""
    rng = np.random.default_rng(3)
    mn, mx = _random_faces(rng, 20000, 0.0, 1.0)
    bvh = po.CellBVH()
    bvh.build(mn, mx, np.array([0, 0, 0, 1, 1, 1], np.float32))
    pts = np.array([[1.02, 0.5, 0.5, 0], [0.5, 0.5, 0.5, 0], [-0.01, 0.5, 0.5, 0]], np.float32)
    qmn, qmx = po.query_boxes(pts, 0.05)
    cand, num, status = bvh.traverse(qmn, qmx, 4096)
    brute = [np.count_nonzero(np.all(qmn[q, :3] <= mx[:, :3], 1) & np.all(qmx[q, :3] >= mn[:, :3], 1))
             for q in range(3)]
    assert brute[0] > 0 and num[0] == 0   # x cell 32 -> flat id > 32767 -> skipped
    assert num[1] == brute[1] > 0
    assert num[2] == brute[2] > 0         # x cell -0.32 truncates to 0 -> not skipped


def test_face_bvh_bruteforce(po):
    rng = np.random.default_rng(11)
    F = 4000
    mn, mx = _random_faces(rng, F, 0.0, 1.0, 0.01)
    box = np.array([0, 0, 0, 1, 1, 1], np.float32)
    b = po.FaceBVH(mn, mx, box, tie=1)
    order = np.argsort(b.codes_unsorted.view(np.uint32), kind="stable")
    assert np.array_equal(b.sorted_ids, order)
    _check_tree(b.child_a, b.child_b, b.range_l, b.range_r, F)
    pts = rng.uniform(0, 1, (300, 4)).astype(np.float32)
    qmn, qmx = po.query_boxes(pts, 0.02)
    cand, num, status = b.traverse(qmn, qmx, 1024)
    assert status == 0
    for q in range(pts.shape[0]):
        ov = np.flatnonzero(np.all(qmn[q, :3] <= mx[:, :3], 1) & np.all(qmx[q, :3] >= mn[:, :3], 1))
        assert np.array_equal(np.sort(cand[q, : num[q]]), ov)


# ---------------------------------------------------------------------------
# point-triangle classification and gradients (distance.py)
# ---------------------------------------------------------------------------
TRI = (np.array([0, 0, 0], np.float32), np.array([1, 0, 0], np.float32), np.array([0, 1, 0], np.float32))


@pytest.mark.parametrize("p,region", [((0.2, 0.2, 1.0), 6), ((-1, -1, 0.5), 0), ((2, -0.5, 0.3), 1),
                                      ((-0.5, 2, 0.1), 2), ((0.5, -1, 0.2), 3), ((1, 1, 0.3), 4),
                                      ((-1, 0.5, 0.0), 5)])
def test_point_triangle_regions(po, p, region):
    dt, d, g = po.point_triangle(np.array(p, np.float32), *TRI)
    assert dt == region
    p64 = np.array(p, np.float64)
    t = [np.asarray(v, np.float64) for v in TRI]
    exact = _sqdist64(region, p64, *t)
    assert abs(d - exact) <= 1e-6 * max(1.0, exact)


def _sqdist64(region, p, t0, t1, t2):
    pp = lambda a, b: float(np.dot(a - b, a - b))  # noqa: E731

    def pe(x, a, b):
        c = np.cross(a - x, b - x)
        e = b - a
        return float(np.dot(c, c) / np.dot(e, e))

    def pt(x, a, b, c):
        n = np.cross(b - a, c - a)
        s = np.dot(x - a, n)
        return float(s * s / np.dot(n, n))

    return [lambda: pp(p, t0), lambda: pp(p, t1), lambda: pp(p, t2), lambda: pe(p, t0, t1),
            lambda: pe(p, t1, t2), lambda: pe(p, t0, t2), lambda: pt(p, t0, t1, t2)][region]()


def test_distance_gradients_finite_difference(po):
    rng = np.random.default_rng(5)
    checked = set()
    for _ in range(400):
        pts = rng.normal(0, 1, (4, 3)).astype(np.float32)
        dt, d, g = po.point_triangle(*pts)
        x = pts.astype(np.float64)
        fd = np.zeros((4, 3))
        h = 1e-6
        for k in range(4):
            for c in range(3):
                xp, xm = x.copy(), x.copy()
                xp[k, c] += h
                xm[k, c] -= h
                fd[k, c] = (_sqdist64(dt, xp[0], xp[1], xp[2], xp[3]) - _sqdist64(dt, xm[0], xm[1], xm[2], xm[3])) / (2 * h)
        scale = max(1.0, np.abs(fd).max())
        assert np.abs(g - fd).max() <= 2e-3 * scale, (dt, g, fd)
        checked.add(dt)
    assert checked == set(range(7))


# ---------------------------------------------------------------------------
# Jacobi sweep vs a literal restatement of XPBD.py:141-184 + :384-387
# ---------------------------------------------------------------------------
def jacobi_literal(x4, y4, fixed, m_inv, edges, l0, bend, bl0, ks, kb):
    f32 = np.float32
    V = x4.shape[0]
    dx = np.zeros((V, 3), f32)
    nc = np.zeros(V, f32)
    E = edges.shape[0]
    ks, kb = f32(ks), f32(kb)
    for i in range(E + bend.shape[0]):
        if i < E:
            v0, v1 = edges[i]
            rest, k, P = l0[i], ks, y4
        else:
            v0, v1 = bend[i - E]
            rest, k, P = bl0[i - E], kb, x4
        x10 = (P[v0, :3] - P[v1, :3]).astype(f32)
        lij = np.sqrt(f32((x10[0] * x10[0] + x10[1] * x10[1]) + x10[2] * x10[2]))
        C = f32(lij - rest)
        n = (f32(f32(1) / lij) * x10).astype(f32)
        schur = f32(f32(fixed[v0] * m_inv[v0] + fixed[v1] * m_inv[v1]) * f32((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]))
        ld = f32(f32(k * C) / f32(k * schur + f32(1)))
        dx[v0] = dx[v0] - f32(fixed[v0] * m_inv[v0] * ld) * n
        dx[v1] = dx[v1] + f32(fixed[v1] * m_inv[v1] * ld) * n
        nc[v0] += 1
        nc[v1] += 1
    y = y4.copy()
    for v in range(V):
        if nc[v] > 0:
            y[v, :3] = y[v, :3] + fixed[v] * (dx[v] / nc[v])
    return y


def test_jacobi_sweep_literal(pkg, po):
    from starlab_physics_gb300 import mesh as M

    x, f = M.grid_cloth(6)
    rng = np.random.default_rng(1)
    x = (x + rng.uniform(-0.01, 0.01, x.shape)).astype(np.float32)
    e = M.edges_from_faces(f)
    l0 = M.rest_lengths(x, e)
    bend = M.bending_pairs(f)
    bl0 = M.rest_lengths(x, bend)
    m_inv = M.inverse_masses(36, e, l0)
    fixed = np.ones(36, np.float32)
    fixed[[30, 35]] = 0
    x4 = np.zeros((36, 4), np.float32)
    x4[:, :3] = x
    y4 = x4.copy()
    y4[:, :3] += rng.normal(0, 0.02, (36, 3)).astype(np.float32)
    ks, kb = 1e8 / 3600.0, 1e5 / 3600.0
    lit = jacobi_literal(x4, y4, fixed, m_inv, e, l0, bend, bl0, ks, kb)
    yo = y4.copy()
    po.spring_sweep(x4, yo, fixed, m_inv, e, l0, bend, bl0, ks, kb)
    assert np.array_equal(lit[:, :3], yo[:, :3])
    # the parallel (atomic) oracle used for timing agrees to float rounding
    yp = y4.copy()
    po.spring_sweep(x4, yp, fixed, m_inv, e, l0, bend, bl0, ks, kb, nthreads=4)
    assert np.allclose(yp, yo, atol=1e-6)


@pytest.mark.parametrize("bend_on_y", [0, 1])
def test_gather_sweep_equals_serial_scatter(pkg, po, bend_on_y):
    """The oracle's per-vertex gather sweep (its multithreaded form for parity
    runs) equals the serial scatter bit for bit at any thread count."""
    from starlab_physics_gb300 import mesh as M

    x, f = M.grid_cloth(40)
    rng = np.random.default_rng(4)
    x = (x + rng.uniform(-0.003, 0.003, x.shape)).astype(np.float32)
    V = x.shape[0]
    e = M.edges_from_faces(f)
    l0 = M.rest_lengths(x, e)
    bend = M.bending_pairs(f)
    bl0 = M.rest_lengths(x, bend)
    m_inv = M.inverse_masses(V, e, l0)
    fixed = np.ones(V, np.float32)
    fixed[[V - 40, V - 1]] = 0
    x4 = np.zeros((V, 4), np.float32)
    x4[:, :3] = x
    y4 = x4.copy()
    y4[:, :3] += rng.normal(0, 0.004, (V, 3)).astype(np.float32)
    ks, kb = 1e8 / 3.6e5, 1e5 / 3.6e5
    ys = y4.copy()
    po.spring_sweep(x4, ys, fixed, m_inv, e, l0, bend, bl0, ks, kb, bend_on_y=bend_on_y)
    ptr, adj = po.adjacency(V, e, l0, bend, bl0)
    for nt in (1, 4):
        yg = y4.copy()
        po.spring_sweep_gather(x4, yg, fixed, m_inv, ptr, adj, ks, kb, nthreads=nt, bend_on_y=bend_on_y)
        assert np.array_equal(yg, ys), nt


def test_collision_parallel_matches_serial(pkg, po):
    """Fixed-point contact accumulation makes the parallel oracle equal the serial one."""
    sc = pkg.scenes.drape256(n=24, sphere_subdiv=2)
    from starlab_physics_gb300 import mesh as M

    cl = M.TriMesh(sc.cloth_x, sc.cloth_faces, device="cpu")
    sp = M.TriMesh(sc.obstacle_x, sc.obstacle_faces, device="cpu")
    y4 = np.zeros((cl.num_verts, 4), np.float32)
    y4[:, :3] = cl.x0_np
    y4[:, 2] = 0.8 + 0.02 * np.sin(9 * y4[:, 0])
    xs4 = np.zeros((sp.num_verts, 4), np.float32)
    xs4[:, :3] = sp.x0_np
    pad, cap, dHat = 0.05, 40, np.float32(0.03 ** 2)
    bd, bs = po.CellBVH(), po.CellBVH()
    mn, mx = po.face_aabbs(y4, cl.fid_np, pad)
    bd.build(mn, mx, po.scene_aabb(y4, pad))
    mn2, mx2 = po.face_aabbs(xs4, sp.fid_np, pad)
    bs.build(mn2, mx2, po.scene_aabb(xs4, pad))
    q1 = po.query_boxes(y4, pad)
    q2 = po.query_boxes(xs4, pad)
    vt_st = bs.traverse(*q1, cap)[:2]
    vt_dy = bd.traverse(*q1, cap)[:2]
    tv_st = bd.traverse(*q2, cap)[:2]
    ys, yp = y4.copy(), y4.copy()
    fixed = np.ones(cl.num_verts, np.float32)
    r1 = po.collision_sweep(cl.fid_np, sp.fid_np, ys, xs4, fixed, cl.m_inv_np, dHat, np.float32(1e8), cap, vt_st,
                            vt_dy, tv_st, want_pairs=True)
    po.collision_sweep(cl.fid_np, sp.fid_np, yp, xs4, fixed, cl.m_inv_np, dHat, np.float32(1e8), cap, vt_st, vt_dy,
                       tv_st, nthreads=4)
    assert (r1["pair_num"] > 0).sum() > 10
    assert np.array_equal(ys, yp)
    assert not np.array_equal(ys, y4)


def _box_d2_np(p, t):
    """Point-to-triangle-box squared distance, float32, the kernels' order."""
    lo = np.minimum(np.minimum(t[:, 0], t[:, 1]), t[:, 2])
    hi = np.maximum(np.maximum(t[:, 0], t[:, 1]), t[:, 2])
    e = np.maximum(np.maximum(lo - p, p - hi), np.float32(0))
    return (e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]) + e[:, 2] * e[:, 2]


def test_contact_cull_never_drops_a_contact(po):
    """Every region's squared distance is at least the box distance: over random
    point-triangle pairs placed around the contact threshold, no pair the cull
    removes (box distance > 1.0625 dHat) has d < dHat."""
    rng = np.random.default_rng(11)
    dHat = np.float32(2e-3) ** 2
    n, culled = 20000, 0
    tri = rng.uniform(-1, 1, (n, 3, 3)).astype(np.float32) * np.float32(4e-3) + np.float32(0.7)
    p = (tri.mean(axis=1) + rng.normal(0, 5e-3, (n, 3))).astype(np.float32)
    bd = _box_d2_np(p, tri)
    for i in range(n):
        dt, d, _ = po.point_triangle(p[i], tri[i, 0], tri[i, 1], tri[i, 2])
        if bd[i] > dHat * np.float32(1.0625):
            culled += 1
            assert not d < dHat, (i, dt, d, bd[i])
    assert culled > n // 10


def test_separating_axis_cull_never_drops_a_contact(po):
    """The second cull stage (separating axes: face normal and in-plane edge
    normals) on adversarial pairs: flat and bent sheets whose vertices sit
    beside the neighbouring triangles (box distance 0), slivers, tiny and
    large triangles, points placed at 0.8-1.3 x the contact distance from
    points of the triangle in random and in-plane directions.  No pair with
    d < dHat is culled, and the stage removes most of the box survivors of
    the sheets.  Triangles too small or too thin for the region classifier's
    float32 solves (where it can return the plane region for a far point) are
    not culled at all."""
    rng = np.random.default_rng(5)
    dHat = np.float32(2e-3) ** 2
    cull = dHat * np.float32(1.0625)
    r = np.sqrt(np.float64(dHat))
    quads = []
    # sheets: grid spacing 1.2-3 r, jittered, flat or bent; every vertex against
    # the triangles of its 5 x 5 neighbourhood that do not contain it
    for h_over_r, bend in ((1.2, 0.0), (1.45, 0.0), (2.0, 0.3), (3.0, 1.0), (1.3, 2.0)):
        n = 9
        h = h_over_r * r
        u, v = np.meshgrid(np.arange(n) * h, np.arange(n) * h, indexing="ij")
        z = bend * h * np.sin(u / (3 * h)) * np.cos(v / (2 * h))
        X = np.stack([u, v, z], -1).reshape(-1, 3) + rng.normal(0, 0.05 * h, (n * n, 3))
        X = (X + 0.5).astype(np.float32)
        F = []
        for i in range(n - 1):
            for j in range(n - 1):
                a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
                F += [(a, b, c), (a, c, d)] if (i + j) % 2 else [(a, b, d), (b, c, d)]
        F = np.array(F)
        for q in range(n * n):
            for f in F:
                if q in f or np.abs(X[f].mean(0) - X[q]).max() > 3 * h:
                    continue
                quads.append(np.concatenate([X[q], X[f[0]], X[f[1]], X[f[2]]]))
    n_sheet = len(quads)
    # random triangles, slivers among them, points near the threshold
    for _ in range(12000):
        size = 10 ** rng.uniform(-4, -1)
        T = rng.normal(0, size, (3, 3))
        if rng.random() < 0.3:  # sliver: the third vertex near the opposite edge
            w = rng.random()
            T[2] = w * T[0] + (1 - w) * T[1] + rng.normal(0, size * 1e-3, 3)
        bary = rng.dirichlet((1, 1, 1)) if rng.random() < 0.5 else np.eye(3)[rng.integers(3)]
        q = bary @ T
        nrm = np.cross(T[1] - T[0], T[2] - T[0])
        if rng.random() < 0.5 and np.linalg.norm(nrm) > 0:
            dirn = np.cross(nrm, rng.normal(size=3))  # in the plane
        else:
            dirn = rng.normal(size=3)
        dirn /= np.linalg.norm(dirn)
        p = q + dirn * r * rng.uniform(0.8, 1.3)
        off = rng.uniform(-2, 2, 3)
        quads.append(np.concatenate([p + off, *(T + off)]).astype(np.float32))
    Q = np.array(quads, np.float32)
    dt, d, _ = po.point_triangles(Q)
    out = po.contact_cull(Q, cull)
    assert not ((out != 0) & (d < dHat)).any()
    assert (d < dHat).sum() > 500
    sheet = out[:n_sheet]
    assert (sheet == 2).sum() > 0.8 * (sheet != 1).sum() - (d[:n_sheet] < dHat).sum()
    assert (out[n_sheet:] == 2).sum() > 500
    # tiny slivers whose classification is arbitrary are never culled, though
    # their box distance exceeds the threshold
    tiny = _box_d2_np(Q[:, :3], Q[:, 3:].reshape(-1, 3, 3)) > cull
    assert ((out == 0) & tiny & (d < dHat)).sum() > 10


def test_contact_cull_keeps_solver_result(pkg, po):
    """The oracle solver gives bit-identical trajectories with and without the
    cull on a colliding scene (plain64, 24x24, with iterations)."""
    scene = pkg.scenes.plain64(n=24, seed=2)
    scene.n_iter = 4
    from starlab_physics_gb300 import mesh as M

    cl = M.TriMesh(scene.cloth_x, scene.cloth_faces, device="cpu")
    ob = M.TriMesh(scene.obstacle_x, scene.obstacle_faces, device="cpu")
    runs = []
    for cull in (False, True):
        orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), dt=scene.dt,
                              g=scene.gravity, k_stretch_stiffness=scene.stiffness_stretch,
                              k_bend_stiffness=scene.stiffness_bending, dHat=scene.dHat, damping=scene.damping,
                              padding=scene.padding, n_iter=scene.n_iter, collisions=True, rebuild=scene.rebuild,
                              cap=scene.cap, bending_on="y", contact_cull=cull)
        for _ in range(8):
            orc.forward(scene.n_substeps)
        runs.append(orc.x4.copy())
    assert np.array_equal(runs[0], runs[1])
    assert np.abs(runs[0][:, 2] - cl.x0_np[:, 2]).max() > 0.01


# ---------------------------------------------------------------------------
# graph colouring (graph_coloring.py:112-201)
# ---------------------------------------------------------------------------
def greedy_literal(E_arr, max_colors=100):
    E = len(E_arr)
    adj = np.zeros((E, E), np.int32)
    for i in range(E):
        for j in range(E):
            if i != j and len({*E_arr[i]} & {*E_arr[j]}) > 0:
                adj[i, j] = 1
    color = np.full(E, -1)
    for i in range(E):
        avail = np.ones(max_colors, np.int32)
        for j in range(E):
            if adj[i, j] == 1 and color[j] != -1:
                avail[color[j]] = 0
        color[i] = np.argmax(avail)
    prefix = np.zeros(max_colors, np.int32)
    for c in color:
        prefix[c] += 1
    for i in range(1, max_colors):
        prefix[i] += prefix[i - 1]
    sorted_idx = np.zeros(E, np.int32)
    for i in range(E - 1, -1, -1):
        prefix[color[i]] -= 1
        sorted_idx[prefix[color[i]]] = i
    return color, sorted_idx, prefix


def test_coloring_literal_9x9(pkg, po):
    from starlab_physics_gb300 import mesh as M

    x, f = M.grid_cloth(9)
    e = M.edges_from_faces(f)
    assert e.shape[0] == 208   # same edge count as the reference's precomputed 9x9 fixture
    c, s, p = po.color_edges(81, e)
    lc, ls, lp = greedy_literal([tuple(r) for r in e])
    assert np.array_equal(c, lc) and np.array_equal(s, ls) and np.array_equal(p, lp)
    # format of the reference fixture: start offsets, E for unused colours
    k = c.max() + 1
    assert np.all(p[k:] == 208) and p[0] == 0
    for a, b in [(i, j) for i in range(208) for j in range(i + 1, 208) if set(e[i]) & set(e[j])]:
        assert c[a] != c[b]


def test_coloring_icosphere(po):
    from starlab_physics_gb300 import mesh as M

    x, f = M.icosphere(1, 1.0)
    e = M.edges_from_faces(f)
    c, s, p = po.color_edges(x.shape[0], e)
    lc, ls, lp = greedy_literal([tuple(r) for r in e])
    assert np.array_equal(c, lc) and np.array_equal(s, ls) and np.array_equal(p, lp)
