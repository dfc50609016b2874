"""Host-side mesh set-up: canonical topology, bending pairs, masses, adjacency
and the benchmark scene sizes (no GPU)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def M(pkg):
    from starlab_physics_gb300 import mesh

    return mesh


def bending_literal(fid_np):
    """Literal restatement of findTriNeighbors + getBendingPair
    (meshTaichiWrapper.py:152-225)."""
    num_f = fid_np.shape[0]
    table = np.zeros((num_f * 3, 3), dtype=int)
    for f in range(num_f):
        v1, v2, v3 = np.sort(fid_np[f])
        table[3 * f:3 * f + 3, :] = [[v1, v2, 3 * f], [v1, v3, 3 * f + 1], [v2, v3, 3 * f + 2]]
    table = table[np.lexsort((table[:, 1], table[:, 0]))]
    nb = np.full(num_f * 3, -1)
    ii = 0
    while ii < 3 * num_f - 1:
        e0, e1 = table[ii], table[ii + 1]
        if e0[0] == e1[0] and e0[1] == e1[1]:
            nb[e0[2]] = e1[2]
            nb[e1[2]] = e0[2]
            ii += 2
        else:
            ii += 1
    pairs = []
    for f in range(num_f):
        for i in range(3):
            ne = nb[3 * f + i]
            if ne >= 0:
                nb[ne] = -1
                v = np.sort(fid_np[f])
                g = int(np.floor(ne / 3.0 + 1e-4) + 1e-4)
                w = np.sort(fid_np[g])
                pairs.append((v[~np.isin(v, w)][0], w[~np.isin(w, v)][0]))
    return np.array(pairs, dtype=np.int32).reshape(-1, 2)


@pytest.mark.parametrize("gen", ["grid3", "grid9", "grid16", "ico2", "box"])
def test_bending_pairs_match_literal(M, gen):
    if gen.startswith("grid"):
        x, f = M.grid_cloth(int(gen[4:]))
    elif gen == "ico2":
        x, f = M.icosphere(2, 1.0)
    else:
        x, f = M.box_mesh(1.0)
    assert np.array_equal(M.bending_pairs(f), bending_literal(f))


def test_benchmark_scene_sizes(pkg, M):
    s0 = pkg.scenes.plain64()
    e = M.edges_from_faces(s0.cloth_faces)
    assert s0.cloth_x.shape == (4096, 3) and s0.cloth_faces.shape == (7938, 3)
    assert e.shape[0] == 12033 and M.bending_pairs(s0.cloth_faces).shape[0] == 11781
    assert s0.obstacle_faces.shape == (12, 3)
    assert np.abs(s0.cloth_x[:, 2] - 1.0).max() <= 1e-4 + 1e-7
    s1 = pkg.scenes.drape256()
    assert s1.cloth_x.shape == (65536, 3) and s1.cloth_faces.shape == (130050, 3)
    assert s1.obstacle_faces.shape == (20480, 3) and s1.obstacle_x.shape == (10242, 3)
    e1 = M.edges_from_faces(s1.cloth_faces)
    assert e1.shape[0] == 195585 and M.bending_pairs(s1.cloth_faces).shape[0] == 194565
    r = np.linalg.norm(s1.obstacle_x.astype(np.float64) - 0.5, axis=1)
    assert np.allclose(r, 0.3, atol=1e-6)


def test_masses_literal(M):
    x, f = M.grid_cloth(7)
    x = (x + np.random.default_rng(0).uniform(-1e-3, 1e-3, x.shape)).astype(np.float32)
    e = M.edges_from_faces(f)
    l0 = M.rest_lengths(x, e)
    m = np.zeros(x.shape[0], np.float32)
    for i, (a, b) in enumerate(e):           # initEdgeIndices, serial order
        m[a] += np.float32(0.5) * l0[i]
        m[b] += np.float32(0.5) * l0[i]
    assert np.array_equal(M.inverse_masses(x.shape[0], e, l0), np.float32(1) / m)


def test_adjacency(M):
    x, f = M.grid_cloth(8)
    e = M.edges_from_faces(f)
    l0 = M.rest_lengths(x, e)
    b = M.bending_pairs(f)
    bl0 = M.rest_lengths(x, b)
    ptr, adj = M.constraint_adjacency(64, e, l0, b, bl0)
    assert ptr[-1] == 2 * (e.shape[0] + b.shape[0])
    # each vertex: springs first, then bending pairs, each in ascending constraint order
    for v in range(64):
        ent = adj[ptr[v]:ptr[v + 1]]
        is_b = ent[:, 0] < 0
        assert not np.any(is_b[:-1] & ~is_b[1:])
        nbrs = ent[:, 0] & 0x7FFFFFFF
        rest = ent[:, 1].view(np.float32)
        for nb, r, bb in zip(nbrs, rest, is_b):
            pair = (min(v, nb), max(v, nb))
            if bb:
                k = [i for i, p in enumerate(b) if set(p) == {v, nb}]
                assert any(bl0[i] == r for i in k)
            else:
                i = np.flatnonzero((e[:, 0] == pair[0]) & (e[:, 1] == pair[1]))[0]
                assert l0[i] == r


def test_soup_generator(pkg):
    v, f, q = pkg.scenes.triangle_soup(4096, seed=1)
    assert v.shape == (3 * 4096, 3) and f.shape == (4096, 3) and q.shape == (4096, 3)
    tri = v[f].astype(np.float64)
    c = tri.mean(1)
    assert c.min() > -0.01 and c.max() < 1.01
    lens = np.linalg.norm(tri[:, 1] - tri[:, 0], axis=1)
    assert lens.min() >= 1e-3 * 0.999 and lens.max() <= 1e-2 * 1.001
