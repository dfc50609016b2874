"""The Jacobi sweep over the packed adjacency (int16 neighbour offsets and
rest-length bits with the bending flag, staged per block in shared memory):
the packing round-trips on the CPU, and on the GPU the packed sweep equals the
int2 sweep bit for bit (exact and fast arithmetic) on a drape, on the
concatenated 512-cloth batch and on a graph with a hub vertex whose block
exceeds the shared-memory capacity (read from global memory instead)."""
import numpy as np
import pytest
import torch


def _random_graph(V, seed, hub=None, span=3000):
    from starlab_physics_gb300.mesh import constraint_adjacency

    rng = np.random.default_rng(seed)
    a = rng.integers(0, V, 6 * V)
    b = np.clip(a + rng.integers(-span, span + 1, 6 * V), 0, V - 1)
    keep = a != b
    pairs = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)[keep]
    if hub is not None:
        others = np.arange(max(hub - span, 0), min(hub + span, V))
        others = others[others != hub]
        pairs = np.concatenate([pairs, np.stack([np.full_like(others, hub), others], 1)])
    pairs = np.unique(pairs, axis=0).astype(np.int32)
    half = pairs.shape[0] // 2
    edges, bend = pairs[:half], pairs[half:]
    l0 = rng.uniform(0.005, 0.02, edges.shape[0]).astype(np.float32)
    bl0 = rng.uniform(0.01, 0.04, bend.shape[0]).astype(np.float32)
    return constraint_adjacency(V, edges, l0, bend, bl0)


def test_packed_adjacency_round_trip(pkg):
    from starlab_physics_gb300.mesh import packed_adjacency

    ptr, adj = _random_graph(5000, 0, hub=2500, span=2000)
    nbr16, rest32 = packed_adjacency(ptr, adj)
    n = adj.shape[0]
    assert nbr16.shape[0] % 8 == 0 and nbr16.shape[0] >= ((n + 7) & ~7) and rest32.shape[0] == nbr16.shape[0]
    owner = np.repeat(np.arange(5000), np.diff(ptr))
    r = rest32[:n].view(np.uint32)
    word = ((owner + nbr16[:n].astype(np.int64)).astype(np.uint32) | (r & np.uint32(0x80000000))).view(np.int32)
    assert np.array_equal(word, adj[:, 0])
    assert np.array_equal((r & np.uint32(0x7FFFFFFF)).view(np.int32), adj[:, 1])
    assert not nbr16[n:].any() and not rest32[n:].any()
    # offsets beyond 16 bits: no packed form
    ptr2, adj2 = _random_graph(70000, 1, span=40000)
    assert packed_adjacency(ptr2, adj2) is None


def _both(L, x4, y4, fixed, ptr, adj, nbr16, rest32, V, fast, bend_y=1):
    from starlab_physics_gb300._lib import ptr as P, stream_handle

    o1, o2, o3 = torch.empty_like(y4), torch.empty_like(y4), torch.empty_like(y4)
    ks, kb = 1e8 / 3.6e5, 1e5 / 3.6e5
    assert L.sx_jacobi_sweep_mode(P(x4), P(y4), P(o1), P(fixed), P(ptr), P(adj), V, ks, kb, bend_y, 0, fast,
                                  stream_handle()) == 0
    assert L.sx_jacobi_sweep_packed(P(x4), P(y4), P(o2), P(fixed), P(ptr), P(nbr16), P(rest32), V, ks, kb, bend_y,
                                    fast, stream_handle()) == 0
    # every direct form (entries read from global memory) gives the same sums
    for form in range(1, int(L.sx_jacobi_sweep_packed_forms())):
        o3.fill_(float("nan"))
        assert L.sx_jacobi_sweep_packed_v(P(x4), P(y4), P(o3), P(fixed), P(ptr), P(nbr16), P(rest32), V, ks, kb,
                                          bend_y, form, fast, stream_handle()) == 0
        torch.cuda.synchronize()
        assert torch.equal(o2, o3), form
    return o1, o2


@pytest.mark.gpu
@pytest.mark.parametrize("fast", [0, 1])
def test_packed_sweep_equals_int2_sweep(pkg, fast):
    from starlab_physics_gb300 import _lib
    from starlab_physics_gb300.mesh import packed_adjacency

    L = _lib.load()
    # the drape's cloth (bending on y and on x)
    scene = pkg.scenes.drape256()
    sim = pkg.scenes.make_solver(scene, device="cuda")
    m = sim.mesh_dy
    y = m.x4.clone()
    y[:, :3] += 1e-3 * torch.randn_like(y[:, :3])
    for bend_y in (1, 0):
        o1, o2 = _both(L, m.x4, y, m.fixed, m.adj_ptr, m.adj, m.adj_nbr16, m.adj_rest32, m.num_verts, fast, bend_y)
        assert torch.equal(o1, o2)
    # the concatenated 512-cloth batch
    bs = pkg.BatchedSolver(pkg.batched_scene(512, seed=0), dHat=(4e-3) ** 2, stiffness_stretch=1e5,
                           stiffness_bending=1e8, g=(0.0, 0.0, -9.81), dt=1 / 60, n_iter=20, padding=8e-3)
    y = bs.x4.clone()
    y[:, :3] += 1e-3 * torch.randn_like(y[:, :3])
    o1, o2 = _both(L, bs.x4, y, bs.fixed, bs.adj_ptr, bs.adj, bs.adj_nbr16, bs.adj_rest32, bs.num_verts, fast)
    assert torch.equal(o1, o2)
    # a hub vertex with 6000 entries: its block reads from global memory
    V = 20000
    ptr, adj = _random_graph(V, 2, hub=10000)
    nbr16, rest32 = packed_adjacency(ptr, adj)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    x4 = torch.zeros((V, 4), device="cuda")
    x4[:, :3] = torch.rand((V, 3), device="cuda")
    x4[:, 3] = 1.0
    y = x4.clone()
    y[:, :3] += 1e-3 * torch.randn_like(y[:, :3])
    fixed = torch.ones(V, device="cuda")
    o1, o2 = _both(L, x4, y, fixed, t(ptr), t(adj), t(nbr16), t(rest32), V, fast)
    assert int(np.diff(ptr)[10000]) >= 6000
    assert torch.equal(o1, o2) and torch.isfinite(o1).all()


@pytest.mark.gpu
def test_packed_sweep_in_solver_frames(pkg):
    """Batched frames with the packed sweep (grid-wide launches, and the
    persistent substep reading the packed arrays) equal the frames with the
    int2 sweep."""
    bs = pkg.BatchedSolver(pkg.batched_scene(64, seed=3), dHat=(4e-3) ** 2, stiffness_stretch=1e5,
                           stiffness_bending=1e8, g=(0.0, 0.0, -9.81), dt=1 / 60, n_iter=20, padding=8e-3)
    bs.use_graph = True
    x0, v0 = bs.x4.clone(), bs.v4.clone()
    out = []
    for persistent, packed in ((False, False), (False, True), (True, True)):
        bs.x4.copy_(x0)
        bs.v4.copy_(v0)
        bs.persistent = persistent
        bs.packed_sweep = packed
        for _ in range(3):
            bs.forward(10)
        out.append(bs.x4.clone())
    assert torch.equal(out[0], out[1]) and torch.equal(out[0], out[2])
