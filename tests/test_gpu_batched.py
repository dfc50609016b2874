"""Batched independent cloths with obstacles: every instance of a BatchedSolver
run equals that instance simulated alone by the CPU oracle (obstacle contacts
only, BVHs rebuilt every substep), bit for bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _instances(pkg, seed=3, n_inst=5):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_inst):
        n = int(rng.integers(6, 15))
        ox = 1.5 * i
        x, f = pkg.grid_cloth(n, origin=(ox, 0.0), height=1.0)
        x = (x + rng.uniform(-1e-4, 1e-4, x.shape).astype(np.float32)).astype(np.float32)
        # box top 6 mm below the cloth, shifted so that some cloth lies past its edges
        bx, bf = pkg.box_mesh(0.5, center=(ox + 0.5 + rng.uniform(-0.3, 0.3), 0.5 + rng.uniform(-0.3, 0.3), 0.744))
        out.append(pkg.Instance(x, f, np.array([(n - 1) * n, n * n - 1]), bx, bf))
    return out


def _oracle_instance(pkg, po, inst, frames, kw):
    from starlab_physics_gb300 import mesh as M

    cl = M.TriMesh(inst.x, inst.faces, device="cpu")
    cl.fixed[np.asarray(inst.pinned)] = 0.0
    ob = M.TriMesh(inst.obstacle_x, inst.obstacle_faces, device="cpu")
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), collisions=True,
                          rebuild="substep", self_collision=False, bending_on="y", **kw)
    for _ in range(frames):
        orc.forward(10)
    return orc


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_equals_single_instances(pkg, po, use_graph):
    insts = _instances(pkg)
    kw = dict(dt=1 / 60, g=(0.0, 0.0, -9.81), k_stretch_stiffness=1e5, k_bend_stiffness=1e8, dHat=(4e-3) ** 2,
              damping=0.001, padding=8e-3, n_iter=3, cap=40)
    sim = pkg.BatchedSolver(insts, dHat=kw["dHat"], stiffness_stretch=1e5, stiffness_bending=1e8, g=kw["g"],
                            dt=kw["dt"], n_iter=3, padding=8e-3)
    sim.use_graph = use_graph
    frames = 4
    for _ in range(frames):
        sim.forward(10)
    torch.cuda.synchronize()
    contacts = 0
    for i, inst in enumerate(insts):
        orc = _oracle_instance(pkg, po, inst, frames, kw)
        got = sim.instance_positions(i).cpu().numpy()
        assert np.array_equal(got, orc.x4[:, :3]), f"instance {i}: max diff {np.abs(got - orc.x4[:, :3]).max()}"
        # the box stops the cloth: some vertex sits above the free-fall height
        contacts += int((orc.x4[:, 2] > 0.99).sum())
    assert contacts > 0
    assert int(sim.status.item()) & 4 == 0


def test_batched_tolerance_mode(pkg):
    """The batched solver's tolerance mode: tol large stops every substep at the
    first check (iteration 4; its block runs to iteration 7, a fixed
    8-iteration run), tol 0 never stops (a full run), and an intermediate
    tolerance stops some substeps; graph replay (a device-side loop) equals
    eager (gated launches)."""
    insts = _instances(pkg, seed=5)

    def run(tol, n_iter=12, use_graph=False, frames=2):
        sim = pkg.BatchedSolver(insts, dHat=(4e-3) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8,
                                g=(0.0, 0.0, -9.81), dt=1 / 60, n_iter=n_iter, padding=8e-3)
        sim.tol = tol
        sim.use_graph = use_graph
        for _ in range(frames):
            sim.forward(10)
        torch.cuda.synchronize()
        return sim

    big, eight = run(1.0), run(None, n_iter=8)
    assert big.convergence_stats()["converged_substeps"] == 20
    assert torch.equal(big.x4, eight.x4)
    assert torch.equal(run(1.0, use_graph=True).x4, eight.x4)
    zero, full = run(0.0), run(None)
    assert zero.convergence_stats()["converged_substeps"] == 0
    assert torch.equal(zero.x4, full.x4)
    assert torch.equal(run(0.0, use_graph=True).x4, full.x4)
    probe = run(0.0, frames=1)
    tol = probe.convergence_stats()["last_residual"]
    mid, mid_g = run(tol), run(tol, use_graph=True)
    n = mid.convergence_stats()["converged_substeps"]
    assert 0 < n < 20
    assert torch.equal(mid.x4, mid_g.x4)
    assert mid_g.convergence_stats()["converged_substeps"] == n


@pytest.mark.parametrize("fast", [False, True])
def test_persistent_substep_equals_grid_launches(pkg, fast):
    """One persistent launch per substep (sx_batched_substep: an instance per
    CTA with block barriers, or per thread-block cluster with cluster barriers)
    gives the same frames as the graph of grid-wide launches, bit for bit, in
    every launch configuration, with the exact and with the fast arithmetic,
    for an even and an odd iteration count."""
    from starlab_physics_gb300._lib import sx

    insts = _instances(pkg, seed=7, n_inst=9)
    for n_iter in (4, 3):
        def run(persistent, variant=0):
            sim = pkg.BatchedSolver(insts, dHat=(4e-3) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8,
                                    g=(0.0, 0.0, -9.81), dt=1 / 60, n_iter=n_iter, padding=8e-3)
            sim.fast_math = fast
            sim.persistent = persistent
            sim.persistent_variant = variant
            sim.use_graph = True
            for _ in range(5):
                sim.forward(10)
            torch.cuda.synchronize()
            return sim

        ref = run(False)
        for v in range(int(sx.sx_batched_substep_variants())):
            got = run(True, v)
            assert torch.equal(got.x4, ref.x4) and torch.equal(got.v4, ref.v4), (n_iter, v)
            assert int(got.status.item()) == int(ref.status.item())
            assert int(got._p_queue.abs().sum().item()) == 0


def test_persistent_substep_batched512(pkg):
    """The 512-cloth batch (3.2 M vertices): two frames of persistent launches
    equal two frames of grid-wide launches bit for bit; the autotuner's pick
    gives the same result."""
    insts = pkg.batched_scene(512, seed=0)

    def make():
        return pkg.BatchedSolver(insts, dHat=(4e-3) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8,
                                 g=(0.0, 0.0, -9.81), dt=1 / 60, n_iter=20, padding=8e-3)

    a = make()
    a.use_graph = True
    for _ in range(2):
        a.forward(10)
    b = make()
    b.persistent = True
    b.use_graph = True
    for _ in range(2):
        b.forward(10)
    torch.cuda.synchronize()
    assert torch.equal(a.x4, b.x4) and torch.equal(a.v4, b.v4)
    variant, times = b.autotune_persistent(reps=1)
    assert 0 <= variant < len(times)
    b.forward(10)
    a.forward(10)
    torch.cuda.synchronize()
    assert torch.equal(a.x4, b.x4)
    # an instance per 8-CTA cluster, reading the packed adjacency
    from starlab_physics_gb300._lib import sx

    b.persistent_variant = next(v for v in range(int(sx.sx_batched_substep_variants()))
                                if int(sx.sx_batched_substep_variant_cluster(v)) == 8)
    b.packed_sweep = True
    b.forward(10)
    a.forward(10)
    torch.cuda.synchronize()
    assert torch.equal(a.x4, b.x4) and torch.equal(a.v4, b.v4)
