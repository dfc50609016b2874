"""Committed golden vectors (tests/golden/golden.npz, made by make_golden.py):
the CPU oracle must reproduce them (regression pin) and the CUDA path must match
them bit for bit."""
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as mg  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "golden.npz"))


@pytest.fixture(scope="module")
def inputs(pkg):
    return mg.cases()[1]


def test_oracle_reproduces_golden(pkg, po, inputs):
    assert np.array_equal(po.morton3d(inputs["morton_pts"]), G["morton_codes"])
    cb = po.CellBVH()
    assert mg.sha(cb.codes, cb.ids, cb.child_a, cb.child_b, cb.range_l, cb.range_r, cb.parent) == str(G["cell_init_sha"])
    V4, faces, Q4 = inputs["soup"]
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    fb = po.FaceBVH(mn, mx, po.scene_aabb(V4, 0.0), tie=1)
    for k, a in [("soup_sorted_codes", fb.sorted_codes), ("soup_sorted_ids", fb.sorted_ids),
                 ("soup_child_a", fb.child_a), ("soup_child_b", fb.child_b), ("soup_range_l", fb.range_l),
                 ("soup_range_r", fb.range_r)]:
        assert np.array_equal(a, G[k]), k
    c, s, p = po.color_edges(81, inputs["grid9_edges"])
    assert np.array_equal(c, G["grid9_color"]) and np.array_equal(s, G["grid9_sorted"])
    assert np.array_equal(p, G["grid9_prefix"])


@pytest.mark.parametrize("name", mg.SOLVER_CASES)
def test_oracle_solver_golden(pkg, name):
    x, v = mg.run_oracle_solver(pkg, name)
    assert np.array_equal(x, G[f"{name}_x"]) and np.array_equal(v, G[f"{name}_v"])


def test_golden_cases_exercise_contacts(pkg):
    """drape24 must reach the sphere: its end state differs from a collision-free run."""
    from oracle import pyoracle as po
    from starlab_physics_gb300 import mesh as M

    s, bend, frames = mg.solver_case(pkg, "drape24")
    cl = M.TriMesh(s.cloth_x, s.cloth_faces, device="cpu")
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), None, dt=s.dt, g=s.gravity,
                          k_stretch_stiffness=s.stiffness_stretch, k_bend_stiffness=s.stiffness_bending,
                          n_iter=s.n_iter, bending_on=bend)
    for _ in range(frames):
        orc.forward(s.n_substeps)
    assert np.abs(orc.x4[:, :3] - G["drape24_x"]).max() > 1e-3


# ---------------------------------------------------------------- GPU ----
@pytest.mark.gpu
def test_gpu_matches_golden_lbvh_and_coloring(pkg, inputs):
    dev = "cuda"
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    from oracle import pyoracle as po

    V4, faces, Q4 = inputs["soup"]
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    box = po.scene_aabb(V4, 0.0)
    b = pkg.LBVH(faces.shape[0], dev, tie=1)
    b.build(t(mn), t(mx), t(box))
    n = faces.shape[0]
    assert np.array_equal(b.codes.cpu().numpy(), G["soup_sorted_codes"])
    assert np.array_equal(b.sorted_ids.cpu().numpy(), G["soup_sorted_ids"])
    assert np.array_equal(b.child_a.cpu().numpy()[: n - 1], G["soup_child_a"])
    assert np.array_equal(b.child_b.cpu().numpy()[: n - 1], G["soup_child_b"])
    cand, num = b.query(t(Q4), 2e-3, 32)
    assert np.array_equal(num.cpu().numpy(), G["soup_num"])
    gc = cand.cpu().numpy()
    for q in range(n):
        k = min(G["soup_num"][q], 32)
        assert np.array_equal(gc[q, :k], G["soup_cand"][q, :k])
    gcol = pkg.GraphColoring(81, inputs["grid9_edges"], device=dev)
    assert np.array_equal(gcol.edges_color.cpu().numpy()[:208], G["grid9_color"])
    assert np.array_equal(gcol.sorted_edges_sequence_for_color.cpu().numpy()[:208], G["grid9_sorted"])
    assert np.array_equal(gcol.color_prefix_sum.cpu().numpy(), G["grid9_prefix"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", mg.SOLVER_CASES)
def test_gpu_solver_golden(pkg, name):
    s, bend, frames = mg.solver_case(pkg, name)
    sim = pkg.scenes.make_solver(s, device="cuda")
    sim.bending_on = bend
    for _ in range(frames):
        sim.forward(s.n_substeps)
    x = sim.mesh_dy.x4[:, :3].cpu().numpy()
    v = sim.mesh_dy.v4[:, :3].cpu().numpy()
    diag = sim.mesh_dy.bbox_diagonal()
    assert np.abs(x - G[f"{name}_x"]).max() <= 1e-4 * diag
    assert np.array_equal(x, G[f"{name}_x"]) and np.array_equal(v, G[f"{name}_v"])
