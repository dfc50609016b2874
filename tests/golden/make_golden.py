"""Generate tests/golden/golden.npz from the CPU oracle.

The reference (Python + Taichi 1.7.1) cannot run in this environment, so the
golden vectors are outputs of the CPU oracle (a restatement of the reference
algorithms, itself pinned by the known-answer and literal-restatement tests in
tests/test_oracle.py) on small seeded inputs.  They freeze the oracle's
behaviour and give the GPU tests fixed expected outputs.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cases():
    """Inputs of every golden case, regenerated identically by the tests."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    from starlab_physics_gb300 import mesh as M

    out = {}
    rng = np.random.default_rng(2024)
    out["morton_pts"] = rng.uniform(-0.1, 1.1, (257, 3)).astype(np.float32)
    verts, faces, queries = pkg.scenes.triangle_soup(2048, seed=9)
    V4 = np.zeros((verts.shape[0], 4), np.float32)
    V4[:, :3] = verts
    Q4 = np.zeros((queries.shape[0], 4), np.float32)
    Q4[:, :3] = queries
    out["soup"] = (V4, faces, Q4)
    x, f = M.grid_cloth(9)
    out["grid9_edges"] = M.edges_from_faces(f)
    return pkg, out


def solver_case(pkg, name):
    """Scenes of the end-to-end golden runs: (scene, bending_on, frames)."""
    if name == "plain16_reference":
        s = pkg.scenes.plain64(n=16, seed=4)
        s.n_iter, s.rebuild, s.padding = 1, "frame", 0.04
        return s, "x", 4
    if name == "plain16_iterated":
        s = pkg.scenes.plain64(n=16, seed=4)
        s.n_iter = 5
        return s, "y", 4
    if name == "drape24":
        s = pkg.scenes.drape256(n=24, seed=4, sphere_subdiv=2, gap=0.003)  # contacts from frame 1
        s.n_iter = 4
        return s, "y", 4
    raise KeyError(name)


SOLVER_CASES = ("plain16_reference", "plain16_iterated", "drape24")


def run_oracle_solver(pkg, name):
    from oracle import pyoracle as po
    from starlab_physics_gb300 import mesh as M

    s, bend, frames = solver_case(pkg, name)
    cl = M.TriMesh(s.cloth_x, s.cloth_faces, device="cpu")
    ob = M.TriMesh(s.obstacle_x, s.obstacle_faces, device="cpu")
    cl.fixed[s.pinned] = 0.0
    orc = po.OracleSolver(pkg.scenes.oracle_inputs(cl), pkg.scenes.oracle_inputs(ob), dt=s.dt, g=s.gravity,
                          k_stretch_stiffness=s.stiffness_stretch, k_bend_stiffness=s.stiffness_bending,
                          dHat=s.dHat, damping=s.damping, padding=s.padding, n_iter=s.n_iter,
                          collisions=s.collisions, rebuild=s.rebuild, cap=s.cap, bending_on=bend)
    for _ in range(frames):
        orc.forward(s.n_substeps)
    return orc.x4[:, :3].copy(), orc.v4[:, :3].copy()


def main():
    from oracle import pyoracle as po

    pkg, c = cases()
    g = {}
    g["morton_codes"] = po.morton3d(c["morton_pts"])
    cb = po.CellBVH()
    g["cell_init_sha"] = np.array(sha(cb.codes, cb.ids, cb.child_a, cb.child_b, cb.range_l, cb.range_r, cb.parent))
    V4, faces, Q4 = c["soup"]
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    box = po.scene_aabb(V4, 0.0)
    fb = po.FaceBVH(mn, mx, box, tie=1)
    g["soup_sorted_codes"] = fb.sorted_codes
    g["soup_sorted_ids"] = fb.sorted_ids
    g["soup_child_a"], g["soup_child_b"] = fb.child_a, fb.child_b
    g["soup_range_l"], g["soup_range_r"] = fb.range_l, fb.range_r
    qmn, qmx = po.query_boxes(Q4, 2e-3)
    cand, num, _ = fb.traverse(qmn, qmx, 32)
    g["soup_num"], g["soup_cand"] = num, cand
    color, sorted_e, prefix = po.color_edges(81, c["grid9_edges"])
    g["grid9_color"], g["grid9_sorted"], g["grid9_prefix"] = color, sorted_e, prefix
    for name in SOLVER_CASES:
        x, v = run_oracle_solver(pkg, name)
        g[f"{name}_x"], g[f"{name}_v"] = x, v
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **g)
    print("wrote", os.path.join(HERE, "golden.npz"), {k: np.asarray(v).shape for k, v in g.items()})


if __name__ == "__main__":
    main()
