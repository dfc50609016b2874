"""OBJ read/write, concatenation with vertex-id offsets (concat.py:11-58) and
per-frame export (meshTaichiWrapper.py:369-386)."""
import os

import numpy as np
import pytest


def test_obj_round_trip_exact(pkg, tmp_path):
    x, f = pkg.grid_cloth(9)
    rng = np.random.default_rng(0)
    x = (x + rng.normal(0, 1e-3, x.shape)).astype(np.float32)
    p = str(tmp_path / "a.obj")
    pkg.meshio.write_obj(p, x, f)
    v2, f2 = pkg.meshio.read_obj(p)
    assert np.array_equal(v2, x) and np.array_equal(f2, f)


def test_obj_corner_forms_and_polygons(pkg, tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("# quad and relative indices\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n"
                 "vt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 3/1/1 4/1/1\nf -4//1 -2//1 -1//1\n")
    v, f = pkg.meshio.read_obj(str(p))
    assert v.shape == (4, 3)
    assert f.tolist() == [[0, 1, 2], [0, 2, 3], [0, 2, 3]]


def test_obj_bad_index(pkg, tmp_path):
    p = tmp_path / "b.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        pkg.meshio.read_obj(str(p))


def test_concat_offsets(pkg, tmp_path):
    x1, f1 = pkg.grid_cloth(4)
    x2, f2 = pkg.box_mesh(0.5, center=(0.0, 0.0, 0.0))
    paths = []
    for i, (x, f) in enumerate(((x1, f1), (x2, f2))):
        paths.append(str(tmp_path / f"m{i}.obj"))
        pkg.meshio.write_obj(paths[-1], x, f)
    out = str(tmp_path / "concat.obj")
    offs = pkg.meshio.concat_obj_files(out, paths, [(1.0, 2.0, 3.0), (0.0, 0.0, -1.0)], [2.0, 0.5])
    assert offs == [0, x1.shape[0], x1.shape[0] + x2.shape[0]]
    v, f = pkg.meshio.read_obj(out)
    assert np.allclose(v[:16], 2.0 * x1 + np.array([1.0, 2.0, 3.0], np.float32), atol=1e-6)
    assert np.allclose(v[16:], 0.5 * x2 + np.array([0.0, 0.0, -1.0], np.float32), atol=1e-6)
    assert np.array_equal(f[: f1.shape[0]], f1) and np.array_equal(f[f1.shape[0]:], f2 + 16)


def test_export_frame_layout(pkg, tmp_path):
    x, f = pkg.grid_cloth(5)
    x4 = np.zeros((x.shape[0], 4), np.float32)
    x4[:, :3] = x
    p = pkg.meshio.export_frame(str(tmp_path), "scene", 7, x4, f)
    assert p == os.path.join(str(tmp_path), "scene", "Mesh_ID_", "Mesh_obj_7.obj")
    ps = pkg.meshio.export_frame(str(tmp_path), "scene", 7, x, f, is_static=True)
    assert "StaticMesh_ID_" in ps
    v, f2 = pkg.meshio.read_obj(p)
    assert np.array_equal(v, x) and np.array_equal(f2, f)


def test_sewing_and_handles_files(pkg, tmp_path):
    p = tmp_path / "sewing.csv"
    p.write_text("3,10\n5,4\n10,7\n")
    pairs = pkg.meshio.load_sewing_pairs(str(p))
    assert pairs.tolist() == [[3, 10], [5, 4], [10, 7]]
    sewn, sptr, partner = pkg.mesh.sewing_adjacency(12, pairs)
    assert sewn.tolist() == [3, 4, 5, 7, 10]
    assert sptr.tolist() == [0, 1, 2, 3, 4, 6]
    # vertex 10: pair 0 (partner 3) before pair 2 (partner 7)
    assert partner.tolist() == [10, 5, 4, 10, 3, 7]
    h = tmp_path / "handle.json"
    h.write_text('{"1": [0, 2], "2": [5], "3": [], "4": []}')
    groups = pkg.meshio.load_handles(str(h))
    assert groups == {1: [0, 2], 2: [5], 3: [], 4: []}
    assert pkg.meshio.handles_mask(groups, 6).tolist() == [1, 0, 1, 0, 0, 1]
    with pytest.raises(ValueError):
        pkg.mesh.sewing_adjacency(4, [[0, 9]])
