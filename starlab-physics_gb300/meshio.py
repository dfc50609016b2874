"""Mesh I/O: OBJ read/write, concatenation with vertex-id offsets, per-frame
export.

Counterparts in the reference: ``framework/meshio/concat.py:11-58``
(``concat_mesh``: read several OBJs, scale then translate each, offset face
indices by the running vertex count, write the concatenation, return the
offsets) and ``MeshTaichiWrapper.export`` (``meshTaichiWrapper.py:369-386``:
one ASCII OBJ per frame under ``<scene>/Mesh_ID_`` or ``StaticMesh_ID_``).
The reference reads and writes through libigl; here the OBJ subset those calls
use -- ``v`` and ``f`` records -- is parsed and written directly, vertices in
file order (the canonical numbering every other part of this package uses).
Faces with more than three corners are split into a fan; ``f a/b/c`` corner
forms and negative (relative) indices are accepted.
"""
from __future__ import annotations

import os

import numpy as np


def read_obj(path):
    """Vertices float32[N, 3] and triangles int32[F, 3] (0-based) of an OBJ file."""
    verts, faces = [], []
    with open(path, "r", encoding="utf-8") as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append((float(parts[1]), float(parts[2]), float(parts[3])))
            elif parts[0] == "f":
                idx = []
                for corner in parts[1:]:
                    k = int(corner.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                if len(idx) < 3:
                    raise ValueError(f"{path}: face with fewer than 3 corners")
                for j in range(1, len(idx) - 1):
                    faces.append((idx[0], idx[j], idx[j + 1]))
    v = np.asarray(verts, dtype=np.float32).reshape(-1, 3)
    f = np.asarray(faces, dtype=np.int32).reshape(-1, 3)
    if f.size and (f.min() < 0 or f.max() >= v.shape[0]):
        raise ValueError(f"{path}: face index out of range")
    return v, f


def write_obj(path, v, f):
    """ASCII OBJ; coordinates with 9 significant digits, so float32 values
    read back exactly."""
    v = np.asarray(v, dtype=np.float32).reshape(-1, 3)
    f = np.asarray(f, dtype=np.int64).reshape(-1, 3)
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w", encoding="utf-8") as fh:
        fh.writelines(f"v {a:.9g} {b:.9g} {c:.9g}\n" for a, b, c in v.tolist())
        fh.writelines(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in f.tolist())


def concat_meshes(meshes, translations, scales):
    """concat_mesh (concat.py:11-58) on in-memory meshes: each (v, f) is scaled,
    then translated; face indices are offset by the vertex counts before it.
    Returns (v, f, vtx_id_offsets) with len(offsets) == len(meshes) + 1."""
    offsets, acc, vs, fs = [], 0, [], []
    for (v, f), t, s in zip(meshes, translations, scales):
        offsets.append(acc)
        v = np.asarray(v, dtype=np.float64)
        vs.append(s * v + np.asarray(t, dtype=np.float64))
        fs.append(np.asarray(f, dtype=np.int64) + acc)
        acc += v.shape[0]
    offsets.append(acc)
    v = np.concatenate(vs, axis=0).astype(np.float32) if vs else np.zeros((0, 3), np.float32)
    f = np.concatenate(fs, axis=0).astype(np.int32) if fs else np.zeros((0, 3), np.int32)
    return v, f, offsets


def concat_obj_files(out_path, model_paths, translations, scales):
    """concat_mesh on files: reads every model, writes the concatenation to
    out_path, returns the vertex-id offsets."""
    v, f, offsets = concat_meshes([read_obj(p) for p in model_paths], translations, scales)
    write_obj(out_path, v, f)
    return offsets


def export_frame(results_dir, scene_name, frame, x, faces, is_static=False):
    """MeshTaichiWrapper.export: positions x ([V, 3] or [V, 4], host or device)
    to <results_dir>/<scene_name>/(Static)Mesh_ID_/Mesh_obj_<frame>.obj."""
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    x = np.asarray(x)[:, :3]
    sub = "StaticMesh_ID_" if is_static else "Mesh_ID_"
    path = os.path.join(results_dir, scene_name, sub, f"Mesh_obj_{frame}.obj")
    write_obj(path, x, faces)
    return path


def load_sewing_pairs(path):
    """Sewing pairs from a CSV of two vertex ids per row (the reference's
    animation/sewing.csv, XPBD.py:407-417)."""
    import csv

    with open(path, "r", encoding="utf-8") as fh:
        rows = [r for r in csv.reader(fh) if r]
    return np.asarray(rows, dtype=np.int32).reshape(-1, 2)


def load_handles(path):
    """Handle groups {group: [vertex ids]} from the selection tool's JSON
    (selection_tool.py:176-228: keys are group numbers as strings)."""
    import json

    with open(path, "r", encoding="utf-8") as fh:
        raw = json.load(fh)
    return {int(k): [int(i) for i in v] for k, v in raw.items()}


def handles_mask(handles, n_verts):
    """A mask for Solver.set_fixed_vertices: 1 where a vertex belongs to any
    handle group."""
    m = np.zeros(n_verts, dtype=np.int32)
    for ids in handles.values():
        m[np.asarray(ids, dtype=np.int64)] = 1
    return m
