"""Seeded synthetic scenes for the benchmark workloads.

The reference ships scene modules (``Scenes/concat_test.py``,
``Scenes/test_ee.py``) that load OBJ assets; the workloads here are synthetic
with the shapes, sizes and parameters of the benchmark configurations:

* ``plain64``   -- 64 x 64 cloth (4096 vertices, 7938 faces, 12033 springs,
  11781 bending pairs) at z = 1, the two corners at y = 1 pinned, uniform
  +-1e-4 jitter, over a static box (side 0.5, centre (0.5, 0.5, 0.3), 12 faces);
  dt = 1/60, 10 substeps, 20 Jacobi iterations; springs 1e8 (compliance 1e-8),
  bending 1e5 (compliance 1e-5); gravity (0, 0, -9.81).
* ``drape256``  -- 256 x 256 cloth (65536 vertices, 130050 faces) 5 mm above a
  static icosphere of 20480 faces, radius 0.3; Gaussian sigma 1e-3 normal (z)
  offsets; contact thickness 2e-3 (dHat = thickness^2, since the reference
  compares squared distances); 10 substeps, 30 iterations; BVHs rebuilt every
  substep.
* ``crossed_layers`` -- two coarse 6 x 6 cloth layers (side 0.7, edges 0.14),
  the lower one turned by 35 degrees, falling onto a box (side 0.5): long
  edges crossing at close range, the case in which the reference's
  edge-edge classifier (whose interior case needs a triple product >= 1e-4)
  reports edge-edge contacts; 5 substeps, 4 iterations, thickness 0.02.
* ``soup``      -- 2^20 random triangles for the standalone broad phase:
  centroids U[0,1]^3, edge lengths U[1e-3, 1e-2], random orientation; queries
  are the first vertex of every triangle with padding 2e-3.

Stiffness arguments follow the reference's constructor, whose stretch springs
use ``stiffness_bending`` and bending pairs ``stiffness_stretch``
(``XPBD.py:354-355``): a scene that wants springs at 1e8 and bending at 1e5
passes ``stiffness_bending=1e8, stiffness_stretch=1e5``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import box_mesh, grid_cloth, icosphere


@dataclass
class Scene:
    name: str
    cloth_x: np.ndarray
    cloth_faces: np.ndarray
    obstacle_x: np.ndarray | None
    obstacle_faces: np.ndarray | None
    pinned: np.ndarray              # vertex ids with fixed = 0
    dt: float
    n_substeps: int
    n_iter: int
    gravity: tuple
    stiffness_stretch: float       # reference argument (used by bending pairs)
    stiffness_bending: float       # reference argument (used by springs)
    dHat: float
    padding: float
    damping: float = 0.001
    collisions: bool = True
    rebuild: str = "substep"
    cap: int = 40
    meta: dict = field(default_factory=dict)


def plain64(n: int = 64, seed: int = 0, collisions: bool = True) -> Scene:
    rng = np.random.default_rng(seed)
    x, f = grid_cloth(n, height=1.0)
    x = (x + rng.uniform(-1e-4, 1e-4, size=x.shape).astype(np.float32)).astype(np.float32)
    bx, bf = box_mesh(0.5, center=(0.5, 0.5, 0.3))
    pinned = np.array([(n - 1) * n, n * n - 1], dtype=np.int64)
    thickness = 4e-3
    return Scene("plain64", x, f, bx, bf, pinned, dt=1.0 / 60.0, n_substeps=10, n_iter=20,
                 gravity=(0.0, 0.0, -9.81), stiffness_stretch=1e5, stiffness_bending=1e8,
                 dHat=thickness * thickness, padding=2 * thickness, collisions=collisions, rebuild="substep",
                 meta={"grid": n, "thickness": thickness})


def drape256(n: int = 256, seed: int = 0, sphere_subdiv: int = 5, gap: float = 0.005) -> Scene:
    rng = np.random.default_rng(seed)
    radius = 0.3
    center = (0.5, 0.5, 0.5)
    x, f = grid_cloth(n, height=center[2] + radius + gap)
    x[:, 2] = (x[:, 2] + rng.normal(0.0, 1e-3, size=x.shape[0]).astype(np.float32)).astype(np.float32)
    sx_, sf = icosphere(sphere_subdiv, radius, center)
    thickness = 2e-3
    return Scene("drape256", x, f, sx_, sf, np.zeros(0, np.int64), dt=1.0 / 60.0, n_substeps=10, n_iter=30,
                 gravity=(0.0, 0.0, -9.81), stiffness_stretch=1e5, stiffness_bending=1e8,
                 dHat=thickness * thickness, padding=thickness, collisions=True, rebuild="substep",
                 meta={"grid": n, "thickness": thickness, "sphere_faces": int(sf.shape[0])})


def crossed_layers() -> Scene:
    a_x, a_f = grid_cloth(6, origin=(0.15, 0.15), size=0.7, height=0.56)
    b_x, b_f = grid_cloth(6, origin=(0.0, 0.0), size=0.7, height=0.53)
    th = np.deg2rad(35.0)
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]], np.float32)
    b_x = b_x.copy()
    b_x[:, :2] = ((b_x[:, :2] - np.float32(0.35)) @ R.T + np.float32(0.5)).astype(np.float32)
    x = np.concatenate([a_x, b_x]).astype(np.float32)
    f = np.concatenate([a_f, b_f + a_x.shape[0]]).astype(np.int32)
    bx, bf = box_mesh(0.5, center=(0.5, 0.5, 0.25))
    thickness = 0.02
    return Scene("crossed_layers", x, f, bx, bf, np.zeros(0, np.int64), dt=1.0 / 60.0, n_substeps=5, n_iter=4,
                 gravity=(0.0, 0.0, -9.81), stiffness_stretch=1e5, stiffness_bending=1e8,
                 dHat=thickness * thickness, padding=2 * thickness, collisions=True, rebuild="substep",
                 meta={"thickness": thickness})


def triangle_soup(n_tris: int = 1 << 20, seed: int = 0):
    """Returns (verts float32[3n,3], faces int32[n,3], queries float32[n,3])."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, size=(n_tris, 3))
    # random orthonormal frame per triangle, then three edge lengths
    q = rng.normal(size=(n_tris, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, a, b, d = q.T
    R = np.stack([np.stack([1 - 2 * (b * b + d * d), 2 * (a * b - d * w), 2 * (a * d + b * w)], -1),
                  np.stack([2 * (a * b + d * w), 1 - 2 * (a * a + d * d), 2 * (b * d - a * w)], -1),
                  np.stack([2 * (a * d - b * w), 2 * (b * d + a * w), 1 - 2 * (a * a + b * b)], -1)], 1)
    L = rng.uniform(1e-3, 1e-2, size=(n_tris, 2))
    ang = rng.uniform(np.pi / 6, 5 * np.pi / 6, size=n_tris)
    p0 = np.zeros((n_tris, 3))
    p1 = np.stack([L[:, 0], np.zeros(n_tris), np.zeros(n_tris)], -1)
    p2 = np.stack([L[:, 1] * np.cos(ang), L[:, 1] * np.sin(ang), np.zeros(n_tris)], -1)
    local = np.stack([p0, p1, p2], 1)
    local -= local.mean(axis=1, keepdims=True)
    world = np.einsum("nij,nkj->nki", R, local) + c[:, None, :]
    verts = world.reshape(-1, 3).astype(np.float32)
    faces = np.arange(3 * n_tris, dtype=np.int32).reshape(n_tris, 3)
    queries = verts[0::3].copy()
    return verts, faces, queries


def make_solver(scene: Scene, device="cuda"):
    """TriMesh objects + Solver configured for ``scene``."""
    from .mesh import TriMesh
    from .solver import Solver
    import torch

    cloth = TriMesh(scene.cloth_x, scene.cloth_faces, device=device)
    obst = None
    if scene.obstacle_x is not None:
        obst = TriMesh(scene.obstacle_x, scene.obstacle_faces, device=device, is_static=True)
    sim = Solver(cloth, obst, dHat=scene.dHat, stiffness_stretch=scene.stiffness_stretch,
                 stiffness_bending=scene.stiffness_bending, g=scene.gravity, dt=scene.dt, n_iter=scene.n_iter,
                 rebuild=scene.rebuild, cap=scene.cap)
    sim.damping = scene.damping
    sim.padding = scene.padding
    sim.enable_collision_handling = scene.collisions
    mask = np.zeros(cloth.num_verts, np.int32)
    mask[scene.pinned] = 1
    sim.set_fixed_vertices(torch.from_numpy(mask))
    return sim


def oracle_inputs(mesh):
    """Host arrays of a TriMesh in the form the CPU oracle takes."""
    return {
        "x": mesh.x0_np, "faces": mesh.fid_np, "edges": mesh.eid_np, "face_edges": mesh.face_edge_np,
        "l0": mesh.l0_np,
        "bend": mesh.bending_np, "bend_l0": mesh.bending_l0_np, "m_inv": mesh.m_inv_np,
        "fixed": mesh.fixed.detach().cpu().numpy(),
    }
