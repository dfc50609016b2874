"""starxpbd: GB300-native (sm_103a) XPBD cloth substep.

A drop-in for the Taichi hot path of medialab-ku/starlab-physics
(``framework/physics/XPBD.py`` Solver, ``framework/collision/lbvh_cell.py``
LBVH_CELL, ``framework/utilities/graph_coloring.py`` GraphColoring): state in
torch CUDA tensors, hand-written CUDA kernels behind the C ABI of
``include/starxpbd.h`` (``libstarxpbd.so``), no CPU fallback.
"""
from . import _lib
from ._lib import SxError, load as load_library, library_path
from .coloring import GraphColoring
from .lbvh import LBVH, LBVH_CELL
from .mesh import TriMesh, box_mesh, grid_cloth, icosphere
from .solver import Solver
from .batched import BatchedSolver, Instance, batched_scene, shard_instances
from . import scenes
from . import learned
from . import meshio
from .learned import WarmStart, WarmStartMLP

__all__ = ["Solver", "BatchedSolver", "Instance", "batched_scene", "shard_instances", "LBVH_CELL", "LBVH", "GraphColoring", "TriMesh",
           "grid_cloth", "box_mesh", "icosphere", "scenes", "learned", "meshio", "WarmStart", "WarmStartMLP", "SxError",
           "load_library", "library_path"]
