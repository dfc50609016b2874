"""Constraint-graph colouring (mirrors framework/utilities/graph_coloring.py).

:class:`GraphColoring` colours the edges of a mesh so that no two edges sharing
a vertex have the same colour -- the grouping a parallel Gauss-Seidel sweep
needs -- and sorts edge ids by colour.  The colouring equals the reference's
sequential first-fit in edge-id order (``colorEdgesGreedy``,
``graph_coloring.py:131-149``) and the sort is its stable counting sort
(``colorCountingSort``, ``graph_coloring.py:172-201``); both run on the GPU
(``sx_color_edges_greedy``).  Results can be cached to / loaded from ``.npy``
files like the reference's ``precomputed/<mesh>_{prefix_sum,
sorted_edges_index}.npy`` (``graph_coloring.py:39-53``, ``:290-299``).
"""
from __future__ import annotations

import os

import numpy as np
import torch

from ._lib import ptr, stream_handle, sx


class GraphColoring:
    max_num_colors = 100

    def __init__(self, num_verts: int, edges, *, device="cuda", max_num_colors: int = 100, cache_dir=None,
                 mesh_name: str | None = None):
        self.num_verts = int(num_verts)
        dev = torch.device(device)
        e = torch.as_tensor(np.asarray(edges, dtype=np.int32).reshape(-1, 2) if not torch.is_tensor(edges)
                            else edges.reshape(-1, 2).to(torch.int32)).to(dev).contiguous()
        self.edges = e
        self.num_edges = e.shape[0]
        self.max_num_colors = int(max_num_colors)
        self.device = dev
        self.edges_color = torch.empty(max(self.num_edges, 1), dtype=torch.int32, device=dev)
        self.sorted_edges_sequence_for_color = torch.empty(max(self.num_edges, 1), dtype=torch.int32, device=dev)
        self.color_prefix_sum = torch.zeros(self.max_num_colors, dtype=torch.int32, device=dev)
        self.cache_dir = cache_dir
        self.mesh_name = mesh_name
        if cache_dir and mesh_name and self._load_cache():
            return
        ws_bytes = int(sx.sx_color_workspace_bytes(self.num_verts, self.num_edges))
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        sx.sx_color_edges_greedy(ptr(e), self.num_edges, self.num_verts, self.max_num_colors, ptr(self.edges_color),
                                 ptr(self.sorted_edges_sequence_for_color), ptr(self.color_prefix_sum), ptr(ws),
                                 ws_bytes, stream_handle())
        # device-side status of the colouring rounds (first int of the workspace)
        status = int(ws[:4].view(torch.int32).item()) if self.num_edges else 0
        if status:
            raise RuntimeError(f"sx_color_edges_greedy: status {status:#x} (a bounded wait gave up)")
        if cache_dir and mesh_name:
            self.exportColorResult()

    @property
    def num_colors(self) -> int:
        if self.num_edges == 0:
            return 0
        return int(self.edges_color[: self.num_edges].max().item()) + 1

    def _paths(self):
        return (os.path.join(self.cache_dir, f"{self.mesh_name}_prefix_sum.npy"),
                os.path.join(self.cache_dir, f"{self.mesh_name}_sorted_edges_index.npy"))

    def _load_cache(self) -> bool:
        a, b = self._paths()
        if not (os.path.isfile(a) and os.path.isfile(b)):
            return False
        self.color_prefix_sum.copy_(torch.from_numpy(np.load(a).astype(np.int32)))
        self.sorted_edges_sequence_for_color[: self.num_edges].copy_(torch.from_numpy(np.load(b).astype(np.int32)))
        return True

    def exportColorResult(self):
        """``graph_coloring.py:290-299``: save prefix sums and sorted edge ids."""
        os.makedirs(self.cache_dir, exist_ok=True)
        a, b = self._paths()
        np.save(a, self.color_prefix_sum.cpu().numpy())
        np.save(b, self.sorted_edges_sequence_for_color[: self.num_edges].cpu().numpy())
