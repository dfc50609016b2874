"""Autotuner for the launch configuration of the Jacobi sweep (and the list
of the contact-pair projection's configurations).

The sweep kernel is compiled in several configurations -- how many adjacency
entries a thread loads before it computes, how many threads a block holds
(``sx_jacobi_sweep_variant_info``), how many lanes share one vertex and
whether the adjacency is read with the streaming cache policy
(``sx_jacobi_sweep_variant_form``); all give bit-identical results.  The best one depends on the mesh: a 65 536-vertex cloth whose sweep
is L2-resident and latency-bound wants more loads in flight per thread, a
3.2 M-vertex batch that streams from HBM wants more resident threads.
:func:`tune_sweep` times every configuration on the caller's own arrays (a
CUDA graph of back-to-back sweeps, CUDA events, median of rounds) and returns
the fastest; results are cached per (device, vertex count, adjacency size).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import load, ptr, stream_handle, sx

_cache: dict = {}


def variants() -> list[tuple[int, int]]:
    """(entries per load batch, threads per block) of every compiled variant."""
    L = load()
    out = []
    for k in range(int(L.sx_jacobi_sweep_variants())):
        g, b = C.c_int(0), C.c_int(0)
        sx.sx_jacobi_sweep_variant_info(k, C.addressof(g), C.addressof(b))
        out.append((g.value, b.value))
    return out


def variant_forms() -> list[tuple[int, int]]:
    """(lanes per vertex, streaming adjacency loads) of every compiled variant."""
    L = load()
    out = []
    for k in range(int(L.sx_jacobi_sweep_variants())):
        lanes, st = C.c_int(0), C.c_int(0)
        sx.sx_jacobi_sweep_variant_form(k, C.addressof(lanes), C.addressof(st))
        out.append((lanes.value, st.value))
    return out


def packed_forms() -> int:
    """Forms of the packed sweep (0 staged, 1.. direct launch configurations)."""
    return int(load().sx_jacobi_sweep_packed_forms())


def _time_variant(v, args, reps, rounds):
    """v: a compiled variant of the int2 sweep, or ("packed", form): the sweep
    over the packed adjacency, staged per block in shared memory (form 0) or
    read from global memory (forms 1..)."""
    x4, y4, out, fixed, adj_ptr, adj, n, ks, kb, bend_y, packed, fast = args

    def run():
        if isinstance(v, tuple):
            sx.sx_jacobi_sweep_packed_v(ptr(x4), ptr(y4), ptr(out), ptr(fixed), ptr(adj_ptr), ptr(packed[0]),
                                        ptr(packed[1]), n, ks, kb, bend_y, v[1], fast, stream_handle())
        else:
            sx.sx_jacobi_sweep_mode(ptr(x4), ptr(y4), ptr(out), ptr(fixed), ptr(adj_ptr), ptr(adj), n, ks, kb, bend_y,
                                    v, fast, stream_handle())

    side = torch.cuda.Stream(device=x4.device)
    side.wait_stream(torch.cuda.current_stream(x4.device))
    with torch.cuda.stream(side):
        run()
    torch.cuda.current_stream(x4.device).wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(reps):
            run()
    g.replay()
    torch.cuda.synchronize()
    ts = []
    for _ in range(rounds):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        g.replay()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / reps)
    return float(np.median(ts))


def tune_sweep(x4, y4, fixed, adj_ptr, adj, n_verts, k_spring, k_bend, bend_on_y=1, reps=20, rounds=5, packed=None,
               fast=False):
    """Fastest sweep variant for these arrays, and the per-variant times (ms).

    ``packed``: the (nbr16, rest32) arrays of the packed adjacency, or None;
    when given, every form of the packed sweep is timed as one more candidate,
    the last entries of the times (index ``len(variants()) + form``).
    ``fast``: time the fast arithmetic."""
    if packed is not None and packed[0] is None:
        packed = None
    key = (torch.cuda.get_device_name(x4.device), int(n_verts), int(adj.shape[0]), packed is not None, bool(fast))
    if key in _cache:
        return _cache[key]
    out = torch.empty_like(y4)
    args = (x4, y4, out, fixed, adj_ptr, adj, int(n_verts), float(k_spring), float(k_bend), int(bend_on_y), packed,
            1 if fast else 0)
    cands = list(range(len(variants()))) + ([("packed", f) for f in range(packed_forms())] if packed is not None
                                            else [])
    times = [_time_variant(v, args, reps, rounds) for v in cands]
    best = int(np.argmin(times))
    _cache[key] = (best, times)
    return best, times


def pairs_project_variants() -> list[tuple[int, int]]:
    """(pair batches box-tested per warp step, resident blocks per SM) of every
    compiled configuration of the contact-pair projection."""
    L = load()
    out = []
    for k in range(int(L.sx_contact_pairs_project_variants())):
        u, b = C.c_int(0), C.c_int(0)
        sx.sx_contact_pairs_project_variant_info(k, C.addressof(u), C.addressof(b))
        out.append((u.value, b.value))
    return out
