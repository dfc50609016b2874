"""ctypes binding of ``libstarxpbd.so`` (declared in include/starxpbd.h).

Every wrapper passes raw device pointers (``tensor.data_ptr()``), sizes and the
current CUDA stream, and raises :class:`SxError` when the C ABI returns a
nonzero code.  There is no CPU fallback: if the library is missing it is built
with nvcc, and if that fails, or no CUDA device is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

P = C.c_void_p
I = C.c_int
F = C.c_float
Z = C.c_size_t

SX_OK = 0
SX_ERR_ARG = -1
SX_ERR_CAPACITY = -2
SX_ERR_TIMEOUT = -3
SX_ERR_CUDA = -4

STATUS_CAND_OVERFLOW = 1
STATUS_STACK_OVERFLOW = 2
STATUS_FIXED_RANGE = 4
STATUS_CLIMB_LIMIT = 8

class SxBatchedSubstep(C.Structure):
    """The argument block of sx_batched_substep (include/starxpbd.h)."""

    _fields_ = [(n, I) for n in ("n_inst", "n_iter", "predict", "cap")] + \
               [(n, P) for n in ("order", "vptr", "fptr", "cptr", "optr", "ob_fptr", "x4", "y4", "y_other4", "v4",
                                 "fixed", "m_inv", "adj_ptr", "adj", "adj_nbr16", "adj_rest32", "faces", "ob_faces",
                                 "xs4", "fmin4", "fmax4", "cmin4", "cmax4", "cl_box6", "ob_box6", "ob_fmin4",
                                 "ob_fmax4", "vmask", "tv_cand", "tv_num", "dx_fix", "nc", "status", "queue")] + \
               [(n, F) for n in ("padding", "dt", "gx", "gy", "gz", "k_spring", "k_bend", "dHat", "compliance",
                                 "damping")]


# name -> (argtypes, restype)
SIGNATURES = {
    "sx_version": ([], I),
    "sx_last_error": ([], C.c_char_p),
    "sx_kernel_launches": ([], C.c_longlong),
    "sx_predict": ([P, P, P, P, I, F, F, F, F, P], I),
    "sx_jacobi_sweep": ([P, P, P, P, P, P, I, F, F, I, P], I),
    "sx_jacobi_sweep_variants": ([], I),
    "sx_jacobi_sweep_variant_info": ([I, P, P], I),
    "sx_jacobi_sweep_variant_form": ([I, P, P], I),
    "sx_set_programmatic_launch": ([I], I),
    "sx_jacobi_sweep_v": ([P, P, P, P, P, P, I, F, F, I, I, P], I),
    "sx_jacobi_sweep_mode": ([P, P, P, P, P, P, I, F, F, I, I, I, P], I),
    "sx_velocity_update": ([P, P, P, P, I, F, F, P], I),
    "sx_compute_velocity": ([P, P, P, P, I, F, F, P], I),
    "sx_update_x": ([P, P, I, F, P], I),
    "sx_velocity_contacts": ([I, I, P, P, I, P, P, P, P, P, P, P, P, P, F, P, P, P, P], I),
    "sx_sewing_sweep": ([P, P, I, P, P, P, F, P, P], I),
    "sx_residual_workspace_bytes": ([I], Z),
    "sx_energy_workspace_bytes": ([I], Z),
    "sx_system_energy": ([P, P, P, P, P, I, F, F, F, F, F, P, P, Z, P], I),
    "sx_constraint_residual": ([P, P, P, I, P, P, Z, P], I),
    "sx_convergence_begin": ([P, I, I, P], I),
    "sx_jacobi_sweep_checked": ([P, P, P, P, P, P, I, F, F, I, I, C.c_double, P, P, P, P, Z, C.c_ulonglong, I, P], I),
    "sx_jacobi_sweep_checked_mode": ([P, P, P, P, P, P, I, F, F, I, I, C.c_double, P, P, P, P, Z, C.c_ulonglong, I,
                                      I, P], I),
    "sx_loop_begin": ([P, P, P, P], I),
    "sx_loop_end": ([P], I),
    "sx_face_aabbs": ([P, P, I, F, P, P, P], I),
    "sx_face_aabbs_chunked": ([P, P, I, F, P, P, P, P, P], I),
    "sx_scene_aabb": ([P, I, F, P, P], I),
    "sx_cell_bvh_workspace_bytes": ([I], Z),
    "sx_cell_bvh_init": ([P, P, P, P, P, P, P, P, Z, P], I),
    "sx_cell_bvh_build": ([P, P, I, P, P, P, P, P, P, P, P, P, P, P, P, Z, P], I),
    "sx_cell_bvh_traverse": ([P, I, F, P, P, P, P, P, P, I, P, P, P, P], I),
    "sx_face_morton": ([P, P, I, P, P, P, P], I),
    "sx_radix_sort_workspace_bytes": ([I], Z),
    "sx_radix_sort_pairs": ([P, P, I, I, P, Z, P], I),
    "sx_radix_sort_pairs_noalloc": ([P, P, I, I, P], I),
    "sx_karras_build": ([P, I, I, P, P, P, P, P, P], I),
    "sx_face_bvh_refit": ([I, P, P, P, P, P, P, P, P, P, P, P], I),
    "sx_face_bvh_refit_tiled": ([I, P, P, P, P, P, P, P, P, P, P, P, P, P], I),
    "sx_face_bvh_traverse": ([I, P, I, F, P, P, P, P, P, I, P, P, P, P], I),
    "sx_face_bvh_traverse_ordered": ([I, P, I, F, P, P, P, P, P, I, P, P, P, P, P], I),
    "sx_collision_sweep": ([I, I, P, P, P, P, P, P, F, F, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P], I),
    "sx_contact_pairs_workspace_bytes": ([I, I], Z),
    "sx_contact_pairs_build": ([I, I, P, P, I, P, P, P, P, P, P, P, C.c_longlong, P, Z, P], I),
    "sx_contact_pairs_sweep": ([I, I, P, P, P, P, P, P, F, F, F, P, P, P, P, I, P], I),
    "sx_contact_pairs_project": ([I, I, P, P, P, P, P, P, F, F, F, P, P, P, P, I, P], I),
    "sx_contact_pairs_project_variants": ([], I),
    "sx_contact_pairs_project_variant_pipelined": ([I], I),
    "sx_contact_pairs_project_variant_info": ([I, P, P], I),
    "sx_contact_pairs_project_v": ([I, I, P, P, P, P, P, P, F, F, F, P, P, P, P, I, I, P], I),
    "sx_contact_apply": ([I, P, P, P, P, P, I, P], I),
    "sx_batched_substep_variants": ([], I),
    "sx_batched_substep_variant_cluster": ([I], I),
    "sx_batched_substep_variant_info": ([I, P, P], I),
    "sx_batched_substep": ([P, I, I, P], I),
    "sx_edge_edge_sweep": ([I, P, P, P, P, P, P, P, P, F, F, I, P, P, P, P, P, P, P, P, P, P, P, P, I, P], I),
    "sx_edge_edge_classify": ([I, P, F, P, P, P, P], I),
    "sx_cell_bvh_traverse_edges": ([P, I, P, F, P, P, P, P, P, P, I, P, P, P, P], I),
    "sx_segment_aabbs": ([P, P, I, F, P, P], I),
    "sx_batched_obstacle_broadphase": ([I, P, P, P, P, P, P, F, P, I, P, P, P, P, P, P, P, P, I, P, P, P, P], I),
    "sx_batched_obstacle_contacts": ([I, P, P, P, P, P, P, P, P, I, P, P, I, P, F, F, P, P, P, P, I, P], I),
    "sx_mlp_param_count": ([], I),
    "sx_mlp_bf16_count": ([], I),
    "sx_warm_features": ([P, P, P, P, P, P, P, I, F, F, F, F, P, P, P], I),
    "sx_mlp_forward": ([P, I, P, P, P, P], I),
    "sx_mlp_forward_tc": ([P, I, P, P, P, P, P], I),
    "sx_warm_apply": ([P, P, P, P, I, P, P], I),
    "sx_warm_select": ([P, P, P, P, I, P, P], I),
    "sx_warm_record": ([P, P, P, P, I, P, P, P], I),
    "sx_mlp_train_workspace_bytes": ([I], Z),
    "sx_mlp_gradients": ([P, P, P, I, I, P, P, P, P, P, Z, P], I),
    "sx_mlp_train_step": ([P, P, P, I, I, P, P, P, P, F, F, F, F, I, P, P, Z, P], I),
    "sx_mlp_sync_bf16": ([P, P, P], I),
    "sx_color_workspace_bytes": ([I, I], Z),
    "sx_color_edges_greedy": ([P, I, I, I, P, P, P, P, Z, P], I),
    "sx_jacobi_sweep_packed": ([P, P, P, P, P, P, P, I, F, F, I, I, P], I),
    "sx_jacobi_sweep_packed_v": ([P, P, P, P, P, P, P, I, F, F, I, I, I, P], I),
    "sx_jacobi_sweep_packed_forms": ([], I),
    "sx_gs_pack": ([P, P, I, P, P, I, P, P, P, P], I),
    "sx_gs_sweep": ([P, P, P, I, F, F, P], I),
}


class SxError(RuntimeError):
    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed with code {code}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library and bind signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build_library()
        if not os.path.exists(path):
            raise RuntimeError(f"starxpbd CUDA library missing: {path}")
        L = C.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def _call(name, *args):
    L = load()
    rc = getattr(L, name)(*args)
    if rc != SX_OK:
        raise SxError(name, rc, L.sx_last_error().decode(errors="replace"))
    return rc


def ptr(t) -> int | None:
    """Device pointer of a tensor (None for None)."""
    return None if t is None else t.data_ptr()


def stream_handle(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class _Calls:
    """Attribute access returns a checked caller: ``sx.sx_predict(...)``."""

    def __getattr__(self, name):
        if name not in SIGNATURES:
            raise AttributeError(name)
        if SIGNATURES[name][1] is I and name not in ("sx_version", "sx_mlp_param_count", "sx_mlp_bf16_count",
                                                     "sx_jacobi_sweep_variants", "sx_jacobi_sweep_packed_forms",
                                                     "sx_contact_pairs_project_variants",
                                                     "sx_contact_pairs_project_variant_pipelined",
                                                     "sx_batched_substep_variants",
                                                     "sx_batched_substep_variant_cluster"):
            return lambda *a: _call(name, *a)
        return getattr(load(), name)


sx = _Calls()
