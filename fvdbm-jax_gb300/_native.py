"""ctypes binding of libfvdbm.so (C ABI declared in include/fvdbm.h).

Loading never falls back to anything: if the library is missing or cannot be
loaded, ``lib()`` raises, so a GPU run can only ever go through the CUDA
kernels.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

FVDBM_UPWIND, FVDBM_LAX_WENDROFF = 0, 1
VARIANT_NONE, VARIANT_FACE_SCALE, VARIANT_FACE_Q_SCALE = 0, 1, 2
ORDER_NONE, ORDER_RCM, ORDER_MORTON = 0, 1, 2
KERNEL_AUTO, KERNEL_STAGED, KERNEL_FUSED, KERNEL_TILE, KERNEL_TILE_SPLIT, KERNEL_ONE = 0, 1, 2, 3, 4, 5
KERNEL_BATCH, KERNEL_FUSED_NODES, KERNEL_PERSIST, KERNEL_FAST = 6, 7, 8, 9

_i32p = C.POINTER(C.c_int32)
_f32p = C.POINTER(C.c_float)


class Mesh(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_nodes", C.c_int32),
        ("cell_face_stride", C.c_int32), ("node_cell_stride", C.c_int32),
        ("cell_face_indices", _i32p), ("cell_face_signs", _i32p),
        ("face_cells", _i32p), ("face_dists", _f32p), ("face_nodes", _i32p),
        ("face_n", _f32p), ("face_L", _f32p), ("face_scale", _f32p),
        ("node_type", _i32p), ("node_cells", _i32p), ("node_dists", _f32p),
        ("cell_xy", _f32p), ("cell_inv_area", _f32p), ("cell_area", _f32p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("flux_scheme", C.c_int32), ("variant", C.c_int32),
        ("inv_tau", C.c_float), ("delta_t", C.c_float),
        ("c2", C.c_float), ("c4x2", C.c_float), ("c2x2", C.c_float),
        ("ordering", C.c_int32), ("kernel", C.c_int32), ("device", C.c_int32),
        ("lattice", C.c_int32), ("c6x2", C.c_float),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_nodes", C.c_int32),
        ("n_bc_nodes", C.c_int32), ("n_ghost_faces", C.c_int32), ("kernel", C.c_int32),
        ("launches_per_step", C.c_int32), ("padded_cells", C.c_int32), ("ctas_per_sm", C.c_int32),
        ("const_division", C.c_int32),
        ("bytes_per_step", C.c_double), ("device_bytes", C.c_double),
    ]


_LIB = None
EXPORTS = ["fvdbm_create", "fvdbm_set_state", "fvdbm_step", "fvdbm_step_phase", "fvdbm_get_cells", "fvdbm_get_nodes",
           "fvdbm_get_face_fluxes", "fvdbm_sync", "fvdbm_stream", "fvdbm_get_info",
           "fvdbm_last_error", "fvdbm_destroy", "fvdbm_abi_version", "fvdbm_const_div_check", "fvdbm_const_div_check_form", "fvdbm_wait_selftest",
           "fvdbm_step_static_scratch", "fvdbm_residual", "fvdbm_run_to_steady",
           "fvdbm_batch_create", "fvdbm_batch_config", "fvdbm_batch_residual", "fvdbm_batch_set_active",
           "fvdbm_batch_run_to_steady", "fvdbm_set_cells_eq", "fvdbm_pack_cells", "fvdbm_unpack_cells",
           "fvdbm_batch_run_to_steady_time", "fvdbm_batch_residual_cases",
           "fvdbm_mp_dense_fwd", "fvdbm_mp_dense_bwd_data", "fvdbm_mp_wgrad_scratch", "fvdbm_mp_dense_bwd_weight",
           "fvdbm_mp_relu_bwd", "fvdbm_mp_spmm", "fvdbm_mp_mse_scratch", "fvdbm_mp_mse", "fvdbm_mp_adam",
           "fvdbm_mp_to_bf16", "fvdbm_mp_spmm_chunked", "fvdbm_pcg_work_bytes", "fvdbm_pcg",
           "fvdbm_ws_wall_distance", "fvdbm_ws_potential_rows", "fvdbm_ws_potential_grad", "fvdbm_ws_mesh_mean",
           "fvdbm_ws_bin_ids", "fvdbm_ws_bin_rows"]


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True) -> C.CDLL:
    """Load libfvdbm.so (building it first when the toolkit is present)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libfvdbm.so not found at {path}; run __graft_entry__.build()")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.fvdbm_create.argtypes = [C.POINTER(Mesh), C.POINTER(Params), C.POINTER(vp)]
    L.fvdbm_set_state.argtypes = [vp, _f32p, _f32p, _f32p, _f32p]
    L.fvdbm_step.argtypes = [vp, C.c_int32]
    L.fvdbm_step_phase.argtypes = [vp, C.c_int32]
    L.fvdbm_step_static_scratch.argtypes = [vp, C.c_int32]
    L.fvdbm_residual.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    _f64p, _i64p = C.POINTER(C.c_double), C.POINTER(C.c_int64)
    L.fvdbm_batch_create.argtypes = [C.POINTER(Mesh), C.POINTER(Params), C.c_int32, C.POINTER(vp)]
    L.fvdbm_batch_config.argtypes = [vp, C.c_int32, C.c_int32]
    L.fvdbm_batch_residual.argtypes = [vp, _f64p, _f64p]
    L.fvdbm_batch_residual_cases.argtypes = [vp, _i32p, _f64p, _f64p]
    L.fvdbm_batch_set_active.argtypes = [vp, _i32p]
    L.fvdbm_batch_run_to_steady.argtypes = [vp, C.c_double, C.c_int32, _i64p, _i64p, _f64p, _i32p]
    L.fvdbm_batch_run_to_steady_time.argtypes = [vp, C.c_double, C.c_int32, C.c_double, _i64p, _i64p, _f64p,
                                                 _i32p]
    L.fvdbm_set_cells_eq.argtypes = [vp, _f32p, _f32p]
    L.fvdbm_pack_cells.argtypes = [vp, _i32p, C.c_int32, C.c_void_p]
    L.fvdbm_unpack_cells.argtypes = [vp, _i32p, C.c_int32, C.c_void_p]
    # learned warm start (include/fvdbm_mpnn.h): device pointers as integers
    u64, i32, sz = C.c_uint64, C.c_int32, C.c_size_t
    L.fvdbm_mp_dense_fwd.argtypes = [u64, i32, u64, i32, i32, u64, u64, i32, i32, u64, u64, u64, u64]
    L.fvdbm_mp_dense_bwd_data.argtypes = [u64, i32, i32, u64, i32, i32, u64, i32, u64, u64]
    L.fvdbm_mp_wgrad_scratch.argtypes = [i32, i32, i32]
    L.fvdbm_mp_wgrad_scratch.restype = sz
    L.fvdbm_mp_dense_bwd_weight.argtypes = [u64, i32, i32, u64, i32, u64, i32, u64, u64, u64, sz, u64]
    L.fvdbm_mp_relu_bwd.argtypes = [u64, u64, u64, sz, u64]
    L.fvdbm_mp_spmm.argtypes = [u64, u64, u64, i32, u64, i32, u64, i32, u64]
    L.fvdbm_mp_spmm_chunked.argtypes = [u64, u64, i32, u64, u64, i32, u64, i32, u64, i32, u64, u64]
    L.fvdbm_mp_mse_scratch.argtypes = [sz]
    L.fvdbm_mp_mse_scratch.restype = sz
    L.fvdbm_mp_mse.argtypes = [u64, u64, u64, sz, C.c_float, u64, u64, sz, u64]
    L.fvdbm_mp_adam.argtypes = [u64, u64, u64, u64, u64, sz, C.c_float, C.c_float, C.c_float, C.c_float, i32, u64]
    L.fvdbm_mp_to_bf16.argtypes = [u64, u64, sz, u64]
    L.fvdbm_pcg_work_bytes.argtypes = [i32]
    L.fvdbm_pcg_work_bytes.restype = sz
    L.fvdbm_pcg.argtypes = [i32, u64, u64, u64, u64, u64, i32, C.c_double, i32, u64, sz, u64,
                            C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.fvdbm_ws_wall_distance.argtypes = [i32, u64, u64, i32, u64, u64, u64, u64]
    L.fvdbm_ws_potential_rows.argtypes = [i32, u64, u64, u64, u64, u64, u64, i32, u64, u64, u64, u64]
    L.fvdbm_ws_potential_grad.argtypes = [i32, u64, u64, u64, u64, u64, u64, u64, u64, u64, u64, u64, u64, u64]
    L.fvdbm_ws_mesh_mean.argtypes = [i32, u64, u64, i32, u64, u64, u64]
    dbl = C.c_double
    L.fvdbm_ws_bin_ids.argtypes = [i32, u64, dbl, dbl, dbl, dbl, i32, u64, u64, u64]
    L.fvdbm_ws_bin_rows.argtypes = [i32, i32, u64, u64, u64, i32, i32, u64, u64, u64, u64]
    L.fvdbm_run_to_steady.argtypes = [vp, C.c_double, C.c_int32, C.c_int64, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double)]
    L.fvdbm_get_cells.argtypes = [vp, _f32p, _f32p, _f32p, _f32p]
    L.fvdbm_get_nodes.argtypes = [vp, _f32p, _f32p, _f32p]
    L.fvdbm_get_face_fluxes.argtypes = [vp, _f32p]
    L.fvdbm_sync.argtypes = [vp]
    L.fvdbm_stream.argtypes = [vp]
    L.fvdbm_stream.restype = vp
    L.fvdbm_get_info.argtypes = [vp, C.POINTER(Info)]
    L.fvdbm_last_error.argtypes = [vp]
    L.fvdbm_last_error.restype = C.c_char_p
    L.fvdbm_destroy.argtypes = [vp]
    L.fvdbm_abi_version.restype = C.c_int
    L.fvdbm_const_div_check.argtypes = [C.c_int32, C.c_float, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    L.fvdbm_wait_selftest.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
    L.fvdbm_const_div_check_form.argtypes = [C.c_int32, C.c_float, C.c_int32, C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_uint32)]
    for name in EXPORTS:
        getattr(L, name)
    if L.fvdbm_abi_version() != 4:
        raise RuntimeError("libfvdbm ABI version mismatch")
    _LIB = L
    return L


def fptr(a):
    return None if a is None else a.ctypes.data_as(_f32p)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_i32p)


class FvdbmError(RuntimeError):
    pass


class NonFiniteError(FvdbmError, FloatingPointError):
    """The state turned non-finite (``FVDBM_ENONFINITE``): the run diverged."""


ENONFINITE = -5
# per-case outcome of fvdbm_batch_run_to_steady
CASE_CAPPED, CASE_CONVERGED, CASE_NONFINITE, CASE_FROZEN, CASE_STALLED = 0, 1, 2, 3, 4


def check(rc: int, handle=None):
    if rc != 0:
        msg = lib().fvdbm_last_error(handle)
        cls = NonFiniteError if rc == ENONFINITE else FvdbmError
        raise cls(f"libfvdbm error {rc}: {msg.decode() if msg else ''}")


def c_contig(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)
