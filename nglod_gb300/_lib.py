"""ctypes binding of the C ABI in include/nglod_gb300.h.

The library is loaded from nglod_gb300/_build/libnglod_gb300.so (built by
``nglod_gb300.build``).  There is no fallback: if it is missing, or a call is
made with CPU tensors, a RuntimeError is raised.
"""
import ctypes
import os

import torch

from . import build as _build

MAX_LODS = 8
F32 = 0
BF16 = 1

STATUS = {
    0: "ok",
    -1: "invalid argument",
    -2: "unsupported configuration",
    -3: "CUDA error",
    -4: "capacity exceeded",
    -5: "misaligned pointer",
    -6: "device wait timed out",
}

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32


class DenseModel(ctypes.Structure):
    _fields_ = [
        ("num_lods", _i32),
        ("base_lod", _i32),
        ("feature_dim", _i32),
        ("hidden_dim", _i32),
        ("grid_dtype", _i32),
        ("reserved", _i32),
        ("grid", _vp * MAX_LODS),
        ("w0", _vp * MAX_LODS),
        ("b0", _vp * MAX_LODS),
        ("w1", _vp * MAX_LODS),
        ("b1", _vp * MAX_LODS),
    ]


class TraceParams(ctypes.Structure):
    _fields_ = [
        ("num_steps", _i32),
        ("min_dis", ctypes.c_float),
        ("osc_dis", ctypes.c_float),
        ("step_size", ctypes.c_float),
        ("far_clip", ctypes.c_float),
        ("lod", _i32),
        ("want_normals", _i32),
    ]


class DenseGrads(ctypes.Structure):
    _fields_ = [
        ("grid", _vp * MAX_LODS),
        ("w0", _vp * MAX_LODS),
        ("b0", _vp * MAX_LODS),
        ("w1", _vp * MAX_LODS),
        ("b1", _vp * MAX_LODS),
    ]


class AdamTensor(ctypes.Structure):
    _fields_ = [("param", _vp), ("grad", _vp), ("exp_avg", _vp), ("exp_avg_sq", _vp), ("numel", _i64)]


class SparseModel(ctypes.Structure):
    _fields_ = [
        ("num_lods", _i32),
        ("feature_dim", _i32),
        ("hidden_dim", _i32),
        ("feat_dtype", _i32),
        ("corner_feats", _vp),
        ("corner_idx", _vp),
        ("parent", _vp),
        ("points", _vp),
        ("level_start", _i64 * 16),
        ("w0", _vp * MAX_LODS),
        ("b0", _vp * MAX_LODS),
        ("w1", _vp * MAX_LODS),
        ("b1", _vp * MAX_LODS),
        ("w0_tile", _vp * MAX_LODS),
        ("corner_chain", _vp * MAX_LODS),
        ("summed", _i32),
    ]


class Bf16Model(ctypes.Structure):
    _fields_ = [
        ("num_lods", _i32),
        ("base_lod", _i32),
        ("feature_dim", _i32),
        ("hidden_dim", _i32),
        ("grid", _vp * MAX_LODS),
        ("w0_tile", _vp * MAX_LODS),
        ("b0", _vp * MAX_LODS),
        ("w1", _vp * MAX_LODS),
        ("b1", _vp * MAX_LODS),
        ("grid_pairs", _vp * MAX_LODS),
        ("summed", _i32),
    ]


BF16_TILE_BYTES = 12288

SERVE_RENDER = 1
SERVE_QUERY = 2


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", _i64), ("num_slots", _i32), ("reserved", _i32)]


class ServeRequest(ctypes.Structure):
    _fields_ = [
        ("kind", _i32),
        ("model", _i32),
        ("lod", _i32),
        ("width", _i32),
        ("height", _i32),
        ("eye", ctypes.c_float * 3),
        ("at", ctypes.c_float * 3),
        ("up", ctypes.c_float * 3),
        ("fov_deg", ctypes.c_float),
        ("trace", TraceParams),
        ("points", _vp),
        ("n", _i64),
        ("has_ready_stream", _i32),
        ("reserved", _i32),
        ("ready_stream", _vp),
    ]


class ServeResult(ctypes.Structure):
    _fields_ = [
        ("ticket", _i64),
        ("kind", _i32),
        ("status", _i32),
        ("t_submit", ctypes.c_double),
        ("t_admit", ctypes.c_double),
        ("t_done", ctypes.c_double),
        ("units", _i64),
        ("x", _vp),
        ("t", _vp),
        ("hit", _vp),
        ("normal", _vp),
        ("sdf", _vp),
    ]


class ServeInfo(ctypes.Structure):
    _fields_ = [
        ("budget_bytes", _i64),
        ("used_bytes", _i64),
        ("peak_used_bytes", _i64),
        ("num_slots", _i32),
        ("pending", _i32),
        ("running", _i32),
        ("unpolled", _i32),
        ("held", _i32),
        ("max_concurrent", _i32),
        ("submitted", _i64),
        ("completed", _i64),
    ]


SERVE_LAUNCH_FN = ctypes.CFUNCTYPE(_i32, _vp, _i64, _i32, ctypes.POINTER(ServeRequest), _i64, _i64)
SERVE_QUERY_FN = ctypes.CFUNCTYPE(_i32, _vp, _i64, _i32)


class ServeExecutor(ctypes.Structure):
    _fields_ = [("ctx", _vp), ("launch", SERVE_LAUNCH_FN), ("query", SERVE_QUERY_FN)]


# C struct name -> ctypes mirror (layouts are checked against the header by tests/test_abi.py)
STRUCTS = {"nglod_dense_grads": DenseGrads, "nglod_adam_tensor": AdamTensor, "nglod_sparse_model": SparseModel,
           "nglod_bf16_model": Bf16Model, "nglod_serve_config": ServeConfig, "nglod_serve_request": ServeRequest,
           "nglod_serve_result": ServeResult, "nglod_serve_info": ServeInfo,
           "nglod_serve_executor": ServeExecutor}

_u32 = ctypes.c_uint32
_f32 = ctypes.c_float

# name -> (restype, argtypes)
SIGNATURES = {
    "nglod_version": (ctypes.c_char_p, []),
    "nglod_last_error": (ctypes.c_char_p, []),
    "nglod_aabb": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "nglod_volume_sample": (ctypes.c_int, [_vp, _i32, _i32, _vp, _i64, _vp, _vp]),
    "nglod_sdf_fwd": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _i32, _i32, _vp, _vp]),
    "nglod_sdf_fwd_simt": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _i32, _i32, _vp, _vp]),
    "nglod_dense_status": (ctypes.c_int, [_vp]),
    "nglod_trace": (ctypes.c_int, [ctypes.POINTER(DenseModel), ctypes.POINTER(TraceParams), _vp, _vp, _i64,
                                   _vp, _vp, _vp, _vp, _vp, _vp]),
    "nglod_sdf_fwd_train": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _u32, _vp, _vp, _vp, _vp]),
    "nglod_train_status": (ctypes.c_int, [ctypes.POINTER(_i32)]),
    "nglod_l2_loss": (ctypes.c_int, [_vp, _vp, _i64, _i32, _u32, _vp, _vp, _vp]),
    "nglod_sdf_bwd": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _u32, _vp, _vp, _vp, _vp,
                                     ctypes.POINTER(DenseGrads), _vp, _vp]),
    "nglod_sdf_bwd_noalloc": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _u32, _vp, _vp, _vp,
                                             ctypes.POINTER(DenseGrads), _vp, _vp]),
    "nglod_spc_build_scratch_bytes": (_i64, [_i32]),
    "nglod_spc_build": (ctypes.c_int, [_vp, _i64, _i32, _vp, _i64, ctypes.POINTER(_i64), _vp, _vp, _vp]),
    "nglod_spc_decode": (ctypes.c_int, [_vp, _i64, _vp, _i64, _vp, _vp, ctypes.POINTER(_i32), _vp]),
    "nglod_spc_prefix": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _vp]),
    "nglod_spc_raytrace": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _i64, _vp, _vp, _i64, _vp,
                                          _vp, _vp, ctypes.POINTER(_i64), ctypes.POINTER(_i32), _vp]),
    "nglod_spc_mark_first": (ctypes.c_int, [_vp, _i64, _vp, _vp]),
    "nglod_voxel_centres": (ctypes.c_int, [_i32, _i64, _i64, _vp, _vp]),
    "nglod_select_band": (ctypes.c_int, [_vp, _i64, _f32, _i32, _i64, _vp, _i64, _i64, _vp, _vp,
                                         ctypes.POINTER(_i64), _vp]),
    "nglod_spc_generate_rays": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "nglod_sparse_build_scratch_bytes": (_i64, [_i32]),
    "nglod_sparse_build": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _vp, _i32, _i32, _vp, _i64, _vp, _vp,
                                          _vp, _vp, _vp]),
    "nglod_sparse_query": (ctypes.c_int, [ctypes.POINTER(SparseModel), _vp, _vp, _i32, _vp, _i64, _vp, _vp]),
    "nglod_sparse_trace": (ctypes.c_int, [ctypes.POINTER(SparseModel), _i32, _i32, _vp, _vp, _i64, _vp, _i64, _vp,
                                          _vp, _vp, _vp, _vp, _vp, _vp]),
    "nglod_sparse_build_chain": (ctypes.c_int, [ctypes.POINTER(SparseModel), _i32, _i64, _vp, _vp]),
    "nglod_sparse_trace_tc": (ctypes.c_int, [ctypes.POINTER(SparseModel), _i32, _i32, _vp, _vp, _i64, _vp, _i64,
                                             _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nglod_bf16_pack_decoder": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp]),
    "nglod_bf16_build_pairs": (ctypes.c_int, [_vp, _i32, _vp, _vp]),
    "nglod_build_summed_volume": (ctypes.c_int, [ctypes.POINTER(DenseModel), _i32, _i32, _vp, _vp]),
    "nglod_measure_line_reads": (ctypes.c_int, [_vp, _i64, _i32, _i32, _vp, _vp]),
    "nglod_measure_fma": (ctypes.c_int, [_i32, _i32, _vp, _vp]),
    "nglod_measure_smem_reads": (ctypes.c_int, [_i32, _i32, _vp, _vp]),
    "nglod_debug_mma_wait_polls": (ctypes.c_int, [_i64]),
    "nglod_sdf_fwd_bf16": (ctypes.c_int, [ctypes.POINTER(Bf16Model), _vp, _i64, _i32, _vp, _vp, _vp]),
    "nglod_trace_bf16": (ctypes.c_int, [ctypes.POINTER(Bf16Model), ctypes.POINTER(TraceParams), _vp, _vp, _i64,
                                        _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nglod_camera_rays": (ctypes.c_int, [_vp, _vp, _vp, _f32, _i32, _i32, _vp, _vp, _vp]),
    "nglod_adam_step": (ctypes.c_int, [_vp, _i32, _i64, _f32, _f32, _f32, _f32, _f32, _i64, _vp]),
    "nglod_host_query_scratch_bytes": (_i64, [_i64]),
    "nglod_sdf_fwd_host": (ctypes.c_int, [ctypes.POINTER(DenseModel), _vp, _i64, _i32, _vp, _i64, _vp, _vp]),
    "nglod_sdf_fwd_bf16_host": (ctypes.c_int, [ctypes.POINTER(Bf16Model), _vp, _i64, _i32, _vp, _i64, _vp, _vp,
                                               _vp]),
    "nglod_mesh_record_floats": (_i64, []),
    "nglod_mesh_prepare": (ctypes.c_int, [_vp, _i64, _vp, _vp]),
    "nglod_mesh_sdf": (ctypes.c_int, [_vp, _i64, _vp, _i64, _vp, _vp]),
    "nglod_shade_min_hit_y": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    "nglod_shade_ground": (ctypes.c_int, [_vp, _vp, _i64, _f32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nglod_shade_shadow_rays": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    "nglod_shade_ao_select": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, ctypes.POINTER(_i64), _vp]),
    "nglod_shade_ao_taps": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _vp]),
    "nglod_shade_ao_reduce": (ctypes.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _vp]),
    "nglod_shade_matcap": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _i32, _i32, _vp, _vp]),
    "nglod_shade_shadow_map": (ctypes.c_int, [_vp, _vp, _i32, _i32, _f32, _vp, _vp, _vp, _vp]),
    "nglod_shade_compose": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _f32, _vp, _vp]),
    "nglod_serve_request_bytes": (_i64, [ctypes.POINTER(ServeRequest)]),
    "nglod_serve_start": (ctypes.c_int, [ctypes.POINTER(ServeConfig), ctypes.POINTER(_vp)]),
    "nglod_serve_start_custom": (ctypes.c_int, [ctypes.POINTER(ServeConfig), ctypes.POINTER(ServeExecutor),
                                                ctypes.POINTER(_vp)]),
    "nglod_serve_add_model_f32": (ctypes.c_int, [_vp, ctypes.POINTER(DenseModel), ctypes.POINTER(_i32)]),
    "nglod_serve_add_model_bf16": (ctypes.c_int, [_vp, ctypes.POINTER(Bf16Model), ctypes.POINTER(_i32)]),
    "nglod_serve_submit": (ctypes.c_int, [_vp, ctypes.POINTER(ServeRequest), ctypes.c_double, ctypes.POINTER(_i64)]),
    "nglod_serve_poll": (ctypes.c_int, [_vp, ctypes.POINTER(ServeResult), _i32, ctypes.POINTER(_i32)]),
    "nglod_serve_release": (ctypes.c_int, [_vp, _i64, _i32, _vp]),
    "nglod_serve_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(ServeInfo)]),
    "nglod_serve_stop": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "nglod_serve_destroy": (ctypes.c_int, [_vp]),
}

_LIB = None


def load():
    """Load the library once and declare every signature; raises if absent."""
    global _LIB
    if _LIB is None:
        path = _build.library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"nglod_gb300 CUDA library not found at {path}; build it with "
                "`python -m nglod_gb300.build` (there is no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def check(status, what):
    if status != 0:
        msg = load().nglod_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed ({STATUS.get(status, status)}): {msg}")


def stream_ptr(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def require_cuda(*tensors):
    for t in tensors:
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise RuntimeError("nglod_gb300 runs on CUDA tensors only (no CPU fallback)")
