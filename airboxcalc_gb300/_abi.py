"""ctypes binding of libairbox.so (include/airbox.h).

The library is built in-tree by ``airboxcalc_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for any compute call.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libairbox.so")

# status codes (abx_status)
OK = 0
ERR_NO_TRIANGLES, ERR_SAME_AXIS, ERR_GRID_TOO_LARGE, ERR_NO_OPENING, ERR_OPENING_TOO_SMALL = 1, 2, 3, 4, 5
ERR_SEAL_OUTSIDE, ERR_LEAK, ERR_LID_TOO_LOW, ERR_BAD_OUTLET, ERR_UNSTABLE = 6, 7, 8, 9, 10
ERR_NOT_PREPARED, ERR_CANCELLED = 11, 12
ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY = 20, 21, 22

STORAGE = {"f32": 0, "f32exact": 1, "f16": 2, "bf16": 3, "f64": 4}

# Every symbol include/airbox.h declares.
ABI_VERSION = 3  # include/airbox.h ABX_ABI_VERSION: the structures below follow that version
MAX_LINE_POINTS = 2001  # include/airbox.h ABX_MAX_LINE_POINTS

EXPORTS = [
    "abx_last_error", "abx_abi_version", "abx_device_count", "abx_parse_stl", "abx_prepare", "abx_geom_free",
    "abx_geom_get_info", "abx_geom_get_masks", "abx_geom_get_fine", "abx_sim_create", "abx_sim_free",
    "abx_sim_get_info", "abx_sim_reset", "abx_sim_step", "abx_sim_run", "abx_sim_get_f", "abx_sim_set_f",
    "abx_sim_get_acc", "abx_sim_clear_acc", "abx_sim_evaluate", "abx_simulate", "abx_sim_set_timing", "abx_sim_get_timing",
    "abx_voxelize_static",
    "abx_net_create", "abx_net_set_tensor_cores", "abx_net_free", "abx_net_get_info", "abx_net_get_weights", "abx_net_set_weights",
    "abx_net_add_sample", "abx_net_clear_samples", "abx_net_get_sample", "abx_net_train", "abx_net_eval_loss",
    "abx_net_forward_backward", "abx_net_predict", "abx_sim_warm_start", "abx_sim_converge", "abx_sim_solve_warm",
    "abx_batch_create", "abx_batch_free", "abx_batch_sim", "abx_batch_tune", "abx_batch_set_shape", "abx_batch_reset",
    "abx_batch_run", "abx_batch_get_info", "abx_batch_set_grouping", "abx_sim_field3d", "abx_sim_planes", "abx_sim_streamlines",
]


class PrepareParams(C.Structure):
    _fields_ = [("dx", C.c_double), ("seal_axis", C.c_int), ("seal_sign", C.c_double), ("seal", C.c_double),
                ("inlet_axis", C.c_int), ("inlet_sign", C.c_double), ("inlet_yaw", C.c_double),
                ("pleat", C.c_double), ("has_click", C.c_int), ("click", C.c_double * 3),
                ("has_outlet", C.c_int), ("outlet_center", C.c_double * 3), ("outlet_diameter", C.c_double),
                ("outlet_height", C.c_double), ("max_cells", C.c_double), ("device", C.c_int)]


class GeomInfo(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("N", C.c_int64), ("nf", C.c_int),
                ("top", C.c_int), ("jm", C.c_int), ("kw0", C.c_int), ("kf", C.c_int),
                ("n_holes", C.c_int), ("n_open", C.c_int), ("af", C.c_int), ("n_out", C.c_int),
                ("leak_cells", C.c_int), ("pleat_ok", C.c_int),
                ("h", C.c_double), ("origin", C.c_double * 3), ("mn", C.c_double * 3), ("mx", C.c_double * 3),
                ("pleat", C.c_double), ("volume_l", C.c_double), ("inlet_cm2", C.c_double),
                ("filter_cm2", C.c_double), ("outlet_cm2", C.c_double), ("outlet_cm2_real", C.c_double),
                ("frame_cy", C.c_double), ("frame_sy", C.c_double), ("kernel_launches", C.c_int64),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("ms_voxelize", C.c_double),
                ("ms_masks", C.c_double), ("ms_device", C.c_double)]


class RunParams(C.Structure):
    _fields_ = [("K", C.c_double), ("aniso", C.c_double), ("u", C.c_double), ("tau", C.c_double),
                ("steps", C.c_int), ("avg", C.c_int), ("every", C.c_int), ("storage", C.c_int),
                ("flags", C.c_uint)]


RUN_ALLOW_BF16 = 1  # include/airbox.h ABX_RUN_ALLOW_BF16


class SimInfo(C.Structure):
    _fields_ = [("NF", C.c_int), ("Ain", C.c_int), ("Af", C.c_int), ("Lp", C.c_int), ("n_layer_m", C.c_int),
                ("n_layer_t", C.c_int), ("u0", C.c_double), ("tau0", C.c_double), ("sig", C.c_double),
                ("aniso", C.c_double), ("cs2s", C.c_double), ("uface", C.c_double), ("step", C.c_int),
                ("nacc", C.c_int), ("Np", C.c_int64), ("state_bytes", C.c_int64), ("tma_pipeline", C.c_int),
                ("vec_width", C.c_int), ("vec_interior_cells", C.c_int64)]


class Progress(C.Structure):
    _fields_ = [("step", C.c_int), ("steps", C.c_int), ("gamma", C.c_double), ("mass_ratio", C.c_double),
                ("elapsed_s", C.c_double), ("eta_s", C.c_double), ("mlups", C.c_double)]


PROGRESS_FN = C.CFUNCTYPE(C.c_int, C.POINTER(Progress), C.c_void_p)


class Metrics(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean",
                                          "zeta", "inlet_cm2", "filter_cm2", "wm", "cm")] + \
               [(k, C.c_int) for k in ("n", "cn", "pinN", "pbN", "jb")]


class Timing(C.Structure):
    _fields_ = [("step_ms", C.c_double), ("step_launches", C.c_int64), ("step_ms_plain", C.c_double),
                ("step_launches_plain", C.c_int64), ("run_ms", C.c_double), ("eval_ms", C.c_double),
                ("cell_updates", C.c_int64), ("kernel_launches", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64)]


class NetParams(C.Structure):
    _fields_ = [("res", C.c_int), ("base", C.c_int), ("levels", C.c_int), ("device", C.c_int),
                ("seed", C.c_ulonglong), ("coords", C.c_int)]


class NetInfo(C.Structure):
    _fields_ = [("res", C.c_int), ("base", C.c_int), ("levels", C.c_int), ("in_channels", C.c_int),
                ("out_channels", C.c_int), ("n_samples", C.c_int), ("n_params", C.c_longlong),
                ("tensor_cores", C.c_int)]


class TrainParams(C.Structure):
    _fields_ = [("first", C.c_int), ("count", C.c_int), ("epochs", C.c_int), ("batch", C.c_int),
                ("lr", C.c_double), ("lr_min", C.c_double), ("seed", C.c_ulonglong), ("flip", C.c_int)]


RULE_CHANGE, RULE_STDERR = 0, 1  # include/airbox.h ABX_RULE_*


class ConvergeParams(C.Structure):
    _fields_ = [("settle", C.c_int), ("window", C.c_int), ("min_avg", C.c_int), ("max_steps", C.c_int),
                ("tol", C.c_double), ("rule", C.c_int), ("min_windows", C.c_int)]


class ConvergeResult(C.Structure):
    _fields_ = [("metrics", Metrics), ("steps", C.c_int), ("windows", C.c_int), ("converged", C.c_int),
                ("change", C.c_double)]


class WarmResult(C.Structure):
    _fields_ = [("run", ConvergeResult), ("fell_back", C.c_int), ("warm_steps", C.c_int), ("infer_ms", C.c_double),
                ("total_ms", C.c_double)]


class Field3DInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("nx", "ny", "nz", "kB", "jm", "top")] + \
               [(k, C.c_double) for k in ("h", "x0", "d0", "z0", "zIn", "pleat", "pin", "rho_ref")]


class PlanesInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("ic", "jc", "jlow", "n1", "n2", "lon_n1", "lon_n2")] + \
               [(k, C.c_double) for k in ("depth_inlet", "depth_low", "x_lon")]


class LinesInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("seeds_opening", "seeds_traced", "n_lines", "n_points")]


class BatchTuning(C.Structure):
    _fields_ = [("shape", C.c_int), ("spw", C.c_int), ("min_blocks", C.c_int), ("grid", C.c_uint),
                ("ntiles", C.c_uint), ("ms_per_step", C.c_double), ("group_bytes", C.c_double),
                ("n_groups", C.c_int), ("n_candidates", C.c_int),
                ("cand_shape", C.c_int * 48), ("cand_grid", C.c_uint * 48), ("cand_group_bytes", C.c_double * 48),
                ("cand_groups", C.c_int * 48), ("cand_ms", C.c_double * 48)]


class BatchInfo(C.Structure):
    _fields_ = [("n", C.c_int), ("cells", C.c_longlong), ("state_bytes", C.c_longlong), ("ntiles1", C.c_uint),
                ("ntiles2", C.c_uint), ("shape", C.c_int), ("grid", C.c_uint), ("run_ms", C.c_double),
                ("kernel_launches", C.c_longlong), ("n_groups", C.c_int), ("group_bytes", C.c_double)]


_lib = None


def load(build_if_missing: bool = True):
    """Load libairbox.so (building it first when it is missing or stale).

    ABX_LIBRARY, when set, names another build of the library to load."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("ABX_LIBRARY", LIB_PATH)
    if build_if_missing and path == LIB_PATH:
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run airboxcalc_gb300.build.build() (needs nvcc)")
    L = C.CDLL(path)
    if L.abx_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path} implements ABI {L.abx_abi_version()}, these bindings ABI {ABI_VERSION}: rebuild it")
    vp = C.c_void_p
    L.abx_last_error.restype = C.c_char_p
    L.abx_parse_stl.argtypes = [C.c_char_p, C.c_size_t, vp, C.c_size_t, C.POINTER(C.c_size_t)]
    L.abx_prepare.argtypes = [vp, C.c_size_t, C.POINTER(PrepareParams), C.POINTER(vp)]
    L.abx_geom_free.argtypes = [vp]
    L.abx_geom_free.restype = None
    L.abx_geom_get_info.argtypes = [vp, C.POINTER(GeomInfo)]
    L.abx_geom_get_masks.argtypes = [vp] + [vp] * 7
    L.abx_geom_get_fine.argtypes = [vp, vp, C.c_size_t]
    L.abx_sim_create.argtypes = [vp, C.POINTER(RunParams), vp, C.POINTER(vp)]
    L.abx_sim_free.argtypes = [vp]
    L.abx_sim_free.restype = None
    L.abx_sim_get_info.argtypes = [vp, C.POINTER(SimInfo)]
    L.abx_sim_reset.argtypes = [vp]
    L.abx_sim_step.argtypes = [vp, C.c_int, C.c_int]
    L.abx_sim_run.argtypes = [vp, PROGRESS_FN, vp]
    L.abx_sim_get_f.argtypes = [vp, vp]
    L.abx_sim_set_f.argtypes = [vp, vp]
    L.abx_sim_get_acc.argtypes = [vp, vp]
    L.abx_sim_clear_acc.argtypes = [vp]
    L.abx_sim_evaluate.argtypes = [vp, C.POINTER(Metrics), vp, vp, C.c_int, C.POINTER(C.c_int)]
    L.abx_simulate.argtypes = [vp, C.POINTER(RunParams), vp, PROGRESS_FN, vp, C.POINTER(Metrics), vp, vp,
                               C.c_int, C.POINTER(C.c_int)]
    L.abx_sim_set_timing.argtypes = [vp, C.c_int]
    L.abx_sim_get_timing.argtypes = [vp, C.POINTER(Timing)]
    L.abx_voxelize_static.argtypes = [vp, C.c_size_t, C.c_double * 3, C.c_double, C.c_int, C.c_int, C.c_int, vp, vp]
    L.abx_net_create.argtypes = [C.POINTER(NetParams), C.POINTER(vp)]
    L.abx_net_free.argtypes = [vp]
    L.abx_net_free.restype = None
    L.abx_net_get_info.argtypes = [vp, C.POINTER(NetInfo)]
    L.abx_net_get_weights.argtypes = [vp, vp]
    L.abx_net_set_weights.argtypes = [vp, vp]
    L.abx_net_add_sample.argtypes = [vp, vp]
    L.abx_net_clear_samples.argtypes = [vp]
    L.abx_net_get_sample.argtypes = [vp, C.c_int, vp, vp, vp]
    L.abx_net_train.argtypes = [vp, C.POINTER(TrainParams), vp]
    L.abx_net_eval_loss.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.abx_net_forward_backward.argtypes = [vp, vp, vp, vp, C.c_int, C.c_double, vp, vp, C.POINTER(C.c_double)]
    L.abx_net_predict.argtypes = [vp, vp, vp, vp]
    L.abx_sim_warm_start.argtypes = [vp, vp]
    L.abx_sim_converge.argtypes = [vp, C.POINTER(ConvergeParams), C.POINTER(ConvergeResult)]
    L.abx_sim_solve_warm.argtypes = [vp, vp, C.POINTER(ConvergeParams), C.POINTER(WarmResult)]
    L.abx_sim_field3d.argtypes = [vp, vp, vp, vp, C.POINTER(Field3DInfo)]
    L.abx_sim_planes.argtypes = [vp, vp, C.POINTER(PlanesInfo)]
    L.abx_sim_streamlines.argtypes = [vp, C.c_int, vp, vp, vp, C.c_size_t, C.c_size_t, C.POINTER(LinesInfo)]
    L.abx_batch_create.argtypes = [C.POINTER(vp), C.POINTER(RunParams), C.c_int, C.POINTER(vp)]
    L.abx_batch_free.argtypes = [vp]
    L.abx_batch_free.restype = None
    L.abx_batch_sim.argtypes = [vp, C.c_int, C.POINTER(vp)]
    L.abx_batch_tune.argtypes = [vp, C.POINTER(BatchTuning)]
    L.abx_batch_set_shape.argtypes = [vp, C.c_int, C.c_uint]
    L.abx_batch_set_grouping.argtypes = [vp, C.c_double]
    L.abx_batch_reset.argtypes = [vp]
    L.abx_batch_run.argtypes = [vp, vp]
    L.abx_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    _lib = L
    return L


def last_error() -> str:
    return load().abx_last_error().decode("utf-8", "replace")
