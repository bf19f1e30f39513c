"""ctypes binding of librmg_gb300.so (the C ABI declared in include/rmg.h).

The shared library is the only compute path of this package: when it is
missing, loading raises RmgError instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "librmg_gb300.so"


class RmgError(RuntimeError):
    """A non-zero rmg_status, raised like rmagine raises CudaException via RM_THROW."""

    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        super().__init__(f"{where}: status {status} ({message})")


# ---- status codes (include/rmg.h) -----------------------------------------
RMG_OK = 0
RMG_ERR_INVALID_ARG = 1
RMG_ERR_CUDA = 2
RMG_ERR_OOM = 3
RMG_ERR_TIMEOUT = 4
RMG_ERR_TRAVERSAL_BUDGET = 5
RMG_ERR_NO_DEVICE = 6
RMG_ERR_UNSUPPORTED = 7
RMG_BUILD_SAH = 0
RMG_BUILD_LBVH = 1

RMG_MODEL_SPHERICAL = 0
RMG_MODEL_PINHOLE = 1
RMG_MODEL_O1DN = 2
RMG_MODEL_ONDN = 3


# ---- structs ---------------------------------------------------------------
class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Quat(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class TransformC(C.Structure):
    _fields_ = [("R", Quat), ("t", Vec3), ("stamp", C.c_uint32)]


class Interval(C.Structure):
    _fields_ = [("min", C.c_float), ("max", C.c_float)]


class DiscreteInterval(C.Structure):
    _fields_ = [("min", C.c_float), ("inc", C.c_float), ("size", C.c_uint32)]


class ModelC(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("range", Interval),
        ("phi", DiscreteInterval),
        ("theta", DiscreteInterval),
        ("f", C.c_float * 2),
        ("c", C.c_float * 2),
        ("orig", Vec3),
        ("dirs", C.c_void_p),
        ("origs", C.c_void_p),
    ]


class OutputsC(C.Structure):
    _fields_ = [
        ("hits", C.c_void_p),
        ("ranges", C.c_void_p),
        ("points", C.c_void_p),
        ("normals", C.c_void_p),
        ("face_ids", C.c_void_p),
        ("geom_ids", C.c_void_p),
        ("object_ids", C.c_void_p),
    ]


class LaunchConfigC(C.Structure):
    _fields_ = [("stack_depth", C.c_uint32), ("block_warps", C.c_uint32), ("tile_w", C.c_uint32),
                ("tile_h", C.c_uint32), ("refill", C.c_uint32), ("chunk", C.c_uint32), ("bvh_width", C.c_uint32),
                ("packet", C.c_uint32)]


class MapInfoC(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_uint32),
        ("n_faces", C.c_uint32),
        ("n_nodes", C.c_uint32),
        ("depth", C.c_uint32),
        ("device_bytes", C.c_uint64),
        ("bounds_lo", C.c_float * 3),
        ("bounds_hi", C.c_float * 3),
    ]


class LbvhBuffersC(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("tris", C.c_void_p), ("leaf_order", C.c_void_p),
                ("leaf_parent", C.c_void_p), ("flags", C.c_void_p)]


class BatchEntryC(C.Structure):
    _fields_ = [("sensor", C.c_void_p), ("Tsb", TransformC), ("Tbm", C.c_void_p), ("n_poses", C.c_uint32),
                ("out", OutputsC)]


class BatchConfigC(C.Structure):
    _fields_ = [("stack_depth", C.c_uint32), ("block_warps", C.c_uint32), ("tile_w", C.c_uint32),
                ("tile_h", C.c_uint32), ("grab", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("use_graph", C.c_uint32)]


class ConstraintsC(C.Structure):
    _fields_ = [("max_dist", C.c_float), ("dataset_id", C.c_uint32), ("model_id", C.c_uint32)]


class InstanceDescC(C.Structure):
    _fields_ = [("geometry", C.c_uint32), ("geom_id", C.c_uint32), ("object_id", C.c_uint32), ("T", TransformC),
                ("scale", C.c_float * 3)]


class NoiseC(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("mean", C.c_float), ("stddev", C.c_float), ("range_exp", C.c_float),
                ("hit_probability", C.c_float), ("return_probability", C.c_float), ("max_range", C.c_float),
                ("seed", C.c_uint64), ("call", C.c_uint64)]


RMG_NOISE_GAUSSIAN, RMG_NOISE_REL_GAUSSIAN, RMG_NOISE_UNIFORM_DUST = 0, 1, 2


class MeshC(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_uint32), ("faces", C.c_void_p), ("n_faces", C.c_uint32),
                ("face_group", C.c_void_p), ("n_groups", C.c_uint32)]


class ScanC(C.Structure):
    _fields_ = [("points", C.c_void_p), ("mask", C.c_void_p), ("ids", C.c_void_p), ("per_pose", C.c_uint32)]


RMG_NOALLOC_MAX_FACES = 65536

# name -> (restype, argtypes); every symbol include/rmg.h declares
_P = C.c_void_p
_U32 = C.c_uint32
SIGNATURES: dict[str, tuple] = {
    "rmg_status_string": (C.c_char_p, [C.c_int]),
    "rmg_last_error": (C.c_char_p, []),
    "rmg_abi_version": (C.c_int, []),
    "rmg_device_info": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rmg_stream_wait": (C.c_int, [_P, _U32]),
    "rmg_map_build": (C.c_int, [_P, _U32, _P, _U32, _P, C.POINTER(_P)]),
    "rmg_map_build_ex": (C.c_int, [_P, _U32, _P, _U32, _U32, _P, C.POINTER(_P)]),
    "rmg_map_refit": (C.c_int, [_P, _P, _U32, _P]),
    "rmg_map_destroy": (C.c_int, [_P]),
    "rmg_map_info_get": (C.c_int, [_P, C.POINTER(MapInfoC)]),
    "rmg_map_export": (C.c_int, [_P, _P, _P, _P]),
    "rmg_map_status": (C.c_int, [_P, C.c_int]),
    "rmg_map_debug_set_child": (C.c_int, [_P, _U32, _U32, C.c_int32]),
    "rmg_sensor_create": (C.c_int, [C.POINTER(ModelC), _P, C.POINTER(_P)]),
    "rmg_sensor_destroy": (C.c_int, [_P]),
    "rmg_sensor_directions": (C.c_int, [_P, _P]),
    "rmg_sensor_size": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U32)]),
    "rmg_sensor_visit_order": (C.c_int, [_P, _P, C.POINTER(C.c_int)]),
    "rmg_simulate": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC), _P]),
    "rmg_simulate_ex": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC),
                                  C.POINTER(LaunchConfigC), _P]),
    "rmg_default_launch_config": (C.c_int, [_P, _P, C.POINTER(LaunchConfigC)]),
    "rmg_simulate_host": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC),
                                    C.POINTER(LaunchConfigC), _P]),
    "rmg_host_set_pipeline": (C.c_int, [C.c_uint64, _U32]),
    "rmg_host_staging_trim": (C.c_int, []),
    "rmg_autotune_launch_config": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC), _U32,
                                             C.POINTER(LaunchConfigC), _P]),
    "rmg_lbvh_build_noalloc": (C.c_int, [_P, _U32, _P, _U32, C.POINTER(LbvhBuffersC), _P]),
    "rmg_statistics_p2p": (C.c_int, [_P, _U32, _P, _P, _P, _P, _P, _P, C.POINTER(ConstraintsC), _U32, _U32,
                                     _P, _P, _P]),
    "rmg_statistics_p2l": (C.c_int, [_P, _U32, _P, _P, _P, _P, _P, _P, _P, C.POINTER(ConstraintsC), _U32, _U32,
                                     _P, _P, _P]),
    "rmg_umeyama_transform": (C.c_int, [_P, _U32, _P, _P]),
    "rmg_svd3": (C.c_int, [_P, _P, _P, _P, _P, _U32, C.c_int, _P]),
    "rmg_map_build_wide8": (C.c_int, [_P, _P]),
    "rmg_host_set_points_policy": (C.c_int, [_U32]),
    "rmg_simulate_statistics": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(ScanC), _P, _U32,
                                          C.POINTER(ConstraintsC), C.c_int, _P, _P, _P]),
    "rmg_simulate_statistics_host": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(ScanC), _P, _U32,
                                               C.POINTER(ConstraintsC), C.c_int, _P, _P, _P]),
    "rmg_transforms_compose": (C.c_int, [_P, _U32, _P, _U32, _P, _U32, _P]),
    "rmg_mesh_read": (C.c_int, [C.c_char_p, C.POINTER(MeshC)]),
    "rmg_mesh_free": (None, [C.POINTER(MeshC)]),
    "rmg_mesh_write_ply": (C.c_int, [C.c_char_p, _P, _U32, _P, _U32]),
    "rmg_map_save": (C.c_int, [_P, C.c_char_p]),
    "rmg_map_load": (C.c_int, [C.c_char_p, _P, C.POINTER(_P)]),
    "rmg_noise_apply": (C.c_int, [C.POINTER(NoiseC), _P, C.c_uint64, _P]),
    "rmg_noise_philox": (C.c_int, [C.POINTER(NoiseC), _P, C.c_uint64, _P]),
    "rmg_noise_status": (C.c_int, [C.POINTER(C.c_uint32), C.c_int]),
    "rmg_scene_create": (C.c_int, [_P, _U32, _P, _U32, _P, C.POINTER(_P)]),
    "rmg_scene_update": (C.c_int, [_P, _P, _U32, C.c_int, _P]),
    "rmg_scene_destroy": (C.c_int, [_P]),
    "rmg_scene_status": (C.c_int, [_P, C.c_int]),
    "rmg_simulate_scene": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC), _P]),
    "rmg_simulate_scene_host": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, C.POINTER(OutputsC), _P]),
    "rmg_batch_default_config": (C.c_int, [C.POINTER(BatchConfigC)]),
    "rmg_batch_create": (C.c_int, [_P, C.POINTER(BatchEntryC), _U32, C.POINTER(_P)]),
    "rmg_batch_set_config": (C.c_int, [_P, C.POINTER(BatchConfigC)]),
    "rmg_batch_get_config": (C.c_int, [_P, C.POINTER(BatchConfigC)]),
    "rmg_batch_info": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "rmg_batch_launch": (C.c_int, [_P, _P]),
    "rmg_batch_autotune": (C.c_int, [_P, _P, _U32, C.POINTER(BatchConfigC)]),
    "rmg_batch_destroy": (C.c_int, [_P]),
    "rmg_range_pose_grad": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, _P, C.c_float, _P, _P, _P, _P, _P]),
    "rmg_range_pose_grad_host": (C.c_int, [_P, _P, C.POINTER(TransformC), _P, _U32, _P, C.c_float, _P, _P, _P, _P,
                                           _P]),
    "rmg_umeyama_backward": (C.c_int, [_P, _U32, _P, _P, _P, _P, _P, _P, C.POINTER(ConstraintsC), _U32, _U32,
                                       _P, _P, _P, _P, _P, _P]),
}

_lib: C.CDLL | None = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads librmg_gb300.so and binds every declared entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RmgError(RMG_ERR_NO_DEVICE, "load",
                       f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != RMG_OK:
        lib = load()
        msg = lib.rmg_last_error().decode(errors="replace") or lib.rmg_status_string(status).decode()
        raise RmgError(status, where, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
