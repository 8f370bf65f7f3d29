"""ctypes binding of librp.so (include/rp.h).

The library is built in-tree (rusty_particles_gb300/_build/librp.so). Loading
fails loudly if it is missing: there is no CPU implementation behind this
module.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

RP_OK = 0
RP_E_INVALID_ARG = -1
RP_E_INDEX = -2
RP_E_IO = -3
RP_E_CUDA = -4
RP_E_DEVICE_FLAG = -5
RP_E_TIMEOUT = -6
RP_E_NOMEM = -7

RP_PREC_FP64, RP_PREC_MIXED = 0, 1
RP_MODE_PARITY, RP_MODE_PHYSICAL = 0, 1

_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)


class RpState(ctypes.Structure):
    _fields_ = [
        ("n_particles", ctypes.c_size_t),
        ("position", _dp),
        ("velocity", _dp),
        ("angular_velocity", _dp),
        ("acceleration", _dp),
        ("torque", _dp),
        ("position_residual", _dp),
        ("velocity_residual", _dp),
        ("angular_velocity_residual", _dp),
        ("radius", _dp),
        ("mass", _dp),
        ("fixed", _u8p),
    ]


class RpStats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_uint64),
        ("particles", ctypes.c_uint64),
        ("removed", ctypes.c_uint64),
        ("neighbor_rebuilds", ctypes.c_uint64),
        ("overlap_warn_steps", ctypes.c_uint64),
        ("status_bits", ctypes.c_uint64),
        ("neighbor_capacity", ctypes.c_uint64),
        ("max_neighbors", ctypes.c_uint64),
        ("kinetic_energy", ctypes.c_double),
        ("device_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64),
        ("force_launches", ctypes.c_uint64),
        ("force_ms", ctypes.c_double),
        ("state_io_direct", ctypes.c_uint64),
        ("state_uploads", ctypes.c_uint64),
        ("state_downloads", ctypes.c_uint64),
        ("compactions", ctypes.c_uint64),
        ("device_inserts", ctypes.c_uint64),
    ]


RP_JKR_NEWTON, RP_JKR_LEARNED, RP_JKR_CERTIFIED = 0, 1, 2
RP_MLP_PARAMS = 8705
_fp = ctypes.POINTER(ctypes.c_float)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
RP_GROUP_ALL = 0xFFFFFFFF


class RpTuneReport(ctypes.Structure):
    _fields_ = [
        ("force_path", ctypes.c_int32),
        ("bs_filter", ctypes.c_int32),
        ("bs_force", ctypes.c_int32),
        ("bs_accum", ctypes.c_int32),
        ("grid_cap", ctypes.c_int32),
        ("candidates", ctypes.c_int32),
        ("default_ms", ctypes.c_double),
        ("best_ms", ctypes.c_double),
    ]


class RpJkrTrainOptions(ctypes.Structure):
    _fields_ = [
        ("rs_min", ctypes.c_double),
        ("rs_max", ctypes.c_double),
        ("es_scale", ctypes.c_double),
        ("gamma_scale", ctypes.c_double),
        ("x_min", ctypes.c_double),
        ("x_max", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("samples", ctypes.c_uint64),
        ("epochs", ctypes.c_int32),
        ("batch", ctypes.c_int32),
        ("lr0", ctypes.c_float),
        ("lr1", ctypes.c_float),
        ("qat_from_epoch", ctypes.c_int32),
    ]


class RpJkrTrainReport(ctypes.Structure):
    _fields_ = [
        ("final_loss", ctypes.c_double),
        ("val_rms", ctypes.c_double),
        ("val_max", ctypes.c_double),
        ("train_ms", ctypes.c_double),
        ("samples", ctypes.c_uint64),
        ("valid_samples", ctypes.c_uint64),
        ("steps", ctypes.c_uint64),
    ]


# name -> (restype, argtypes); the list of exported entry points of rp.h
SIGNATURES = {
    "rp_create": (ctypes.c_void_p, [ctypes.c_double, _dp, _dp, ctypes.c_size_t]),
    "rp_destroy": (None, [ctypes.c_void_p]),
    "rp_add_particle": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int]),
    "rp_add_particles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp, _dp, _dp, _u8p]),
    "rp_add_mesh_stl": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "rp_add_mesh_triangles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_float)]),
    "rp_set_particle_material": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_double] * 6),
    "rp_set_wall_material": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_double] * 6),
    "rp_set_contact_models": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "rp_parse_contact_models": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_int)]),
    "rp_set_periodic": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "rp_enable_gpu": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "rp_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "rp_particle_count": (ctypes.c_size_t, [ctypes.c_void_p]),
    "rp_get_particle_position": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp]),
    "rp_get_particle_velocity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp]),
    "rp_get_particle_angular_velocity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp]),
    "rp_set_particle_velocity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t] + [ctypes.c_double] * 3),
    "rp_set_particle_angular_velocity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t] + [ctypes.c_double] * 3),
    "rp_write_vtk": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "rp_read_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RpState)]),
    "rp_write_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RpState)]),
    "rp_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_set_interaction_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_set_gravity": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_double] * 3),
    "rp_set_reference_cell_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "rp_set_skin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "rp_set_neighbor_capacity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_set_device_loop": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_set_force_path": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_set_threads": (ctypes.c_int, [ctypes.c_int]),
    "rp_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RpStats)]),
    "rp_bed_statistics": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "rp_measure_fp64_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "rp_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_last_error": (ctypes.c_char_p, []),
    "rp_version": (ctypes.c_char_p, []),
    "rp_set_debug": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_debug_last_forces": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "rp_debug_contact_pairs": (ctypes.c_int, [ctypes.c_void_p, _i64p, _i64p, _i32p, ctypes.c_size_t,
                                              ctypes.POINTER(ctypes.c_size_t)]),
    "rp_debug_triangle_grid": (ctypes.c_int, [ctypes.c_void_p, _i32p, _dp, _u32p, ctypes.c_size_t, _u32p,
                                              ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                              ctypes.POINTER(ctypes.c_size_t)]),
    "rp_debug_reference_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _i64p, _i64p,
                                               ctypes.POINTER(ctypes.c_size_t), _i32p]),
    "rp_cell_sort_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp, ctypes.c_double, _i32p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "rp_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RpTuneReport)]),
    "rp_set_launch_shape": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_int] * 4),
    "rp_add_mesh_triangles_group": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _fp, _fp, ctypes.c_uint32]),
    "rp_add_mesh_triangles_moving": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _fp, _fp, ctypes.c_uint32,
                                                    _dp, _dp, _dp]),
    "rp_set_particle_groups": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _u32p]),
    "rp_get_particle_groups": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _u32p]),
    "rp_set_group_material": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_double] * 6),
    "rp_jkr_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RpJkrTrainOptions),
                                    ctypes.POINTER(RpJkrTrainReport)]),
    "rp_set_jkr_solver": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "rp_jkr_get_network": (ctypes.c_int, [ctypes.c_void_p, _fp, _fp, _fp]),
    "rp_jkr_set_network": (ctypes.c_int, [ctypes.c_void_p, _fp, _fp, _fp]),
    "rp_jkr_counters": (ctypes.c_int, [ctypes.c_void_p, _u64p]),
    "rp_mlp_loss_grad": (ctypes.c_int, [_fp, _fp, _fp, _fp, ctypes.c_size_t, ctypes.c_int, _fp,
                                        ctypes.POINTER(ctypes.c_double)]),
    "rp_mlp_infer": (ctypes.c_int, [_fp, _fp, ctypes.c_size_t, _fp]),
    "rp_jkr_samples": (ctypes.c_int, [_dp, ctypes.c_uint64, ctypes.c_size_t, _fp, _fp, _fp, _dp, _i32p, _dp]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load librp.so (building it first if absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"librp.so not built ({path}); run rusty_particles_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    msg = load().rp_last_error()
    return msg.decode() if msg else ""


def check(code: int) -> int:
    """Map an RP_E_* code to the reference's Python exception types (src/lib.rs)."""
    if code == RP_OK:
        return code
    msg = last_error()
    if code == RP_E_INVALID_ARG:
        raise ValueError(msg)
    if code == RP_E_INDEX:
        raise IndexError(msg)
    if code == RP_E_IO:
        raise IOError(msg)
    if code == RP_E_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg or f"rp error {code}")
