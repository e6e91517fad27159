"""ctypes binding of libvsim's C ABI (include/vsim.h).

Loading fails loudly when the library has not been built: there is no
fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

# The server's request loop keeps up to ten streams busy at once (eight
# session launch slots, the pool's stream, its capture stream). The CUDA
# driver feeds streams to the GPU through CUDA_DEVICE_MAX_CONNECTIONS hardware
# queues, eight unless set, assigned in turn as streams are created: with
# eight, a slot's stream shares the pool stream's queue, and a tick's
# launches wait behind a session job of several milliseconds queued ahead of
# them. 32 (the most the driver takes) gives every stream its own queue. The
# driver reads the variable when the process creates its CUDA context, so it
# acts only if nothing has touched CUDA yet; a value the caller set is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

LIB_PATH = Path(__file__).resolve().parent / "libvsim.so"
HEADER = Path(__file__).resolve().parents[2] / "include" / "vsim.h"

VSIM_OK = 0
VSIM_ERR_RANGE = 1
VSIM_ERR_INVALID = 2
VSIM_ERR_CUDA = 3
VSIM_ERR_NOMEM = 4
VSIM_ERR_DESTROYED = 5
VSIM_ERR_CAPACITY = 6
VSIM_ERR_TIMEOUT = 7
VSIM_DRIVE_HARD = 0
VSIM_DRIVE_COMPLIANT = 1
VSIM_MAX_DRIVEN = 4096

MAT_YOUNGS = 1 << 0
MAT_POISSON = 1 << 1
MAT_DENSITY = 1 << 2
MAT_FRICTION = 1 << 3
MAT_DAMPING = 1 << 4
MAT_RELAXATION = 1 << 5
MAT_MAX_STRETCH = 1 << 6


class Material(C.Structure):
    _fields_ = [
        ("youngs_modulus", C.c_double),
        ("poisson_ratio", C.c_double),
        ("density", C.c_double),
        ("friction", C.c_double),
        ("damping", C.c_double),
        ("relaxation", C.c_double),
        ("max_stretch", C.c_double),
    ]


class BodyDesc(C.Structure):
    _fields_ = [
        ("cell_dims", C.c_uint32 * 3),
        ("origin", C.c_double * 3),
        ("h", C.c_double),
        ("occupancy", C.POINTER(C.c_uint8)),
        ("material", Material),
        ("static_nodes", C.POINTER(C.c_uint32)),
        ("static_count", C.c_uint32),
    ]


class Tank(C.Structure):
    _fields_ = [("min", C.c_double * 3), ("max", C.c_double * 3)]


class Stats(C.Structure):
    _fields_ = [
        ("body_count", C.c_uint32),
        ("nodes", C.c_uint32),
        ("active_nodes", C.c_uint32),
        ("cells", C.c_uint32),
        ("contact_nodes", C.c_uint32),
        ("contact", C.c_int32),
        ("self_contact", C.c_int32),
        ("iterations", C.c_uint32),
        ("steps", C.c_uint64),
        ("last_steps", C.c_uint32),
        ("max_steps_per_frame", C.c_uint32),
        ("step_duration", C.c_double),
        ("simulated_time", C.c_double),
        ("backlog_time", C.c_double),
        ("frame_dropped_time", C.c_double),
        ("dropped_time", C.c_double),
        ("overloaded", C.c_int32),
        ("cfl", C.c_double),
        ("limited_by", C.c_int32),
        ("driven", C.c_uint32),
        ("drive_capacity", C.c_uint32),
    ]


class ContactCensus(C.Structure):
    _fields_ = [("records", C.c_uint64), ("occupied_buckets", C.c_uint64), ("candidates", C.c_uint64),
                ("ms", C.c_double * 5)]


class Profile(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("launches", C.c_uint32 * 8)]


KINDS = ("predict", "drive", "elastic", "limit", "contact", "finalize", "splat", "sort")


class ClockReport(C.Structure):
    _fields_ = [
        ("step_duration", C.c_double),
        ("max_steps_per_frame", C.c_uint32),
        ("steps", C.c_uint32),
        ("elapsed", C.c_double),
        ("total_steps", C.c_uint64),
        ("simulated_time", C.c_double),
        ("backlog_time", C.c_double),
        ("frame_dropped_time", C.c_double),
        ("dropped_time", C.c_double),
        ("overloaded", C.c_int32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("step_duration", C.c_double), ("substeps", C.c_uint32),
                ("self_contact", C.c_int32)]


class Drag(C.Structure):
    _fields_ = [("node", C.c_uint32), ("control", (C.c_float * 3) * 4), ("speed", C.c_double)]


class Completion(C.Structure):
    _fields_ = [("request", C.c_uint64), ("session", C.c_uint32), ("frames", C.c_uint32),
                ("submitted", C.c_double), ("completed", C.c_double), ("first_tick", C.c_uint64),
                ("last_tick", C.c_uint64)]


class GrabResult(C.Structure):
    _fields_ = [("body", C.c_int32), ("anchor", C.c_uint32), ("position", C.c_double * 3), ("held", C.c_uint32),
                ("found", C.c_uint32)]


class CloudOptions(C.Structure):
    _fields_ = [("element_size", C.c_double), ("sigma", C.c_double), ("padding", C.c_uint32), ("seal", C.c_uint32),
                ("fill", C.c_int32)]


class CloudGrid(C.Structure):
    _fields_ = [("dims", C.c_uint32 * 3), ("origin", C.c_double * 3), ("h", C.c_double), ("occupied", C.c_uint64),
                ("filled", C.c_uint64)]


VSIM_GRIP_SINGLE_NODE = 0
VSIM_GRIP_WITHIN_RADIUS = 1


class ScheduledRequest(C.Structure):
    _fields_ = [("arrival", C.c_double), ("session", C.c_uint32), ("frames", C.c_uint32), ("drag", C.c_uint32),
                ("pad", C.c_uint32)]


class RunReport(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("frames", C.c_uint64), ("ticks", C.c_uint64), ("returned", C.c_uint32),
                ("pad", C.c_uint32), ("seconds", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("sessions", C.c_uint32), ("rejected", C.c_uint32), ("resident_bytes", C.c_double),
                ("ticks", C.c_uint64), ("session_frames", C.c_uint64), ("cell_updates", C.c_uint64),
                ("pending", C.c_uint32), ("tick_seconds", C.c_double), ("prepare_seconds", C.c_double),
                ("frame_seconds", C.c_double)]


VSIM_CREATE_ISOLATED = 1

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_U = C.POINTER(C.c_uint32)
_SZ = C.c_size_t

SIGNATURES = {
    "vsim_last_error": (C.c_char_p, []),
    "vsim_abi_version": (C.c_int, []),
    "vsim_create": (C.c_int, [C.POINTER(BodyDesc), C.c_uint32, C.POINTER(Tank), _P, C.POINTER(_P)]),
    "vsim_destroy": (C.c_int, [_P]),
    "vsim_create_ex": (C.c_int, [C.POINTER(BodyDesc), C.c_uint32, C.POINTER(Tank), _P, C.c_uint32, C.POINTER(_P)]),
    "vsim_set_bodies_active": (C.c_int, [_P, C.POINTER(C.c_uint8), C.c_uint32]),
    "vsim_server_create": (C.c_int, [C.POINTER(BodyDesc), C.c_uint32, C.POINTER(Tank), C.POINTER(ServerConfig), _P,
                                     C.POINTER(_P)]),
    "vsim_server_destroy": (C.c_int, [_P]),
    "vsim_server_admitted": (C.c_uint32, [_P]),
    "vsim_server_resident": (C.c_int, [_P, _U, C.c_uint32, _U]),
    "vsim_server_set_resident": (C.c_int, [_P, _U, C.c_uint32]),
    "vsim_server_clock": (C.c_double, [_P]),
    "vsim_server_submit": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(Drag), C.POINTER(C.c_uint64)]),
    "vsim_server_tick": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "vsim_server_set_tick_budget": (C.c_int, [_P, C.c_uint64]),
    "vsim_server_set_engine": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_uint32]),
    "vsim_server_run": (C.c_int, [_P, C.POINTER(ScheduledRequest), C.c_uint32, C.POINTER(Drag), C.c_double,
                                  C.POINTER(Completion), C.c_uint32, C.POINTER(RunReport)]),
    "vsim_server_poll": (C.c_int, [_P, C.POINTER(Completion), C.c_uint32, C.POINTER(C.c_uint32)]),
    "vsim_server_get_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "vsim_server_node_count": (C.c_uint32, [_P, C.c_uint32]),
    "vsim_server_read_positions": (C.c_int, [_P, C.c_uint32, _F, _SZ]),
    "vsim_server_read_state": (C.c_int, [_P, C.c_uint32, _F, _F, _F, _SZ]),
    "vsim_server_write_state": (C.c_int, [_P, C.c_uint32, _F, _F, _F, _SZ]),
    "vsim_server_reset_session": (C.c_int, [_P, C.c_uint32]),
    "vsim_step": (C.c_int, [_P, C.c_double]),
    "vsim_request_step": (C.c_int, [_P]),
    "vsim_dispatch": (C.c_int, [_P, C.c_uint32]),
    "vsim_reset": (C.c_int, [_P]),
    "vsim_synchronize": (C.c_int, [_P]),
    "vsim_read_positions": (C.c_int, [_P, _F, _SZ]),
    "vsim_read_state": (C.c_int, [_P, _F, _F, _F, _SZ]),
    "vsim_write_state": (C.c_int, [_P, _F, _F, _F, _SZ]),
    "vsim_node_count": (C.c_uint32, [_P]),
    "vsim_body_node_offset": (C.c_uint32, [_P, C.c_uint32]),
    "vsim_read_inv_mass": (C.c_int, [_P, _F, _SZ]),
    "vsim_hold": (C.c_int, [_P, _U, _F, C.c_uint32]),
    "vsim_move_grab": (C.c_int, [_P, _D]),
    "vsim_place_grab": (C.c_int, [_P, _D]),
    "vsim_release": (C.c_int, [_P]),
    "vsim_set_drive_law": (C.c_int, [_P, C.c_int]),
    "vsim_set_drive_response_time": (C.c_int, [_P, C.c_double]),
    "vsim_set_material": (C.c_int, [_P, C.c_uint32, C.POINTER(Material), C.c_uint32]),
    "vsim_set_contact": (C.c_int, [_P, C.c_int]),
    "vsim_set_self_contact": (C.c_int, [_P, C.c_int]),
    "vsim_set_gravity": (C.c_int, [_P, _D]),
    "vsim_set_paused": (C.c_int, [_P, C.c_int]),
    "vsim_set_step_duration": (C.c_int, [_P, C.c_double]),
    "vsim_set_iterations": (C.c_int, [_P, C.c_uint32]),
    "vsim_set_graph": (C.c_int, [_P, C.c_int]),
    "vsim_set_launch_shape": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "vsim_tune": (C.c_int, [_P, C.c_uint32, _U, _U]),
    "vsim_set_pdl": (C.c_int, [_P, C.c_int]),
    "vsim_set_gather_mapping": (C.c_int, [_P, C.c_int]),
    "vsim_set_tma_pass": (C.c_int, [_P, C.c_int]),
    "vsim_set_cell_lanes": (C.c_int, [_P, C.c_uint32]),
    "vsim_grab": (C.c_int, [_P, _D, _D, C.c_int, C.c_double, C.POINTER(GrabResult)]),
    "vsim_time_colour_passes": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_float)]),
    "vsim_kuhn_rest_inverse": (C.c_int, [_F]),
    "vsim_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "vsim_cfl_number": (C.c_int, [_P, _D]),
    "vsim_contact_pairs": (C.c_int, [_P, _U, _SZ, C.POINTER(_SZ)]),
    "vsim_contact_surface": (C.c_int, [_P, _U, _U, _SZ, C.POINTER(_SZ)]),
    "vsim_contact_census": (C.c_int, [_P, C.POINTER(ContactCensus)]),
    "vsim_splats_bind": (C.c_int, [_P, C.c_uint32, _F, _F, _F, C.c_uint32]),
    "vsim_splats_count": (C.c_uint32, [_P]),
    "vsim_splats_deform": (C.c_int, [_P, _F]),
    "vsim_splats_sort": (C.c_int, [_P]),
    "vsim_splats_deform_axes": (C.c_int, [_P, _F]),
    "vsim_splats_read_axes": (C.c_int, [_P, _F, _F, _SZ]),
    "vsim_splats_read": (C.c_int, [_P, _F, _F, _U, _SZ]),
    "vsim_radix_sort_u32": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, _P, C.POINTER(_SZ), _P]),
    "vsim_voxelize_cloud": (C.c_int, [_F, _F, _F, C.c_uint64, C.POINTER(CloudOptions), C.POINTER(_P)]),
    "vsim_voxelize_cloud_device": (C.c_int, [_P, _P, _P, C.c_uint64, C.POINTER(CloudOptions), _P, C.POINTER(_P)]),
    "vsim_cloud_volume_grid": (C.c_int, [_P, C.POINTER(CloudGrid)]),
    "vsim_cloud_volume_read": (C.c_int, [_P, C.POINTER(C.c_uint8), _SZ]),
    "vsim_cloud_volume_destroy": (C.c_int, [_P]),
    "vsim_cloud_set_flood_rounds": (C.c_uint32, [C.c_uint32]),
    "vsim_radix_sort_u32_noalloc": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, _P]),
    "vsim_profile_frame": (C.c_int, [_P, C.c_uint32, C.c_int, _F, C.POINTER(Profile)]),
    "vsim_color_counts": (C.c_int, [_P, _U]),
    "vsim_frame_launches": (C.c_uint32, [_P, C.c_uint32]),
    "vsim_splat_launches": (C.c_uint32, [_P]),
    "vsim_stable_step_duration": (C.c_int, [C.c_double, _D]),
    "vsim_clock_create": (C.c_int, [C.c_double, C.c_uint32, C.POINTER(_P)]),
    "vsim_clock_destroy": (C.c_int, [_P]),
    "vsim_clock_consume": (C.c_int, [_P, C.c_double, C.c_int, C.POINTER(ClockReport)]),
    "vsim_clock_idle": (C.c_int, [_P, C.POINTER(ClockReport)]),
    "vsim_clock_single_step": (C.c_int, [_P, C.POINTER(ClockReport)]),
    "vsim_clock_set_step_duration": (C.c_int, [_P, C.c_double]),
    "vsim_clock_reset": (C.c_int, [_P]),
    "vsim_clock_snapshot": (C.c_int, [_P, C.POINTER(ClockReport)]),
    "vsim_lame_parameters": (C.c_int, [C.POINTER(Material), _D, _D]),
    "vsim_element_compliance": (C.c_int, [C.POINTER(Material), C.c_double, _D, _D, _D]),
    "vsim_collapse_scale": (C.c_double, [C.c_double]),
    "vsim_wave_speed": (C.c_double, [C.POINTER(Material)]),
}


def header_symbols(header: Path = HEADER) -> list[str]:
    """Every function the public header declares."""
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vsim_[a-z0-9_]+)\s*\(", text)))


_lib = None


def lib() -> C.CDLL:
    """The loaded library with every signature declared."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"libvsim.so is not built ({LIB_PATH}); run __graft_entry__.build() first")
        handle = C.CDLL(str(LIB_PATH))
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = handle
    return _lib


class VsimError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class VsimRangeError(VsimError, ValueError):
    """The reference's RangeError."""


def check(code: int) -> None:
    if code == VSIM_OK:
        return
    msg = lib().vsim_last_error().decode()
    if code == VSIM_ERR_RANGE:
        raise VsimRangeError(code, msg)
    raise VsimError(code, msg)


def fptr(arr):
    return arr.ctypes.data_as(_F) if arr is not None else None


def uptr(arr):
    return arr.ctypes.data_as(_U) if arr is not None else None


def dptr(arr):
    return arr.ctypes.data_as(_D) if arr is not None else None
