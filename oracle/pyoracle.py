"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle
(oracle/vsim_oracle.cpp), the restatement of the reference step the GPU
library is checked against. Only tests, the smoke check and the bench's CPU
legs import this.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "_build" / "libvsim_oracle.so"

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_U = C.POINTER(C.c_uint32)

_lib = None


def build():
    proc = subprocess.run(["make", "-C", str(ORACLE_DIR), "-s"], capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{proc.stdout}\n{proc.stderr}")
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        sig = {
            "vo_create": (C.c_int, [_P, C.c_uint32, _P, C.c_int, C.POINTER(_P)]),
            "vo_create_ex": (C.c_int, [_P, C.c_uint32, _P, C.c_int, C.c_uint32, C.POINTER(_P)]),
            "vo_destroy": (None, [_P]),
            "vo_set_threads": (None, [C.c_int]),
            "vo_max_threads": (C.c_int, []),
            "vo_set_step_duration": (C.c_int, [_P, C.c_double]),
            "vo_set_gravity": (C.c_int, [_P, _D]),
            "vo_set_contact": (C.c_int, [_P, C.c_int]),
            "vo_set_self_contact": (C.c_int, [_P, C.c_int]),
            "vo_set_iterations": (C.c_int, [_P, C.c_uint32]),
            "vo_set_material": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32]),
            "vo_hold": (C.c_int, [_P, _U, _F, C.c_uint32]),
            "vo_release": (C.c_int, [_P]),
            "vo_set_drive_law": (C.c_int, [_P, C.c_int]),
            "vo_set_drive_response_time": (C.c_int, [_P, C.c_double]),
            "vo_set_grab": (C.c_int, [_P, _D, _D]),
            "vo_dispatch": (C.c_int, [_P, C.c_uint32]),
            "vo_node_count": (C.c_uint32, [_P]),
            "vo_cell_count": (C.c_uint32, [_P]),
            "vo_surface_count": (C.c_uint32, [_P]),
            "vo_body_node_offset": (C.c_uint32, [_P, C.c_uint32]),
            "vo_get_state": (C.c_int, [_P, _F, _F, _F]),
            "vo_get_state_f64": (C.c_int, [_P, _D, _D, _D]),
            "vo_set_state": (C.c_int, [_P, _F, _F, _F]),
            "vo_inv_mass": (C.c_int, [_P, _F]),
            "vo_cells": (C.c_int, [_P, C.c_uint32, _U, _U]),
            "vo_surface": (C.c_int, [_P, _U, _U]),
            "vo_contact_pairs": (C.c_size_t, [_P, _U, C.c_size_t]),
            "vo_contact_grid": (C.c_int, [_P, _D, _D, _U]),
            "vo_splat_deform": (C.c_int, [_P, C.c_uint32, _F, _F, _F, C.c_uint32, _F, _F, _F, _U]),
            "vo_stable_sort_u32": (None, [_U, C.c_uint32, C.c_uint32, _U]),
            "vo_kuhn_tets": (None, [_U]),
            "vo_kuhn_rest_inverses": (None, [C.c_double, _D]),
            "vo_kuhn_rest_shapes": (None, [C.c_double, _D]),
            "vo_project_tet_f64": (None, [_D, _D, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double, _D]),
            "vo_run_free_tet_f64": (None, [_D, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_uint32]),
            "vo_tet_constraints_f64": (None, [_D, _D, C.c_double, _D, _D, _D, _D]),
            "vo_resolve_pair_f64": (C.c_int, [_D, _D, C.c_uint32, C.c_uint32, _D]),
            "vo_drive_hard_f64": (None, [_D, _D, _D, C.c_double, _D, _D]),
            "vo_drive_compliant_f64": (None, [_D, _D, C.c_double, C.c_double, _D]),
            "vo_stretch_pair_f64": (None, [_D, _D, C.c_double, C.c_double, C.c_double]),
            "vo_resolve_plane_f64": (None, [_D, _D, _D, C.c_double, C.c_double, _D]),
            "vo_deformation_at_f64": (None, [_D, _U, _U, _D, C.c_double, _D, _D, _D]),
            "vo_deformed_covariance_f64": (None, [_D, _D, _D, _D]),
            "vo_ellipsoid_axes_f64": (None, [_D, _D, _D]),
            "vo_ellipsoid_axes_f32": (None, [_F, C.c_uint32, _F, _F]),
            "vo_stretch_edges": (None, [_D]),
            "vo_broadphase_grid": (None, [_D, _D, C.c_double, _D, _D, _U]),
            "vo_bucket_of": (C.c_uint32, [_D, C.c_double, _U, _D]),
            "vo_surface_nodes": (C.c_uint32, [_U, C.POINTER(C.c_uint8), _U]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def f64(a):
    a = np.ascontiguousarray(a, np.float64)
    return a, a.ctypes.data_as(_D)


def set_threads(n: int):
    lib().vo_set_threads(int(n))


def max_threads() -> int:
    return int(lib().vo_max_threads())


class Oracle:
    """The reference step on the CPU for one scene, in float (precision 32,
    the GPU's arithmetic) or double (64, the drift reference)."""

    def __init__(self, scene, precision: int = 32):
        import vsim.scenes as scenes  # the scene's ctypes descriptors

        self._descs = scenes.Descs(scene)
        h = C.c_void_p()
        flags = 1 if getattr(scene, "isolated", False) else 0
        rc = lib().vo_create_ex(C.cast(self._descs.bodies, _P), self._descs.count,
                                C.cast(C.byref(self._descs.tank), _P), precision, flags, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"vo_create failed with {rc}")
        self._h = h
        self.scene = scene
        self.node_count = int(lib().vo_node_count(h))
        if scene.step_duration is not None:
            lib().vo_set_step_duration(h, float(scene.step_duration))
        lib().vo_set_iterations(h, int(scene.iterations))
        lib().vo_set_contact(h, int(scene.contact))
        lib().vo_set_self_contact(h, int(scene.self_contact))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().vo_destroy(self._h)
            self._h = None

    def dispatch(self, steps: int):
        lib().vo_dispatch(self._h, int(steps))

    def state(self):
        pos, prev, vel = (np.zeros((self.node_count, 4), np.float32) for _ in range(3))
        lib().vo_get_state(self._h, pos.ctypes.data_as(_F), prev.ctypes.data_as(_F), vel.ctypes.data_as(_F))
        return pos, prev, vel

    def state_f64(self):
        pos, prev, vel = (np.zeros((self.node_count, 4), np.float64) for _ in range(3))
        lib().vo_get_state_f64(self._h, pos.ctypes.data_as(_D), prev.ctypes.data_as(_D), vel.ctypes.data_as(_D))
        return pos, prev, vel

    def set_state(self, pos=None, prev=None, vel=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (pos, prev, vel)]
        lib().vo_set_state(self._h, *(None if a is None else a.ctypes.data_as(_F) for a in arrs))

    def inv_mass(self):
        out = np.zeros(self.node_count, np.float32)
        lib().vo_inv_mass(self._h, out.ctypes.data_as(_F))
        return out

    def surface(self):
        n = int(lib().vo_surface_count(self._h))
        nodes, bodies = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        lib().vo_surface(self._h, nodes.ctypes.data_as(_U), bodies.ctypes.data_as(_U))
        return nodes, bodies

    def cells(self, body: int):
        counts = np.zeros(8, np.uint32)
        lib().vo_cells(self._h, body, None, counts.ctypes.data_as(_U))
        out = np.zeros(int(counts.sum()), np.uint32)
        lib().vo_cells(self._h, body, out.ctypes.data_as(_U), counts.ctypes.data_as(_U))
        return out, counts

    def contact_pairs(self):
        total = int(lib().vo_contact_pairs(self._h, None, 0))
        out = np.zeros((max(total, 1), 2), np.uint32)
        lib().vo_contact_pairs(self._h, out.ctypes.data_as(_U), total)
        out = out[:total]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def hold(self, nodes, offsets):
        nodes = np.ascontiguousarray(nodes, np.uint32)
        offsets = np.ascontiguousarray(offsets, np.float32).reshape(-1, 3)
        return lib().vo_hold(self._h, nodes.ctypes.data_as(_U), offsets.ctypes.data_as(_F), int(nodes.size))

    def release(self):
        lib().vo_release(self._h)

    def set_drive_law(self, law: str):
        lib().vo_set_drive_law(self._h, 0 if law == "hard" else 1)

    def set_drive_response_time(self, seconds):
        lib().vo_set_drive_response_time(self._h, float(seconds))

    def set_grab(self, target, velocity):
        t, tp = f64(target)
        v, vp = f64(velocity)
        lib().vo_set_grab(self._h, tp, vp)

    def set_material(self, body, changes: dict):
        import vsim._ffi as ffi

        m = ffi.Material()
        bits = {"youngs_modulus": ffi.MAT_YOUNGS, "poisson_ratio": ffi.MAT_POISSON, "density": ffi.MAT_DENSITY,
                "friction": ffi.MAT_FRICTION, "damping": ffi.MAT_DAMPING, "relaxation": ffi.MAT_RELAXATION,
                "max_stretch": ffi.MAT_MAX_STRETCH}
        fields = 0
        for k, v in changes.items():
            setattr(m, k, float(v))
            fields |= bits[k]
        return lib().vo_set_material(self._h, int(body), C.cast(C.byref(m), _P), fields)

    def set_gravity(self, g):
        a, p = f64(g)
        lib().vo_set_gravity(self._h, p)

    def set_step_duration(self, seconds):
        lib().vo_set_step_duration(self._h, float(seconds))

    def set_contact(self, enabled: bool):
        lib().vo_set_contact(self._h, int(bool(enabled)))

    def set_self_contact(self, enabled: bool):
        lib().vo_set_self_contact(self._h, int(bool(enabled)))

    def splat_deform(self, body, means, quats, scales, view_dir=(0.0, 0.0, -1.0)):
        n = means.shape[0]
        means = np.ascontiguousarray(means, np.float32)
        quats = np.ascontiguousarray(quats, np.float32)
        scales = np.ascontiguousarray(scales, np.float32)
        view = np.ascontiguousarray(view_dir, np.float32)
        out_m = np.zeros((n, 3), np.float32)
        out_c = np.zeros((n, 6), np.float32)
        keys = np.zeros(n, np.uint32)
        lib().vo_splat_deform(self._h, body, means.ctypes.data_as(_F), quats.ctypes.data_as(_F),
                              scales.ctypes.data_as(_F), n, view.ctypes.data_as(_F), out_m.ctypes.data_as(_F),
                              out_c.ctypes.data_as(_F), keys.ctypes.data_as(_U))
        return out_m, out_c, keys


def ellipsoid_axes_f64(cov6) -> tuple:
    """(rotation xyzw, scale xyz) of one covariance (xx, xy, xz, yy, yz, zz)."""
    c = np.ascontiguousarray(cov6, np.float64)
    rot, sc = np.zeros(4), np.zeros(3)
    lib().vo_ellipsoid_axes_f64(c.ctypes.data_as(_D), rot.ctypes.data_as(_D), sc.ctypes.data_as(_D))
    return rot, sc


def ellipsoid_axes_f32(cov6: np.ndarray) -> tuple:
    """Rotations (n, 4) and scales (n, 3) of n float covariances (n, 6)."""
    c = np.ascontiguousarray(cov6, np.float32).reshape(-1, 6)
    n = c.shape[0]
    rot, sc = np.zeros((n, 4), np.float32), np.zeros((n, 3), np.float32)
    lib().vo_ellipsoid_axes_f32(c.ctypes.data_as(_F), n, rot.ctypes.data_as(_F), sc.ctypes.data_as(_F))
    return rot, sc


def stable_sort(keys: np.ndarray, key_bits: int = 32) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.uint32)
    order = np.zeros(keys.size, np.uint32)
    lib().vo_stable_sort_u32(keys.ctypes.data_as(_U), keys.size, key_bits, order.ctypes.data_as(_U))
    return order
