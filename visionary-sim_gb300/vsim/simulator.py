"""The reference's `Simulator` surface (packages/visionary-sim/src/sim/
simulator.js:35-518) over libvsim's C ABI.

Method names and argument meanings follow the reference; errors raise
`VsimRangeError` where the reference throws RangeError and `VsimError` where
it throws Error. Positions come back as float32 arrays of shape (nodes, 4),
w = 0, exactly what `readPositions()` resolves to.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import check, dptr, fptr, lib, uptr
from .scenes import Descs, Scene

GRIPS = ("singleNode", "withinRadius")
DEFAULT_GRIPPED_PART_RADIUS = 0.03  # grip.js:156


# ---- pick and grip (pick.js:41-83, grip.js:58-138), host-side ---------------

def is_grabbable(inv_mass: np.ndarray, static: np.ndarray) -> np.ndarray:
    """pick.js:26-28: material and not static."""
    return (inv_mass > 0) & ~static


def nearest_node_to_ray(nodes, inv_mass, origin, direction, radius, static) -> int:
    """pick.js:41-68: the nearest grabbable node along the ray within `radius`
    of it; -1 if none. Ties along the ray keep the lowest index."""
    d = nodes[:, :3].astype(np.float64) - np.asarray(origin, np.float64)
    u = np.asarray(direction, np.float64)
    # Left to right, as JavaScript evaluates pick.js:57-62.
    depth = d[:, 0] * u[0] + d[:, 1] * u[1] + d[:, 2] * u[2]
    off_axis = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2] - depth * depth
    ok = is_grabbable(inv_mass, static) & (depth > 0) & (off_axis <= radius * radius)
    if not ok.any():
        return -1
    candidates = np.flatnonzero(ok)
    return int(candidates[np.argmin(depth[candidates])])


def body_of_node(offsets, node: int) -> int:
    """pick.js:77-83."""
    body = 0
    while body + 1 < len(offsets) and node >= offsets[body + 1]:
        body += 1
    return body


def single_node(positions, inv_mass, anchor, static):
    """grip.js:58-63."""
    if not (inv_mass[anchor] > 0 and not static[anchor]):
        return [], np.zeros((0, 3), np.float32), 0
    return [anchor], np.zeros((1, 3), np.float32), 1


def within_radius(positions, inv_mass, anchor, radius, offsets, static, limit):
    """grip.js:99-136: the anchor's own body's movable nodes within `radius`,
    nearest first, ties by index, the anchor first."""
    if not (inv_mass[anchor] > 0 and not static[anchor]):
        return [], np.zeros((0, 3), np.float32), 0
    body = body_of_node(offsets, anchor)
    start = offsets[body]
    end = offsets[body + 1] if body + 1 < len(offsets) else len(inv_mass)
    idx = np.arange(start, end)
    ok = is_grabbable(inv_mass[start:end], static[start:end]) & (idx != anchor)
    rel = positions[start:end, :3].astype(np.float64) - positions[anchor, :3].astype(np.float64)
    dist2 = rel[:, 0] * rel[:, 0] + rel[:, 1] * rel[:, 1] + rel[:, 2] * rel[:, 2]  # grip.js:118-121
    ok &= dist2 <= radius * radius
    cand = idx[ok]
    order = np.lexsort((cand, dist2[ok]))
    found = cand.size + 1
    kept = cand[order][: max(0, limit - 1)]
    nodes = [anchor] + [int(n) for n in kept]
    offs = np.vstack([np.zeros((1, 3)), rel[kept - start]]).astype(np.float32)
    return nodes, offs, found


class Simulator:
    """`new Simulator(device, bodies, tank)` with the CUDA device current."""

    def __init__(self, scene: Scene, stream=None):
        self._descs = Descs(scene)
        handle = C.c_void_p()
        flags = _ffi.VSIM_CREATE_ISOLATED if scene.isolated else 0
        check(lib().vsim_create_ex(self._descs.bodies, self._descs.count, C.byref(self._descs.tank),
                                   C.c_void_p(stream), flags, C.byref(handle)))
        self._h = handle
        self.scene = scene
        self.node_count = int(lib().vsim_node_count(handle))
        self.offsets = [int(lib().vsim_body_node_offset(handle, b)) for b in range(len(scene.bodies))]
        self.inv_mass = np.zeros(self.node_count, np.float32)
        check(lib().vsim_read_inv_mass(handle, fptr(self.inv_mass), self.node_count))
        self.static = np.zeros(self.node_count, bool)
        for b, body in enumerate(scene.bodies):
            self.static[self.offsets[b] + np.asarray(body.static_nodes, np.int64)] = True
        self.grip = {"strategy": "withinRadius", "radius": DEFAULT_GRIPPED_PART_RADIUS}
        self._gravity = (0.0, -9.81, 0.0)
        self._paused = False
        if scene.step_duration is not None:
            self.set_step_duration(scene.step_duration)
        if scene.iterations != 1:
            check(lib().vsim_set_iterations(handle, scene.iterations))
        self.set_contact(scene.contact)
        if scene.self_contact:
            check(lib().vsim_set_self_contact(handle, 1))
        for b, (means, quats, scales, *_rest) in scene.splats.items():
            self.bind_splats(b, means, quats, scales)

    # -- lifecycle ------------------------------------------------------------
    def destroy(self):
        if self._h:
            lib().vsim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- stepping ---------------------------------------------------------------
    def step(self, dt: float):
        check(lib().vsim_step(self._h, float(dt)))

    def request_step(self):
        check(lib().vsim_request_step(self._h))

    def dispatch(self, steps: int):
        check(lib().vsim_dispatch(self._h, int(steps)))

    def reset(self):
        check(lib().vsim_reset(self._h))

    def synchronize(self):
        check(lib().vsim_synchronize(self._h))

    # -- state ------------------------------------------------------------------
    def read_positions(self) -> np.ndarray:
        out = np.zeros((self.node_count, 4), np.float32)
        check(lib().vsim_read_positions(self._h, fptr(out), self.node_count))
        return out

    def read_state(self):
        pos, prev, vel = (np.zeros((self.node_count, 4), np.float32) for _ in range(3))
        check(lib().vsim_read_state(self._h, fptr(pos), fptr(prev), fptr(vel), self.node_count))
        return pos, prev, vel

    def write_state(self, pos=None, prev=None, vel=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (pos, prev, vel)]
        check(lib().vsim_write_state(self._h, *(fptr(a) for a in arrs), self.node_count))

    # -- grab (simulator.js:383-492) ---------------------------------------------
    def grab(self, origin, direction):
        """Simulator.grab (simulator.js:383-425), picked and gripped on the
        device (vsim_grab): {'bodyIndex', 'position', 'held'} or None."""
        res = _ffi.GrabResult()
        o = np.asarray(origin, np.float64)
        d = np.asarray(direction, np.float64)
        grip = _ffi.VSIM_GRIP_SINGLE_NODE if self.grip["strategy"] == "singleNode" else _ffi.VSIM_GRIP_WITHIN_RADIUS
        check(lib().vsim_grab(self._h, dptr(o), dptr(d), grip, float(self.grip["radius"]), C.byref(res)))
        if res.body < 0:
            return None
        return {"bodyIndex": int(res.body), "position": [float(v) for v in res.position], "held": int(res.held),
                "anchor": int(res.anchor), "found": int(res.found)}

    def grab_on_host(self, origin, direction):
        """The same grab with every node position read back and picked and
        gripped in Python, as the reference does (pick.js, grip.js)."""
        nodes = self.read_positions()
        aim = max(b.h for b in self.scene.bodies) * 1.2
        anchor = nearest_node_to_ray(nodes, self.inv_mass, origin, direction, aim, self.static)
        if anchor < 0:
            return None
        if self.grip["strategy"] == "singleNode":
            held, offs, _found = single_node(nodes, self.inv_mass, anchor, self.static)
        else:
            held, offs, _found = within_radius(nodes, self.inv_mass, anchor, self.grip["radius"], self.offsets,
                                               self.static, _ffi.VSIM_MAX_DRIVEN)
        position = [float(v) for v in nodes[anchor, :3]]
        self.hold(held, offs)
        check(lib().vsim_place_grab(self._h, dptr(np.asarray(position, np.float64))))
        return {"bodyIndex": body_of_node(self.offsets, anchor), "position": position, "held": len(held)}

    def hold(self, nodes, offsets):
        nodes = np.ascontiguousarray(nodes, np.uint32)
        offsets = np.ascontiguousarray(offsets, np.float32).reshape(-1, 3)
        check(lib().vsim_hold(self._h, uptr(nodes), fptr(offsets), int(nodes.size)))

    def place_grab(self, position):
        check(lib().vsim_place_grab(self._h, dptr(np.asarray(position, np.float64))))

    def move_grab(self, position):
        check(lib().vsim_move_grab(self._h, dptr(np.asarray(position, np.float64))))

    def release_grab(self):
        check(lib().vsim_release(self._h))

    def set_grip(self, strategy: str):
        if strategy not in GRIPS:
            raise _ffi.VsimError(_ffi.VSIM_ERR_INVALID, f'[grip] unknown strategy "{strategy}"')
        self.grip["strategy"] = strategy

    def set_grip_radius(self, radius: float):
        self.grip["radius"] = float(radius)

    def set_drive_law(self, law: str):
        code = {"hard": _ffi.VSIM_DRIVE_HARD, "compliant": _ffi.VSIM_DRIVE_COMPLIANT}.get(law)
        if code is None:
            raise _ffi.VsimError(_ffi.VSIM_ERR_INVALID, f'[drive] unknown law "{law}"')
        check(lib().vsim_set_drive_law(self._h, code))

    def set_drive_response_time(self, seconds: float):
        check(lib().vsim_set_drive_response_time(self._h, float(seconds)))

    # -- settings -------------------------------------------------------------
    def set_material(self, body: int, changes: dict):
        m = _ffi.Material()
        fields = 0
        bits = {"youngs_modulus": _ffi.MAT_YOUNGS, "poisson_ratio": _ffi.MAT_POISSON, "density": _ffi.MAT_DENSITY,
                "friction": _ffi.MAT_FRICTION, "damping": _ffi.MAT_DAMPING, "relaxation": _ffi.MAT_RELAXATION,
                "max_stretch": _ffi.MAT_MAX_STRETCH}
        for k, v in changes.items():
            setattr(m, k, float(v))
            fields |= bits[k]
        check(lib().vsim_set_material(self._h, int(body), C.byref(m), fields))
        check(lib().vsim_read_inv_mass(self._h, fptr(self.inv_mass), self.node_count))

    def set_bodies_active(self, active):
        """Which bodies take part in the following frames (None: all)."""
        if active is None:
            check(lib().vsim_set_bodies_active(self._h, None, len(self.scene.bodies)))
            return
        flags = np.ascontiguousarray(np.asarray(active, bool), np.uint8)
        check(lib().vsim_set_bodies_active(self._h, flags.ctypes.data_as(C.POINTER(C.c_uint8)), int(flags.size)))

    def set_contact(self, enabled: bool):
        check(lib().vsim_set_contact(self._h, int(bool(enabled))))

    def set_self_contact(self, enabled: bool):
        check(lib().vsim_set_self_contact(self._h, int(bool(enabled))))

    @property
    def gravity(self):
        return self._gravity

    @gravity.setter
    def gravity(self, g):
        self._gravity = tuple(float(v) for v in g)
        check(lib().vsim_set_gravity(self._h, dptr(np.asarray(self._gravity, np.float64))))

    @property
    def paused(self):
        return self._paused

    @paused.setter
    def paused(self, value):
        self._paused = bool(value)
        check(lib().vsim_set_paused(self._h, int(self._paused)))

    def set_step_duration(self, seconds: float):
        check(lib().vsim_set_step_duration(self._h, float(seconds)))

    def set_iterations(self, iterations: int):
        check(lib().vsim_set_iterations(self._h, int(iterations)))

    def set_graph(self, enabled: bool):
        check(lib().vsim_set_graph(self._h, int(bool(enabled))))

    def set_pdl(self, enabled: bool):
        check(lib().vsim_set_pdl(self._h, int(bool(enabled))))

    def set_gather_mapping(self, mapping: str):
        """'auto', 'warp' or 'thread' (vsim_set_gather_mapping)."""
        code = {"auto": 0, "warp": 1, "thread": 2}[mapping]
        check(lib().vsim_set_gather_mapping(self._h, code))

    def set_launch_shape(self, block: int, brick: int):
        check(lib().vsim_set_launch_shape(self._h, int(block), int(brick)))

    def set_cell_lanes(self, lanes: int):
        """Small colour passes with each cell over 1 or 4 lanes (vsim_set_cell_lanes)."""
        check(lib().vsim_set_cell_lanes(self._h, int(lanes)))

    def set_tma_pass(self, enabled: bool):
        """Large colour passes through TMA brick tiles (vsim_set_tma_pass)."""
        check(lib().vsim_set_tma_pass(self._h, int(bool(enabled))))

    def tune(self, frames: int = 3):
        block, brick = C.c_uint32(), C.c_uint32()
        check(lib().vsim_tune(self._h, int(frames), C.byref(block), C.byref(brick)))
        return int(block.value), int(brick.value)

    # -- readout --------------------------------------------------------------
    def stats(self) -> dict:
        s = _ffi.Stats()
        check(lib().vsim_get_stats(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def cfl_number(self) -> float:
        out = C.c_double()
        check(lib().vsim_cfl_number(self._h, C.byref(out)))
        return out.value

    def contact_pairs(self) -> np.ndarray:
        """Directed hits (record, other) of the current positions, sorted."""
        count = C.c_size_t()
        rc = lib().vsim_contact_pairs(self._h, None, 0, C.byref(count))
        if rc not in (_ffi.VSIM_OK, _ffi.VSIM_ERR_CAPACITY):
            check(rc)
        cap = max(int(count.value), 1)
        out = np.zeros((cap, 2), np.uint32)
        check(lib().vsim_contact_pairs(self._h, uptr(out), cap, C.byref(count)))
        out = out[: int(count.value)]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def contact_surface(self):
        count = C.c_size_t()
        lib().vsim_contact_surface(self._h, None, None, 0, C.byref(count))
        n = int(count.value)
        nodes, bodies = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        check(lib().vsim_contact_surface(self._h, uptr(nodes), uptr(bodies), n, C.byref(count)))
        return nodes, bodies

    def contact_census(self) -> dict:
        """The gather's work on the current positions (vsim_contact_census):
        live records, occupied buckets, visible candidates, and each contact
        kernel's device time in ms. Moves no node."""
        c = _ffi.ContactCensus()
        check(lib().vsim_contact_census(self._h, C.byref(c)))
        return {"records": int(c.records), "occupied_buckets": int(c.occupied_buckets),
                "candidates": int(c.candidates),
                "ms": dict(zip(("bin", "segment", "scatter", "order", "gather"), (float(v) for v in c.ms)))}

    # -- profiling --------------------------------------------------------------
    def profile_frame(self, steps: int, splats: bool = False, view_dir=(0.0, 0.0, -1.0)) -> dict:
        """One frame with every kernel group timed by CUDA events:
        {group: (milliseconds, launches)}."""
        prof = _ffi.Profile()
        v = np.asarray(view_dir, np.float32)
        check(lib().vsim_profile_frame(self._h, int(steps), int(bool(splats)), fptr(v), C.byref(prof)))
        return {k: (prof.ms[i], prof.launches[i]) for i, k in enumerate(_ffi.KINDS) if prof.launches[i]}

    def time_colour_passes(self, sweeps: int) -> float:
        """Milliseconds for `sweeps` x 8 colour passes run back to back
        (vsim_time_colour_passes); the state is left unchanged."""
        ms = C.c_float()
        check(lib().vsim_time_colour_passes(self._h, int(sweeps), C.byref(ms)))
        return float(ms.value)

    def color_counts(self) -> np.ndarray:
        out = np.zeros(8, np.uint32)
        check(lib().vsim_color_counts(self._h, uptr(out)))
        return out

    def frame_launches(self, steps: int) -> int:
        return int(lib().vsim_frame_launches(self._h, int(steps)))

    def splat_launches(self) -> int:
        return int(lib().vsim_splat_launches(self._h))

    # -- splats ----------------------------------------------------------------
    def bind_splats(self, body, means, quats, scales):
        means = np.ascontiguousarray(means, np.float32)
        quats = np.ascontiguousarray(quats, np.float32)
        scales = np.ascontiguousarray(scales, np.float32)
        check(lib().vsim_splats_bind(self._h, int(body), fptr(means), fptr(quats), fptr(scales),
                                     int(means.shape[0])))

    @property
    def splat_count(self) -> int:
        return int(lib().vsim_splats_count(self._h))

    def deform_splats(self, view_dir=(0.0, 0.0, -1.0)):
        v = np.asarray(view_dir, np.float32)
        check(lib().vsim_splats_deform(self._h, fptr(v)))

    def sort_splats(self):
        check(lib().vsim_splats_sort(self._h))

    def deform_splats_axes(self, view_dir=(0.0, 0.0, -1.0)):
        """deform_splats, plus each ellipsoid's rotation and axis lengths."""
        v = np.asarray(view_dir, np.float32)
        check(lib().vsim_splats_deform_axes(self._h, fptr(v)))

    def read_splat_axes(self):
        """(rotations (n, 4) xyzw, axis lengths (n, 3)) of the last deform_splats_axes."""
        n = self.splat_count
        rot = np.zeros((n, 4), np.float32)
        scale = np.zeros((n, 3), np.float32)
        check(lib().vsim_splats_read_axes(self._h, fptr(rot), fptr(scale), n))
        return rot, scale

    def read_splats(self, order: bool = True):
        n = self.splat_count
        means = np.zeros((n, 3), np.float32)
        cov = np.zeros((n, 6), np.float32)
        perm = np.zeros(n, np.uint32) if order else None
        check(lib().vsim_splats_read(self._h, fptr(means), fptr(cov), uptr(perm), n))
        return means, cov, perm
