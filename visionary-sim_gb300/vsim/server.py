"""Python surface of libvsim's session server (vsim_server_* in
include/vsim.h): a pool of sessions resident on the device, stepped in
shared frames with requests joining at every frame boundary."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import check, fptr, lib
from .scenes import Descs, Scene


class Server:
    def __init__(self, bodies, tank, budget_bytes: float = 150e9, step_duration: float = 1 / 600,
                 substeps: int = 10, self_contact: bool = True, stream=None):
        self._descs = Descs(Scene(list(bodies), tank))
        cfg = _ffi.ServerConfig(float(budget_bytes), float(step_duration), int(substeps), int(bool(self_contact)))
        handle = C.c_void_p()
        check(lib().vsim_server_create(self._descs.bodies, self._descs.count, C.byref(self._descs.tank),
                                       C.byref(cfg), C.c_void_p(stream), C.byref(handle)))
        self._h = handle
        self.bodies = list(bodies)
        self._buf = (_ffi.Completion * 4096)()

    @property
    def admitted(self) -> int:
        """How many sessions are resident (vsim_server_admitted)."""
        return int(lib().vsim_server_admitted(self._h))

    def destroy(self):
        if self._h:
            lib().vsim_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def clock(self) -> float:
        return float(lib().vsim_server_clock(self._h))

    @property
    def resident(self) -> list:
        """The resident sessions, in device-pool order (vsim_server_resident)."""
        count = C.c_uint32()
        check(lib().vsim_server_resident(self._h, None, 0, C.byref(count)))
        out = np.zeros(count.value, np.uint32)
        check(lib().vsim_server_resident(self._h, out.ctypes.data_as(C.POINTER(C.c_uint32)), count.value,
                                         C.byref(count)))
        return [int(v) for v in out]

    def set_resident(self, sessions):
        """Make exactly `sessions` resident (vsim_server_set_resident): sessions
        leaving are checkpointed on the host, sessions returning resume from
        their checkpoint."""
        ids = np.ascontiguousarray(np.asarray(list(sessions), np.uint32))
        check(lib().vsim_server_set_resident(self._h, ids.ctypes.data_as(C.POINTER(C.c_uint32)), int(ids.size)))

    def submit(self, session: int, frames: int, drag=None) -> int:
        """Queue `frames` frames for `session`; drag = (node, control 4x3, speed)."""
        rid = C.c_uint64()
        d = None
        if drag is not None:
            node, control, speed = drag
            d = _ffi.Drag()
            d.node = int(node)
            ctl = np.asarray(control, np.float32).reshape(4, 3)
            for i in range(4):
                for a in range(3):
                    d.control[i][a] = float(ctl[i, a])
            d.speed = float(speed)
        check(lib().vsim_server_submit(self._h, int(session), int(frames), C.byref(d) if d is not None else None,
                                       C.byref(rid)))
        return int(rid.value)

    def set_tick_budget(self, cells: int):
        """Cap the occupied cells one tick steps (0: no cap); see
        vsim_server_set_tick_budget."""
        check(lib().vsim_server_set_tick_budget(self._h, int(cells)))

    FRAMES, SESSIONS = 0, 1

    def set_engine(self, engine: int, block_cells: int = 32, cluster_cells: int = 512):
        """How run() executes requests (vsim_server_set_engine): FRAMES,
        ticks of shared frames; SESSIONS, a session whose largest colour has
        at most `block_cells` cells runs each request whole in one block of
        the session kernel, at most `cluster_cells` in one cluster, the rest
        in ticks alongside."""
        check(lib().vsim_server_set_engine(self._h, int(engine), int(block_cells), int(cluster_cells)))

    def run(self, arrivals, sessions, frames, drag_flags, drags=None, closed_loop_seconds: float = 0.0,
            keep: int | None = None):
        """The library's request loop (vsim_server_run) over a schedule:
        arrival times (seconds from the start), sessions, frames, drag flags,
        and per-session drags [(node, control 4x3, speed)] indexed by session
        id (None: no drags). Returns (completions as dicts, report dict)."""
        n = len(frames)
        if keep is None:
            keep = n if closed_loop_seconds == 0 else 0
        reqs = (_ffi.ScheduledRequest * max(n, 1))()
        for i in range(n):
            reqs[i].arrival = float(arrivals[i]) if arrivals is not None else 0.0
            reqs[i].session = int(sessions[i]) if sessions is not None else i % max(1, self.admitted)
            reqs[i].frames = int(frames[i])
            reqs[i].drag = int(bool(drag_flags[i]))
        table = None
        if drags is not None:
            table = (_ffi.Drag * len(drags))()
            for k, d in enumerate(drags):
                if d is None:
                    continue
                node, control, speed = d
                table[k].node = int(node)
                ctl = np.asarray(control, np.float32).reshape(4, 3)
                for i in range(4):
                    for a in range(3):
                        table[k].control[i][a] = float(ctl[i, a])
                table[k].speed = float(speed)
        out = (_ffi.Completion * keep)() if keep > 0 else None
        report = _ffi.RunReport()
        check(lib().vsim_server_run(self._h, reqs, n, table, float(closed_loop_seconds), out, keep,
                                    C.byref(report)))
        done = [{"request": out[i].request, "session": out[i].session, "frames": out[i].frames,
                 "submitted": out[i].submitted, "completed": out[i].completed, "first_tick": out[i].first_tick,
                 "last_tick": out[i].last_tick} for i in range(report.returned)]
        return done, {name: getattr(report, name) for name, _ in report._fields_ if name != "pad"}

    def tick(self) -> int:
        stepped = C.c_uint32()
        check(lib().vsim_server_tick(self._h, C.byref(stepped)))
        return int(stepped.value)

    def poll(self) -> list:
        out = []
        while True:
            n = C.c_uint32()
            check(lib().vsim_server_poll(self._h, self._buf, len(self._buf), C.byref(n)))
            for i in range(n.value):
                c = self._buf[i]
                out.append({"request": c.request, "session": c.session, "frames": c.frames,
                            "submitted": c.submitted, "completed": c.completed, "first_tick": c.first_tick,
                            "last_tick": c.last_tick})
            if n.value < len(self._buf):
                return out

    def stats(self) -> dict:
        s = _ffi.ServerStats()
        check(lib().vsim_server_get_stats(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def read_positions(self, session: int) -> np.ndarray:
        n = int(lib().vsim_server_node_count(self._h, int(session)))
        out = np.zeros((n, 4), np.float32)
        check(lib().vsim_server_read_positions(self._h, int(session), fptr(out), n))
        return out

    def read_state(self, session: int):
        """(pos, prev, vel) of one session, (n, 4) float32 each, w = 0."""
        n = int(lib().vsim_server_node_count(self._h, int(session)))
        out = [np.zeros((n, 4), np.float32) for _ in range(3)]
        check(lib().vsim_server_read_state(self._h, int(session), fptr(out[0]), fptr(out[1]), fptr(out[2]), n))
        return tuple(out)

    def write_state(self, session: int, pos, prev, vel):
        """Restore a checkpoint of an idle session (read_state's arrays)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (pos, prev, vel)]
        check(lib().vsim_server_write_state(self._h, int(session), fptr(arrs[0]), fptr(arrs[1]), fptr(arrs[2]),
                                            arrs[0].shape[0]))

    def reset_session(self, session: int):
        """An idle session back to its rest state."""
        check(lib().vsim_server_reset_session(self._h, int(session)))

