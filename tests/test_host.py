"""CPU tests of libvsim's host side: the library loads and exports every
symbol its header declares; the fixed timestep clock and the material
arithmetic (no device work) behave like the reference's."""
import ctypes as C
import math

import numpy as np
import pytest


def test_exports_every_header_symbol(vsimlib):
    lib = vsimlib.lib()
    declared = vsimlib.header_symbols()
    assert len(declared) > 40
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing
    assert set(vsimlib.SIGNATURES) <= set(declared)
    assert lib.vsim_abi_version() == 1


def clock(vsimlib, duration, max_steps=0):
    h = C.c_void_p()
    rc = vsimlib.lib().vsim_clock_create(duration, max_steps, C.byref(h))
    return rc, h


def consume(vsimlib, h, elapsed, force=False):
    r = vsimlib.ClockReport()
    rc = vsimlib.lib().vsim_clock_consume(h, elapsed, int(force), C.byref(r))
    assert rc == 0
    return r


def snapshot(vsimlib, h):
    r = vsimlib.ClockReport()
    assert vsimlib.lib().vsim_clock_snapshot(h, C.byref(r)) == 0
    return r


def test_stable_step_duration(vsimlib):
    # timestep.test.js:20-28
    out = C.c_double()
    rate = 383.7879251340593
    assert vsimlib.lib().vsim_stable_step_duration(rate, C.byref(out)) == 0
    assert abs(out.value * rate - 0.75) < 5e-13
    assert out.value <= 1 / 240
    vsimlib.lib().vsim_stable_step_duration(0.0, C.byref(out))
    assert out.value == 1 / 240
    vsimlib.lib().vsim_stable_step_duration(1.0, C.byref(out))
    assert out.value == 1 / 240
    assert vsimlib.lib().vsim_stable_step_duration(-1.0, C.byref(out)) == vsimlib.VSIM_ERR_RANGE


def test_same_time_at_every_refresh(vsimlib):
    # timestep.test.js:30-42
    totals = set()
    for hz in (30, 38, 60, 144):
        rc, h = clock(vsimlib, 1 / 500)
        for _ in range(hz * 3):
            r = consume(vsimlib, h, 1 / hz)
            assert r.steps <= 24
        r = snapshot(vsimlib, h)
        assert abs(r.simulated_time - 3) < 5e-11
        assert abs(r.backlog_time) < 5e-11
        assert r.dropped_time == 0
        totals.add(r.total_steps)
        vsimlib.lib().vsim_clock_destroy(h)
    assert len(totals) == 1


def test_irregular_frames(vsimlib):
    # timestep.test.js:44-60
    rc, h = clock(vsimlib, 1 / 512)
    elapsed = 0
    for dt in (1 / 60, 1 / 58, 1 / 38, 1 / 60, 1 / 30, 1 / 144, 1 / 60):
        elapsed += dt
        r = consume(vsimlib, h, dt)
        assert r.step_duration == 1 / 512 and r.steps <= 24 and r.dropped_time == 0
    r = snapshot(vsimlib, h)
    assert abs(r.simulated_time + r.backlog_time - elapsed) < 5e-13


def test_long_stall(vsimlib):
    # timestep.test.js:62-73
    rc, h = clock(vsimlib, 0.002)
    r = consume(vsimlib, h, 0.2)
    assert r.steps == 24 and r.step_duration == 0.002 and r.overloaded
    assert abs(r.frame_dropped_time - 0.152) < 5e-13
    assert r.backlog_time < 0.002
    assert abs(r.simulated_time + r.backlog_time + r.dropped_time - 0.2) < 5e-13


def test_idle_and_single_step(vsimlib):
    # timestep.test.js:75-87
    rc, h = clock(vsimlib, 0.002)
    consume(vsimlib, h, 0.001)
    before = snapshot(vsimlib, h)
    r = vsimlib.ClockReport()
    vsimlib.lib().vsim_clock_idle(h, C.byref(r))
    assert r.backlog_time == before.backlog_time and r.simulated_time == before.simulated_time
    vsimlib.lib().vsim_clock_single_step(h, C.byref(r))
    assert r.steps == 1 and abs(r.simulated_time - 0.002) < 5e-13 and r.backlog_time == before.backlog_time


def test_force_step(vsimlib):
    # timestep.test.js:89-106
    rc, h = clock(vsimlib, 0.1)
    r = consume(vsimlib, h, 0.01, True)
    assert r.steps == 1 and abs(r.simulated_time - 0.1) < 5e-13 and abs(r.backlog_time - 0.01) < 5e-13
    rc, h = clock(vsimlib, 0.002)
    r = consume(vsimlib, h, 0.0025, True)
    assert r.steps == 1 and abs(r.backlog_time - 0.0005) < 5e-13


def test_step_duration_change_keeps_seconds(vsimlib):
    # timestep.test.js:108-118
    rc, h = clock(vsimlib, 0.004)
    consume(vsimlib, h, 0.003)
    assert vsimlib.lib().vsim_clock_set_step_duration(h, 0.001) == 0
    r = consume(vsimlib, h, 0.001)
    assert r.steps == 4 and abs(r.simulated_time - 0.004) < 5e-13 and abs(r.backlog_time) < 5e-13


def test_rejects_undefined_time(vsimlib):
    # timestep.test.js:120-127
    rc, h = clock(vsimlib, 0)
    assert rc == vsimlib.VSIM_ERR_RANGE
    rc, h = clock(vsimlib, 0.01)
    r = vsimlib.ClockReport()
    assert vsimlib.lib().vsim_clock_consume(h, math.inf, 0, C.byref(r)) == vsimlib.VSIM_ERR_RANGE
    assert b"elapsed" in vsimlib.lib().vsim_last_error()


def test_material_arithmetic(vsimlib):
    # material.js:101-108 and compliance.test.js:9-50
    m = vsimlib.Material(1.2e5, 0.10, 1000.0, 0.4, 0.6, 0.012, 0.0)
    mu, lam = C.c_double(), C.c_double()
    vsimlib.lib().vsim_lame_parameters(C.byref(m), C.byref(mu), C.byref(lam))
    nu = 0.25  # clamped
    assert abs(mu.value - 1.2e5 / (2 * (1 + nu))) < 1e-6
    assert abs(lam.value - 1.2e5 * nu / ((1 + nu) * (1 - 2 * nu))) < 1e-6
    d, hh, g = C.c_double(), C.c_double(), C.c_double()
    vsimlib.lib().vsim_element_compliance(C.byref(m), 0.02 ** 3, C.byref(d), C.byref(hh), C.byref(g))
    assert g.value < 4 and vsimlib.lib().vsim_collapse_scale(g.value) < 0.6
    soft = vsimlib.Material(1e4, 0.4, 1000.0, 0.4, 0.6, 0.012, 0.0)
    stiff = vsimlib.Material(1e6, 0.4, 1000.0, 0.4, 0.6, 0.012, 0.0)
    ds, dh = C.c_double(), C.c_double()
    vsimlib.lib().vsim_element_compliance(C.byref(stiff), 0.02 ** 3, C.byref(ds), C.byref(dh), C.byref(g))
    vsimlib.lib().vsim_element_compliance(C.byref(soft), 0.02 ** 3, C.byref(d), C.byref(hh), C.byref(g))
    assert ds.value < d.value and dh.value < hh.value
    speed = vsimlib.lib().vsim_wave_speed(C.byref(stiff))
    vsimlib.lib().vsim_lame_parameters(C.byref(stiff), C.byref(mu), C.byref(lam))
    assert abs(speed - math.sqrt((lam.value + 2 * mu.value) / 1000)) < 1e-9


def test_scene_generators():
    import vsim.scenes as sc

    s0 = sc.single_box()
    assert s0.bodies[0].node_count == 425 and s0.cells == 256
    assert s0.bodies[0].static_nodes.size == 25
    occ = sc.noise_occupancy(32, seed=3)
    assert 0.2 < occ.mean() < 0.8
    again = sc.noise_occupancy(32, seed=3)
    assert np.array_equal(occ, again)
    batch = sc.box_batch(16, seed=5)
    sides = np.array([b.cell_dims for b in batch.bodies])
    assert sides.min() >= 4 and sides.max() <= 48
    assert all(b.static_nodes.size > 0 for b in batch.bodies)
    means, quats, scales, opacity, rgb = sc.splats_in(s0.bodies[0], 1000, 9)
    assert np.allclose(np.linalg.norm(quats, axis=1), 1, atol=1e-6)
    assert scales.min() >= 1e-3 * 0.999 and scales.max() <= 1e-2 * 1.001
    lo = np.asarray(s0.bodies[0].origin)
    assert np.all(means >= lo - 1e-6) and np.all(means <= lo + np.array([16, 4, 4]) * sc.H + 1e-6)


# ---- material.test.js ----------------------------------------------------------------

def _lame(vsimlib, youngs, nu, density=1000.0):
    m = vsimlib.Material(youngs, nu, density, 0.4, 0.6, 0.012, 0.0)
    mu, lam = C.c_double(), C.c_double()
    assert vsimlib.lib().vsim_lame_parameters(C.byref(m), C.byref(mu), C.byref(lam)) == 0
    return mu.value, lam.value


def _engineering(mu, lam):
    """The inverse of the Lame conversion: E and nu."""
    return mu * (3 * lam + 2 * mu) / (lam + mu), lam / (2 * (lam + mu))


def test_material_round_trips_through_lame(vsimlib):
    # material.test.js:19-28
    for youngs in (1e4, 1.2e5, 5e6):
        for nu in (0.25, 0.3, 0.35, 0.4, 0.45, 0.49):
            e, n = _engineering(*_lame(vsimlib, youngs, nu))
            assert abs(e - youngs) < 0.05 and abs(n - nu) < 5e-9


def test_material_clamps_poisson_ratio(vsimlib):
    # material.test.js:30-43: finite, lambda > 0, nu back inside [0.25, 0.49]
    for nu in (-1.0, 0.0, 0.5, 0.99):
        mu, lam = _lame(vsimlib, 1e5, nu)
        assert math.isfinite(mu) and math.isfinite(lam) and lam > 0
        _, back = _engineering(mu, lam)
        assert 0.25 - 1e-9 <= back <= 0.49 + 1e-9


def test_material_wave_speed(vsimlib):
    # material.test.js:46-59
    def speed(youngs, density, nu=0.4):
        return vsimlib.lib().vsim_wave_speed(C.byref(vsimlib.Material(youngs, nu, density, 0.4, 0.6, 0.012, 0.0)))

    assert speed(1e7, 1000.0) > speed(1e5, 1000.0)
    assert speed(1e5, 4000.0) < speed(1e5, 1000.0)
    assert 5 < speed(1e5, 1000.0, 0.35) < 30


def _cuda_present():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


# The argument checks return before any device work; with a GPU present a
# broken check would launch on the made-up addresses below, so this runs only
# where there is none.
@pytest.mark.skipif(_cuda_present(), reason="made-up device addresses; argument checks are tested without a GPU")
def test_sort_entry_points_reject_bad_arguments(vsimlib):
    lib = vsimlib.lib()
    ok, rng_err, inv = vsimlib.VSIM_OK, vsimlib.VSIM_ERR_RANGE, vsimlib.VSIM_ERR_INVALID
    keys, order = 0x10000, 0x20000  # never dereferenced
    # the sort without allocation
    noalloc = lib.vsim_radix_sort_u32_noalloc
    assert noalloc(None, None, 0, 32, None) == ok  # nothing to sort
    assert noalloc(keys, order, 10, 0, None) == rng_err
    assert noalloc(keys, order, 10, 33, None) == rng_err
    assert noalloc(None, order, 10, 32, None) == inv
    assert noalloc(keys, None, 10, 32, None) == inv
    assert noalloc(keys, keys, 10, 32, None) == inv  # in place
    assert noalloc(keys, keys + 36, 10, 32, None) == inv  # order starts inside keys
    assert noalloc(keys + 36, keys, 10, 32, None) == inv  # keys start inside order
    assert b"overlap" in lib.vsim_last_error()
    # the allocating sort, past its size query
    need = C.c_size_t()
    assert lib.vsim_radix_sort_u32(None, None, 10, 32, None, C.byref(need), None) == ok
    temp = 0x30000
    sort = lib.vsim_radix_sort_u32
    assert sort(keys, order, 10, 0, temp, C.byref(need), None) == rng_err
    assert sort(None, order, 10, 32, temp, C.byref(need), None) == inv
    assert sort(keys, keys + 4, 10, 32, temp, C.byref(need), None) == inv
    assert b"overlap" in lib.vsim_last_error()


def test_package_gives_each_stream_a_hardware_queue():
    """Importing the package asks the CUDA driver for 32 hardware queues (the
    serving engine keeps ten streams busy; with the default eight a launch
    slot shares the ticks' queue) and keeps a value the caller set."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    pkg = str(Path(__file__).resolve().parent.parent / "visionary-sim_gb300")
    code = "import os, vsim._ffi; print(os.environ['CUDA_DEVICE_MAX_CONNECTIONS'])"
    env = {k: v for k, v in os.environ.items() if k != "CUDA_DEVICE_MAX_CONNECTIONS"}
    env["PYTHONPATH"] = pkg + os.pathsep + env.get("PYTHONPATH", "")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    assert out.stdout.strip() == "32"
    env["CUDA_DEVICE_MAX_CONNECTIONS"] = "1"
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    assert out.stdout.strip() == "1"
