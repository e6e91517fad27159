"""GPU parity: libvsim's kernels against the float CPU oracle, through the C
ABI, frame by frame from one shared state.

The kernels evaluate every operation in the oracle's order, fusing a
multiply and an add exactly where the oracle does and rounding everything
else once, so the expected agreement is exact equality (`==`: -0 and +0
compare equal). The configured tolerance -- 1e-5 relative,
max_i |x_gpu - x_oracle| / max(|x_oracle|, L_body) -- is asserted as well, so
a failure reports both how far apart and whether the bar itself is met.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def lib(vsimlib, gpu):
    return vsimlib


def rel_error(gpu_pos, ref_pos, scene):
    """max_i |x_gpu - x_oracle| / max(|x_oracle|_inf, L_body), per body."""
    worst = 0.0
    at = 0
    for b in scene.bodies:
        n = b.node_count
        g = gpu_pos[at:at + n, :3].astype(np.float64)
        r = ref_pos[at:at + n, :3].astype(np.float64)
        diag = float(np.linalg.norm(np.asarray(b.cell_dims) * b.h))
        scale = max(float(np.max(np.abs(r))), diag)
        worst = max(worst, float(np.max(np.abs(g - r))) / scale)
        at += n
    return worst


def assert_same(sim, orc, scene, what=""):
    gp, gq, gv = sim.read_state()
    op, oq, ov = orc.state()
    err = rel_error(gp, op, scene)
    assert err <= TOL, f"{what}: relative position error {err:.3e}"
    for name, g, o in (("pos", gp, op), ("prev", gq, oq), ("vel", gv, ov)):
        bad = np.flatnonzero(np.any(g != o, axis=1))
        assert bad.size == 0, (f"{what}: {name} differs at {bad.size} nodes, first {bad[:5]}, "
                               f"max |diff| {np.max(np.abs(g - o)):.3e}")


def make(scene):
    import pyoracle
    from vsim import Simulator

    return Simulator(scene), pyoracle.Oracle(scene, 32)


def test_single_box_frames_bit_exact(lib):
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, orc = make(scene)
    assert np.array_equal(sim.inv_mass, orc.inv_mass())
    for frame in range(40):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    sim.destroy()


@pytest.mark.parametrize("graph,pdl", [(False, False), (False, True), (True, False)])
def test_launch_modes_agree(lib, graph, pdl):
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, orc = make(scene)
    sim.set_graph(graph)
    sim.set_pdl(pdl)
    for frame in range(5):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, f"graph={graph} pdl={pdl}")


def test_blob_contact_self_contact(lib):
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=3, splats=0)
    sim, orc = make(scene)
    nodes_g, bodies_g = sim.contact_surface()
    nodes_o, bodies_o = orc.surface()
    assert np.array_equal(nodes_g, nodes_o) and np.array_equal(bodies_g, bodies_o)
    for frame in range(20):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    assert sim.read_positions()[:, 1].min() > -0.01  # the ground held


def test_large_colour_passes_stream_bit_exact(lib):
    """A body whose colour passes exceed 155,648 cells (two cells per resident
    thread: 4 blocks of 128 on each of 152 SMs), so the streaming colour pass
    runs; one frame with ground contact, compared node for node."""
    import vsim.scenes as sc

    nx, ny, nz = 128, 96, 128  # 1,572,864 cells, 196,608 per colour
    mat = dict(sc.DEFAULT_MATERIAL, youngs_modulus=2e5, poisson_ratio=0.45, density=1000.0)
    body = sc.Body((nx, ny, nz), (0.0, 2 * sc.H, 0.0), sc.H, np.ones(nx * ny * nz, np.uint8), mat)
    ext = (nx * sc.H, (ny + 4) * sc.H, nz * sc.H)
    scene = sc.Scene([body], ((-0.1, 0.0, -0.1), (ext[0] + 0.1, ext[1] + 0.1, ext[2] + 0.1)),
                     step_duration=1 / 600, substeps=10)
    sim, orc = make(scene)
    assert min(sim.color_counts()) >= 155_648
    sim.dispatch(scene.substeps)
    orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, "streamed frame")


def test_cell_split_over_four_lanes_bit_exact(lib):
    """The small colour passes with each cell split over four lanes
    (vsim_set_cell_lanes) equal the oracle frame by frame: a noise blob with
    ground and self contact, and the pinned bar with a stretch limit."""
    import vsim.scenes as sc

    blob = sc.noise_blob(n=16, seed=5, splats=0)
    sim, orc = make(blob)
    sim.set_cell_lanes(4)
    for frame in range(6):
        sim.dispatch(blob.substeps)
        orc.dispatch(blob.substeps)
        assert_same(sim, orc, blob, f"blob frame {frame}")
    bar = sc.single_box()
    bar.bodies[0].material["max_stretch"] = 1.05
    sim, orc = make(bar)
    sim.set_cell_lanes(4)
    for frame in range(4):
        sim.dispatch(bar.substeps)
        orc.dispatch(bar.substeps)
        assert_same(sim, orc, bar, f"bar frame {frame}")


def test_tma_colour_pass_bit_exact(lib):
    """The TMA brick form of the large colour passes (vsim_set_tma_pass)
    leaves every node where the streaming form leaves it: a dense box whose
    cell grid is no multiple of a brick (boxes reaching past the node grid)
    and a noise blob (bricks partly empty), one frame with ground and self
    contact each, synchronised with the fault word checked. More than four
    bodies are refused."""
    import vsim.scenes as sc
    from vsim import _ffi
    from vsim.simulator import Simulator

    mat = dict(sc.DEFAULT_MATERIAL, youngs_modulus=2e5, poisson_ratio=0.45, density=1000.0)
    nx, ny, nz = 130, 90, 135  # 1,579,500 cells
    box = sc.Body((nx, ny, nz), (0.0, 2 * sc.H, 0.0), sc.H, np.ones(nx * ny * nz, np.uint8), mat)
    ext = (nx * sc.H, (ny + 4) * sc.H, nz * sc.H)
    dense = sc.Scene([box], ((-0.1, 0.0, -0.1), (ext[0] + 0.1, ext[1] + 0.1, ext[2] + 0.1)),
                     step_duration=1 / 600, substeps=10)
    blob = sc.noise_blob(n=160, seed=4, splats=0)
    for name, scene in (("dense box", dense), ("noise blob", blob)):
        plain, tiled = Simulator(scene), Simulator(scene)
        tiled.set_tma_pass(True)
        assert min(tiled.color_counts()) >= 155_648, name
        for sim in (plain, tiled):
            sim.dispatch(scene.substeps)
            sim.synchronize()
        for a, b, what in zip(plain.read_state(), tiled.read_state(), ("pos", "prev", "vel")):
            assert np.array_equal(a, b), f"{name}: {what}"
        plain.destroy()
        tiled.destroy()
    many = Simulator(sc.box_batch(5))
    with pytest.raises(_ffi.VsimError):
        many.set_tma_pass(True)
    many.destroy()


@pytest.mark.parametrize("mapping", ["warp", "thread"])
def test_gather_mappings_agree(lib, mapping):
    """Both record-to-thread mappings of the contact gather give the oracle's
    result, on a state squeezed into heavy self contact."""
    import vsim.scenes as sc

    scene = sc.noise_blob(n=20, seed=5, splats=0)
    sim, orc = make(scene)
    sim.set_gather_mapping(mapping)
    pos, prev, vel = orc.state()
    squashed = squeeze(pos, scene, 0.5)
    sim.write_state(squashed, pos, vel)
    orc.set_state(squashed, pos, vel)
    assert np.array_equal(sim.contact_pairs(), orc.contact_pairs())
    for frame in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"{mapping} frame {frame}")


def squeeze(pos, scene, factor=0.6):
    """A shared state with overlapping surfaces: every body squashed toward
    its own bottom plane."""
    out = pos.copy()
    at = 0
    for b in scene.bodies:
        n = b.node_count
        y0 = b.origin[1]
        out[at:at + n, 1] = y0 + (out[at:at + n, 1] - y0) * factor
        at += n
    return out


def test_contact_pairs_bit_exact(lib):
    import vsim.scenes as sc

    scene = sc.noise_blob(n=20, seed=5, splats=0)
    sim, orc = make(scene)
    pos, prev, vel = orc.state()
    squashed = squeeze(pos, scene, 0.4)
    for s in (sim, orc):
        s.write_state(squashed, pos, vel) if s is sim else s.set_state(squashed, pos, vel)
    gp = sim.contact_pairs()
    op = orc.contact_pairs()
    assert op.shape[0] > 100
    assert np.array_equal(gp, op)
    sim.dispatch(scene.substeps)
    orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, "after squeeze")


def test_two_bodies_contact(lib):
    """Inter-body contact as the reference has it: a box dropped on another."""
    import vsim.scenes as sc

    a = sc.Body((8, 4, 8), (0.0, 0.0, 0.0), sc.H, np.ones(256, np.uint8), dict(sc.DEFAULT_MATERIAL))
    b = sc.Body((6, 4, 6), (0.01, 4 * sc.H + 0.004, 0.012), sc.H, np.ones(144, np.uint8),
                dict(sc.DEFAULT_MATERIAL, density=600.0, friction=0.2))
    scene = sc.Scene([a, b], ((-0.5, 0.0, -0.5), (0.5, 1.0, 0.5)), step_duration=1 / 1200, substeps=20)
    sim, orc = make(scene)
    pairs = sim.contact_pairs()
    assert np.array_equal(pairs, orc.contact_pairs())
    for frame in range(15):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    assert len(sim.contact_pairs()) > 0


def test_box_batch_frames(lib):
    import vsim.scenes as sc

    scene = sc.box_batch(12, seed=7)
    sim, orc = make(scene)
    for frame in range(8):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")


def test_iterations_and_stretch(lib):
    import vsim.scenes as sc

    scene = sc.single_box()
    scene.iterations = 2
    scene.bodies[0].material["max_stretch"] = 1.05
    sim, orc = make(scene)
    for frame in range(10):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")


def grab_velocity(pos, prev_pos, steps, dt):
    return [(pos[a] - prev_pos[a]) / (steps * dt) for a in range(3)]


@pytest.mark.parametrize("law", ["hard", "compliant"])
def test_drive_laws(lib, law):
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, orc = make(scene)
    sim.set_drive_law(law)
    orc.set_drive_law(law)
    dims = scene.bodies[0].node_dims
    tip = [sc.node_index(dims, 16, j, k) for j in range(5) for k in range(5)]
    rest = sim.read_positions()
    anchor = rest[tip[0], :3].astype(np.float64)
    offsets = (rest[tip, :3] - rest[tip[0], :3]).astype(np.float32)
    sim.hold(tip, offsets)
    assert orc.hold(tip, offsets) == 0
    sim.place_grab(anchor)
    target = anchor.copy()
    previous = anchor.copy()
    dt = scene.step_duration
    for frame in range(12):
        target = target + np.array([0.0, 0.004, 0.002])
        sim.move_grab(target)
        orc.set_grab(target, grab_velocity(target, previous, scene.substeps, dt))
        previous = target.copy()
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"{law} frame {frame}")
    sim.release_grab()
    orc.release()
    for frame in range(4):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, f"{law} after release")


@pytest.mark.parametrize("strategy", ["singleNode", "withinRadius"])
def test_device_grab_matches_host_grab(lib, strategy):
    """vsim_grab (pick and grip on the device) holds what pick.js / grip.js
    pick and grip from read-back positions: same anchor, same held set and
    offsets (the next frames equal the oracle holding the host's set), and a
    ray that misses holds nothing."""
    import vsim.scenes as sc
    from vsim import simulator as vs

    scene = sc.noise_blob(n=16, seed=3, splats=0)
    sim, orc = make(scene)
    for _ in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    sim.set_grip(strategy)
    sim.set_grip_radius(0.03)
    nodes = sim.read_positions()
    centre = nodes[np.asarray(sim.inv_mass) > 0, :3].mean(axis=0).astype(np.float64)
    origin = centre + np.array([0.05, 0.6, 0.1])
    direction = (centre - origin) / np.linalg.norm(centre - origin)

    aim = max(b.h for b in scene.bodies) * 1.2
    anchor = vs.nearest_node_to_ray(nodes, sim.inv_mass, origin, direction, aim, sim.static)
    assert anchor >= 0
    if strategy == "singleNode":
        held, offs, found = vs.single_node(nodes, sim.inv_mass, anchor, sim.static)
    else:
        held, offs, found = vs.within_radius(nodes, sim.inv_mass, anchor, 0.03, sim.offsets, sim.static, 4096)
    got = sim.grab(origin, direction)
    assert got["anchor"] == anchor and got["held"] == len(held) and got["found"] == found
    assert got["position"] == [float(v) for v in nodes[anchor, :3]]
    assert orc.hold(np.asarray(held, np.uint32), np.asarray(offs, np.float32).reshape(-1, 3)) == 0
    target = np.asarray(got["position"], np.float64)
    previous = target.copy()
    for frame in range(4):
        target = target + np.array([0.0, 0.003, 0.001])
        sim.move_grab(target)
        orc.set_grab(target, grab_velocity(target, previous, scene.substeps, scene.step_duration))
        previous = target.copy()
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"{strategy} frame {frame}")
    sim.release_grab()
    assert sim.grab(origin, -direction) is None


def test_errors_map_to_reference_throws(lib):
    import vsim.scenes as sc
    from vsim import VsimError, VsimRangeError

    scene = sc.single_box()
    sim, _ = make(scene)
    with pytest.raises(VsimError) as info:
        sim.hold([0], np.zeros((1, 3)))  # node 0 is on the pinned face
    assert info.value.code == lib.VSIM_ERR_INVALID
    with pytest.raises(VsimRangeError):
        sim.set_drive_response_time(-1.0)
    with pytest.raises(VsimRangeError):
        sim.set_material(0, {"max_stretch": 0.5})
    with pytest.raises(VsimError):
        sim.set_drive_law("sticky")
    sim.step(float("nan"))  # garbage dt is a frame of no time
    assert sim.stats()["last_steps"] == 0


def test_material_change_midrun(lib):
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, orc = make(scene)
    for frame in range(3):
        sim.dispatch(10)
        orc.dispatch(10)
    change = {"density": 1500.0, "youngs_modulus": 3e5, "damping": 1.0}
    sim.set_material(0, change)
    orc.set_material(0, change)
    sim.set_step_duration(1 / 600)  # keep the fixed step of the workload
    orc.set_step_duration(1 / 600)
    assert np.array_equal(sim.inv_mass, orc.inv_mass())
    for frame in range(5):
        sim.dispatch(10)
        orc.dispatch(10)
        assert_same(sim, orc, scene, f"after change {frame}")


def test_state_io_through_pinned_and_pageable_buffers(lib, gpu):
    """Node state written from and read into page-locked host buffers
    (asynchronous copies) equals the same through pageable numpy buffers
    (copies the driver stages): a frame from a written state, then every
    array read back both ways, bit for bit."""
    import torch
    import vsim.scenes as sc
    from vsim._ffi import check, fptr

    scene = sc.noise_blob(n=12, seed=7, splats=0)
    a, b = make(scene)[0], make(scene)[0]
    for _ in range(3):
        a.dispatch(scene.substeps)
    state = a.read_state()
    n = a.node_count
    pinned = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(6)]
    for t, arr in zip(pinned[:3], state):
        t.numpy()[:] = arr
    L = lib.lib()
    check(L.vsim_write_state(b.handle, *(fptr(t.numpy()) for t in pinned[:3]), n))  # pinned in
    a.write_state(*state)  # pageable in (same values)
    a.dispatch(scene.substeps)
    b.dispatch(scene.substeps)
    check(L.vsim_read_state(b.handle, *(fptr(t.numpy()) for t in pinned[3:]), n))  # pinned out
    for x, y in zip(a.read_state(), pinned[3:]):  # pageable out
        assert np.array_equal(x, y.numpy())
    check(L.vsim_read_positions(b.handle, fptr(pinned[3].numpy()), n))
    assert np.array_equal(a.read_positions(), pinned[3].numpy())
    assert np.all(pinned[3].numpy()[:, 3] == 0)


def test_timing_colour_passes_leaves_state(lib):
    """vsim_time_colour_passes restores what the timed passes moved: the
    next frame still equals the oracle's."""
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=3, splats=0)
    sim, orc = make(scene)
    for _ in range(2):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    before = sim.read_state()
    assert sim.time_colour_passes(3) > 0
    after = sim.read_state()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    sim.dispatch(scene.substeps)
    orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, "after timing")


def test_run_twice_identical(lib):
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=11, splats=0)
    out = []
    for _ in range(2):
        sim, _o = make(scene)
        for _f in range(5):
            sim.dispatch(scene.substeps)
        out.append(sim.read_positions())
        sim.destroy()
    assert np.array_equal(out[0], out[1])


def test_reset_and_step_clock(lib):
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, _ = make(scene)
    rest = sim.read_positions()
    sim.step(1 / 60)
    st = sim.stats()
    assert st["last_steps"] == 10 and abs(st["step_duration"] - 1 / 600) < 1e-15
    assert not np.array_equal(sim.read_positions(), rest)
    sim.reset()
    assert np.array_equal(sim.read_positions(), rest)
    assert sim.stats()["steps"] == 0


def test_splats_and_sort(lib):
    import pyoracle
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=2, splats=20000)
    sim, orc = make(scene)
    for frame in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    view = (0.3, -0.2, -0.93)
    sim.deform_splats(view)
    sim.sort_splats()
    means, cov, order = sim.read_splats()
    m, q, s, *_ = scene.splats[0]
    om, oc, keys = orc.splat_deform(0, m, q, s, view)
    assert np.array_equal(means, om)
    assert np.array_equal(cov, oc)
    assert np.array_equal(order, pyoracle.stable_sort(keys))


def test_splat_axes(lib):
    """The fused ellipsoid decomposition equals the oracle's float evaluation
    of the same covariances, and leaves means, covariances and keys as the
    plain deformation writes them."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=2, splats=20000)
    sim, orc = make(scene)
    for frame in range(3):
        sim.dispatch(scene.substeps)
    view = (0.3, -0.2, -0.93)
    sim.deform_splats(view)
    sim.sort_splats()
    means, cov, order = sim.read_splats()
    sim.deform_splats_axes(view)
    sim.sort_splats()
    means2, cov2, order2 = sim.read_splats()
    assert np.array_equal(means, means2) and np.array_equal(cov, cov2) and np.array_equal(order, order2)
    rot, scale = sim.read_splat_axes()
    orot, oscale = pyoracle.ellipsoid_axes_f32(cov)
    assert np.array_equal(rot, orot)
    assert np.array_equal(scale, oscale)
    assert np.all(np.abs(np.linalg.norm(rot.astype(np.float64), axis=1) - 1) < 1e-6)


def test_captured_cloud_body(lib):
    """A Gaussian cloud voxelised by the reference's cloud path (stamp, seal,
    fill) steps as a body, and its own Gaussians deform and sort through the
    cells they were stamped into, equal to the oracle."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.captured_cloud(count=50_000, radius=0.08, element_size=0.008)
    sim, orc = make(scene)
    for frame in range(4):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    view = (0.0, -0.6, -0.8)
    sim.deform_splats(view)
    sim.sort_splats()
    means, cov, order = sim.read_splats()
    m, q, s, *_ = scene.splats[0]
    om, oc, keys = orc.splat_deform(0, m, q, s, view)
    assert np.array_equal(means, om)
    assert np.array_equal(cov, oc)
    assert np.array_equal(order, pyoracle.stable_sort(keys))


# 2^20 keys fill exactly 256 tiles of the histogram, 1.1M keys go past it;
# past ~4.2M keys (64 scan chunks) the scan takes three launches a pass
@pytest.mark.parametrize("n,bits", [(1, 32), (4095, 32), (4097, 8), (1_000_003, 32), (300_000, 20), (1 << 20, 32),
                                    (1_100_000, 32), (4_500_000, 32)])
def test_radix_sort_matches_stable_sort(lib, gpu, n, bits):
    import torch
    import pyoracle

    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[n // 2] if n > 2 else keys[: n // 3]  # many duplicates
    dk = torch.from_numpy(keys.view(np.int32)).to(gpu)
    do = torch.empty(n, dtype=torch.int32, device=gpu)
    need = C.c_size_t()
    L = lib.lib()
    assert L.vsim_radix_sort_u32(dk.data_ptr(), do.data_ptr(), n, bits, None, C.byref(need), None) == 0
    temp = torch.empty(need.value, dtype=torch.uint8, device=gpu)
    stream = torch.cuda.current_stream().cuda_stream
    assert L.vsim_radix_sort_u32(dk.data_ptr(), do.data_ptr(), n, bits, temp.data_ptr(), C.byref(need), stream) == 0
    torch.cuda.synchronize()
    got = do.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, pyoracle.stable_sort(keys, bits))
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), keys)  # input untouched


def test_scene_with_no_bodies(lib):
    """A scene can be all backdrop (simulator.js:162-187): nothing steps, no
    body limits the CFL, and every call still answers."""
    import vsim.scenes as sc

    scene = sc.Scene([], ((-1.0, 0.0, -1.0), (1.0, 1.0, 1.0)), step_duration=1 / 600, substeps=10)
    sim, orc = make(scene)
    assert sim.node_count == 0
    sim.dispatch(10)
    sim.step(1 / 60)
    sim.synchronize()
    assert sim.read_positions().shape == (0, 4)
    st = sim.stats()
    assert st["body_count"] == 0 and st["limited_by"] == -1 and st["cells"] == 0
    assert sim.contact_pairs().shape[0] == 0
    sim.reset()
    sim.destroy()


def test_degenerate_bodies_dispatch_zero_and_pause(lib):
    """A body with no occupied cell beside a normal one and a body whose
    every node is static: frames equal the oracle and the static body never
    moves; dispatch(0) changes nothing; a paused simulator takes a step only
    when one is requested (simulator.js:239-318)."""
    import vsim.scenes as sc

    live = sc.Body((4, 4, 4), (0.0, 0.02, 0.0), sc.H, np.ones(64, np.uint8))
    empty = sc.Body((3, 3, 3), (0.2, 0.02, 0.0), sc.H, np.zeros(27, np.uint8))
    pinned = sc.Body((4, 4, 4), (0.4, 0.02, 0.0), sc.H, np.ones(64, np.uint8),
                     static_nodes=np.arange(125, dtype=np.uint32))
    scene = sc.Scene([live, empty, pinned], ((-1.0, 0.0, -1.0), (1.0, 1.0, 1.0)), step_duration=1 / 600,
                     substeps=10)
    sim, orc = make(scene)
    rest = sim.read_positions()
    sim.dispatch(0)
    assert np.array_equal(sim.read_positions(), rest)
    for frame in range(5):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    first = sim.offsets[2]
    assert np.array_equal(sim.read_positions()[first:first + 125], rest[first:first + 125])
    sim.paused = True
    before = sim.read_positions()
    sim.step(1 / 60)
    assert np.array_equal(sim.read_positions(), before)
    sim.request_step()
    sim.step(1 / 60)
    orc.dispatch(1)
    assert_same(sim, orc, scene, "requested step while paused")


@pytest.mark.parametrize("block,brick", [(128, 0), (512, 4), (256, 8)])
def test_launch_shapes_agree(lib, block, brick):
    """Every elastic block size and cell order (lattice order, 4^3 and 8^3
    bricks) the autotuner chooses from gives the oracle's frames: cells of
    one colour share no node, so their order cannot change a result."""
    import vsim.scenes as sc

    scene = sc.box_batch(12, seed=7)
    sim, orc = make(scene)
    sim.set_launch_shape(block, brick)
    for frame in range(4):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"block {block} brick {brick} frame {frame}")


def test_tune_keeps_state(lib):
    """vsim_tune times every shape on the live state, puts the state back,
    and keeps a valid shape; frames afterwards equal the oracle's."""
    import vsim.scenes as sc

    scene = sc.box_batch(12, seed=7)
    sim, orc = make(scene)
    for frame in range(2):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    before = sim.read_state()
    block, brick = sim.tune(1)
    assert block in (128, 256, 512) and brick in (0, 4, 8)
    for a, b in zip(before, sim.read_state()):
        assert np.array_equal(a, b)
    for frame in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"after tuning, frame {frame}")


def test_gravity_and_contact_switched_midrun(lib):
    """params.gravity and setContact (simulator.js:60-66, 470-480) changed
    between frames: the blob's frames equal the oracle's with the same
    switches -- contact off and on again, self contact off, sideways
    gravity."""
    import vsim.scenes as sc

    scene = sc.noise_blob(n=16, seed=3, splats=0)
    sim, orc = make(scene)
    steps = [("frames", 3), ("contact", False), ("frames", 2), ("contact", True), ("self", False),
             ("frames", 2), ("gravity", (2.0, -4.0, 1.0)), ("frames", 3), ("self", True), ("frames", 2)]
    for what, arg in steps:
        if what == "contact":
            sim.set_contact(arg)
            orc.set_contact(arg)
        elif what == "self":
            sim.set_self_contact(arg)
            orc.set_self_contact(arg)
        elif what == "gravity":
            sim.gravity = arg
            orc.set_gravity(arg)
        else:
            for frame in range(arg):
                sim.dispatch(scene.substeps)
                orc.dispatch(scene.substeps)
                assert_same(sim, orc, scene, f"{what} {frame}")


@pytest.mark.parametrize("law", ["hard", "compliant"])
def test_grab_respects_static_material(lib, law):
    """staticPrescription.test.js:104-149 on the device: a sphere (radius
    0.04 m, 0.02 m cells) whose z < 0 half is static. A ray along +z from
    z = -0.2 grabs past the static material (the anchor has z >= 0) and
    holds several nodes within the grip radius; a single-node grip holds
    one; frames under the drag leave every static node where it rests; a
    body that is static everywhere is missed."""
    import vsim.scenes as sc
    from vsim import Simulator
    from vsim import voxelize as vz

    grid = vz.voxelize_sdf(vz.sphere(0.04), 0.02)
    base = sc.Body(tuple(grid.dims), tuple(grid.origin), grid.h, grid.occupancy)
    tank = ((-0.2, -0.2, -0.2), (0.2, 0.2, 0.2))
    body = sc.with_static_region(base, lambda x, y, z: z < 0)
    assert 0 < body.static_nodes.size < body.node_count
    sim = Simulator(sc.Scene([body], tank, contact=False))
    sim.set_drive_law(law)
    rest = sim.read_positions()
    hit = sim.grab((0.0, 0.0, -0.2), (0.0, 0.0, 1.0))
    assert hit is not None and hit["held"] > 1 and hit["position"][2] >= 0
    statics = body.static_nodes.astype(np.int64)
    near = np.linalg.norm(rest[statics, :3] - np.asarray(hit["position"], np.float32), axis=1)
    assert np.any((sim.inv_mass[statics] > 0) & (near < sim.grip["radius"]))  # static material was within reach
    for _ in range(3):
        sim.move_grab(np.asarray(hit["position"]) + [0.0, 0.01, 0.0])
        sim.dispatch(10)
    assert np.array_equal(sim.read_positions()[statics], rest[statics])
    sim.release_grab()
    sim.set_grip("singleNode")
    assert sim.grab((0.0, 0.0, -0.2), (0.0, 0.0, 1.0))["held"] == 1
    sim.destroy()

    pinned = sc.with_static_region(base, lambda x, y, z: True)
    sim = Simulator(sc.Scene([pinned], tank, contact=False))
    sim.set_drive_law(law)
    assert sim.grab((0.0, 0.0, -0.2), (0.0, 0.0, 1.0)) is None
    sim.destroy()


def test_simulator_timing(lib):
    """simulatorTiming.test.js:23-150 through vsim_step and the stats, on the
    pinned bar with a 0.002 s step: render dt becomes a count of fixed
    steps with the remainder banked; paused frames bank nothing; a
    requested step runs once, paused or not, and a running frame's time
    stays banked; a scene with no bodies does no timing work; reset clears
    the clock; garbage dt is no time; a material change shortens only
    future steps and keeps the backlog."""
    import vsim.scenes as sc
    from vsim import Simulator

    def fresh(step=0.002):
        scene = sc.single_box()
        scene.step_duration = None
        sim = Simulator(scene)
        if step:
            sim.set_step_duration(step)
        return sim

    sim = fresh()
    sim.step(0.005)
    st = sim.stats()
    assert st["last_steps"] == 2 and abs(st["backlog_time"] - 0.001) < 1e-12
    sim.step(0.001)
    st = sim.stats()
    assert st["last_steps"] == 1 and st["steps"] == 3

    sim = fresh()
    sim.paused = True
    sim.step(10)
    st = sim.stats()
    assert st["steps"] == 0 and st["backlog_time"] == 0 and st["dropped_time"] == 0
    sim.request_step()
    sim.step(10)
    st = sim.stats()
    assert st["steps"] == 1 and abs(st["simulated_time"] - 0.002) < 1e-12 and st["dropped_time"] == 0
    sim.step(10)
    assert sim.stats()["steps"] == 1  # the request was used up

    empty = Simulator(sc.Scene([], ((-1.0, 0.0, -1.0), (1.0, 1.0, 1.0))))
    empty.request_step()
    empty.step(1)
    assert empty.stats()["steps"] == 0 and empty.stats()["simulated_time"] == 0
    empty.destroy()

    sim = fresh()
    sim.step(0.2)
    sim.request_step()
    sim.reset()
    st = sim.stats()
    assert st["steps"] == 0 and st["simulated_time"] == 0 and st["backlog_time"] == 0 and st["dropped_time"] == 0
    sim.step(0.001)
    assert sim.stats()["steps"] == 0  # no request survived the reset

    sim = fresh()
    sim.request_step()
    sim.step(0.0005)
    st = sim.stats()
    assert st["last_steps"] == 1 and abs(st["backlog_time"] - 0.0005) < 1e-12 and st["dropped_time"] == 0

    sim = fresh()
    sim.request_step()
    sim.step(0.003)
    st = sim.stats()
    assert st["last_steps"] == 1 and abs(st["backlog_time"] - 0.001) < 1e-12

    sim = fresh()
    for dt in (-1.0, float("nan"), float("inf")):
        sim.step(dt)
    st = sim.stats()
    assert st["backlog_time"] == 0 and st["steps"] == 0

    sim = fresh(step=None)  # the CFL rule sets the step
    sim.set_material(0, {"youngs_modulus": 2e3, "density": 700.0})
    before = sim.stats()["step_duration"]
    sim.step(before / 2)
    backlog = sim.stats()["backlog_time"]
    sim.set_material(0, {"youngs_modulus": 1e5})
    st = sim.stats()
    assert st["step_duration"] < before and st["backlog_time"] == backlog


def test_lattice_masses_follow_density(lib):
    """discretize.test.js:59-140 through the library: a sphere (radius
    0.05 m, 0.1/8 m cells) whose lumped node masses sum to density x volume;
    a density change doubles them and leaves material-less nodes inert; a
    chain of density edits comes back to the original masses; every kind of
    rest geometry (shape, mesh, cloud) becomes a body with material."""
    import vsim.scenes as sc
    from vsim import Simulator
    from vsim import voxelize as vz
    from vsim._ffi import fptr

    def inverse_masses(sim):
        out = np.zeros(sim.node_count, np.float32)
        assert lib.lib().vsim_read_inv_mass(sim.handle, fptr(out), sim.node_count) == 0
        return out

    def lumped(inv):
        live = inv[inv > 0].astype(np.float64)
        return float(np.sum(1.0 / live))

    grid = vz.voxelize_sdf(vz.sphere(0.05), 0.1 / 8)
    body = sc.Body(tuple(grid.dims), tuple(grid.origin), grid.h, grid.occupancy,
                   dict(sc.DEFAULT_MATERIAL, density=1000.0))
    tank = ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))
    sim = Simulator(sc.Scene([body], tank, contact=False))
    volume = body.cell_count * grid.h ** 3
    first = inverse_masses(sim)
    assert abs(lumped(first) - 1000.0 * volume) < 1e-5 * 1000.0 * volume
    inert = int(np.count_nonzero(first == 0))
    sim.set_material(0, {"density": 2000.0})
    doubled = inverse_masses(sim)
    assert abs(lumped(doubled) - 2000.0 * volume) < 1e-5 * 2000.0 * volume
    assert int(np.count_nonzero(doubled == 0)) == inert
    for density in (1500.0, 700.0, 2400.0, 1000.0):
        sim.set_material(0, {"density": density})
    assert np.all(np.abs(inverse_masses(sim) - first) < 5e-4)
    sim.destroy()

    cube = vz.box([0.04, 0.04, 0.04])
    corners = [[x, y, z] for x in (-0.04, 0.04) for y in (-0.04, 0.04) for z in (-0.04, 0.04)]
    mesh = vz.Mesh(np.asarray(corners, np.float32), np.asarray(
        [[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
         [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], np.uint32))
    cloud = sc.capture_cloud(3000, 0.04, seed=2)
    for kind, source in (("shape", cube), ("mesh", mesh), ("cloud", cloud)):
        g = vz.voxelize_source(kind, source, 0.01)
        b = sc.Body(tuple(g.dims), tuple(g.origin), g.h, g.occupancy)
        s = Simulator(sc.Scene([b], tank, contact=False))
        assert s.stats()["cells"] > 0 and lumped(inverse_masses(s)) > 0, kind
        s.destroy()


@pytest.mark.parametrize("shape", ["sphere", "box"])
def test_lattice_proxy_contract(lib, shape):
    """proxyGeometry.test.js:150-338 for the lattice the library builds, on
    its shapes (a 0.05 m sphere, a 0.04 x 0.02 x 0.03 m box, 0.015 m cells):
    finite, non-negative inverse masses with material on some nodes; every
    contact node carries material and the surface is listed in ascending
    node order; the material nodes' nearest-neighbour distance is the cell
    edge; a positive stability number; a fourfold density divides every
    inverse mass by four and gives no empty node material."""
    import vsim.scenes as sc
    from vsim import Simulator
    from vsim import voxelize as vz
    from vsim._ffi import fptr

    source = vz.sphere(0.05) if shape == "sphere" else vz.box([0.04, 0.02, 0.03])
    grid = vz.voxelize_sdf(source, 0.015)
    body = sc.Body(tuple(grid.dims), tuple(grid.origin), grid.h, grid.occupancy,
                   dict(sc.DEFAULT_MATERIAL, density=1000.0))
    sim = Simulator(sc.Scene([body], ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)), contact=True))

    def inverse_masses():
        out = np.zeros(sim.node_count, np.float32)
        assert lib.lib().vsim_read_inv_mass(sim.handle, fptr(out), sim.node_count) == 0
        return out

    inv = inverse_masses()
    assert np.all(np.isfinite(inv)) and np.all(inv >= 0) and np.count_nonzero(inv) > 0
    nodes, bodies = sim.contact_surface()
    assert nodes.size > 0 and np.all(bodies == 0) and np.all(nodes < sim.node_count)
    assert np.all(np.diff(nodes.astype(np.int64)) > 0)
    assert np.all(inv[nodes] > 0)
    rest = sc.rest_positions(body).astype(np.float64)[inv > 0]
    d = np.linalg.norm(rest[:, None, :] - rest[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    nearest = d.min(axis=1)
    assert abs(nearest.min() - grid.h) <= 1e-5 * grid.h and abs(nearest.max() - grid.h) <= 1e-5 * grid.h
    assert sim.cfl_number() > 0 and np.isfinite(sim.cfl_number())
    sim.set_material(0, {"density": 4000.0})
    after = inverse_masses()
    assert np.all(after[inv == 0] == 0)
    assert np.all(np.abs(after[inv > 0] - inv[inv > 0] / 4) <= 1e-6 * inv[inv > 0])
    sim.destroy()


@pytest.mark.parametrize("mapping", ["warp", "thread"])
def test_contact_bucket_overflow(lib, mapping):
    """Buckets holding more records than their 32 visible slots
    (contacts.wgsl:75; sort.wgsl:27-40 keeps the 32 lowest record indices):
    a blob squeezed to a fifth of its size about its centre puts up to ~80
    surface records in one bucket and ~65 buckets over capacity. The pair
    set and the frames equal the oracle's under both gather mappings."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.noise_blob(n=20, seed=5, splats=0)
    sim, orc = make(scene)
    sim.set_gather_mapping(mapping)
    pos, prev, vel = orc.state()
    live = orc.inv_mass() > 0
    centre = pos[live, :3].mean(axis=0)
    squeezed = pos.copy()
    squeezed[:, :3] = centre + (squeezed[:, :3] - centre) * 0.2
    sim.write_state(squeezed, squeezed, np.zeros_like(vel))
    orc.set_state(squeezed, squeezed, np.zeros_like(vel))
    assert np.array_equal(sim.contact_pairs(), orc.contact_pairs())
    for frame in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"{mapping} frame {frame}")


def test_splats_on_many_bodies(lib):
    """Splats bound to several bodies of uneven sizes (each body's splats
    embedded in its own lattice, concatenated in body order): after two
    frames their means and covariances equal the oracle's body by body, and
    the depth order over all of them equals a stable sort of the oracle's
    keys."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.box_batch(6, seed=3, splats_per_body=700)
    sim, orc = make(scene)
    for frame in range(2):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
    view = (0.2, -0.5, -0.84)
    sim.deform_splats(view)
    sim.sort_splats()
    means, cov, order = sim.read_splats()
    parts = [orc.splat_deform(b, *scene.splats[b][:3], view) for b in sorted(scene.splats)]
    assert np.array_equal(means, np.concatenate([p[0] for p in parts]))
    assert np.array_equal(cov, np.concatenate([p[1] for p in parts]))
    assert np.array_equal(order, pyoracle.stable_sort(np.concatenate([p[2] for p in parts])))


def test_reset_releases_the_grab(lib):
    """reset() lets the grab go and returns every node to rest
    (simulator.js:495-500 calls releaseGrab): after a dragged frame and a
    reset, frames equal a fresh oracle's, with no node held."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.single_box()
    sim, _ = make(scene)
    rest = sim.read_positions()
    dims = scene.bodies[0].node_dims
    tip = [sc.node_index(dims, 16, j, k) for j in range(5) for k in range(5)]
    offsets = (rest[tip, :3] - rest[tip[0], :3]).astype(np.float32)
    sim.hold(tip, offsets)
    sim.place_grab(rest[tip[0], :3].astype(np.float64))
    sim.move_grab(rest[tip[0], :3].astype(np.float64) + [0.0, 0.05, 0.0])
    sim.dispatch(scene.substeps)
    assert not np.array_equal(sim.read_positions(), rest)
    sim.reset()
    assert np.array_equal(sim.read_positions(), rest)
    assert sim.stats()["driven"] == 0
    orc = pyoracle.Oracle(scene, 32)
    for frame in range(3):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"after reset, frame {frame}")
