"""The Gaussian-cloud voxeliser on the GPU (`vsim_voxelize_cloud`,
csrc/cloud_volume.cu) against the host restatement of cloudVolume.js
(vsim.voxelize.voxelize_cloud), which the reference's own cloud tests pin
(tests/test_host_pins.py): the same grid (dims, origin, h) and the same
occupancy byte for byte, and the same occupied and filled counts.

The fill's flood runs by rounds of sweeps and, past a cap of rounds, by a
union-find; the fill cases run both ways (`flood`), and nested shells whose
inner cavity is reached only by a winding path take several rounds, or the
union-find when the cap is lower. The seal and flood pack 32 cells to a word
along x; box shells with rows of 8, 31, 32, 33, 64 and 65 cells take the
word edges.

Cases: the reference tests' sphere shell at its element sizes, with and
without the fill; an open capture; anisotropic randomly rotated Gaussians;
boxes large enough to go to the block-per-Gaussian stamp; degenerate
Gaussians; padding under two cells (boxes that leave the grid); seal 0 and
3, sigma 1; samples exactly on an ellipsoid's surface and one float ulp
off it (which the stamp's float test must hand to its double evaluation);
inputs already on the device; the errors.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vz(vsimlib, gpu):
    from vsim import voxelize

    return voxelize


@pytest.fixture(params=["sweeps", "union-find"])
def flood(request, vz):
    before = vz.set_flood_rounds(24 if request.param == "sweeps" else 0)
    yield request.param
    vz.set_flood_rounds(before)


def _cloud_at(points, radius):
    pos = np.asarray(points, np.float32).reshape(-1, 3)
    rot = np.zeros((len(pos), 4), np.float32)
    rot[:, 3] = 1
    return pos, rot, np.full((len(pos), 3), radius, np.float32)


def _shell(radius, count, cover=1.0):
    golden = math.pi * (3 - math.sqrt(5))
    i = np.arange(count, dtype=np.float64)
    y = 1 - 2 * (i + 0.5) / count
    keep = y <= 2 * cover - 1
    ring = np.sqrt(np.maximum(0.0, 1 - y * y))
    pts = np.stack([np.cos(golden * i) * ring * radius, y * radius, np.sin(golden * i) * ring * radius], axis=1)
    return pts[keep]


def _same(vz, cloud, element, **kw):
    host_stats, dev_stats = {}, {}
    host = vz.voxelize_cloud(*cloud, element, stats=host_stats, **kw)
    dev = vz.voxelize_cloud_on_device(*cloud, element, stats=dev_stats, **kw)
    assert dev.dims == host.dims, (dev.dims, host.dims)
    assert dev.origin == host.origin and dev.h == host.h
    diff = np.flatnonzero(dev.occupancy != host.occupancy)
    assert diff.size == 0, f"{diff.size} cells differ, first {diff[:8]}"
    assert dev_stats == host_stats, (dev_stats, host_stats)
    return dev


@pytest.mark.parametrize("element", [0.013, 0.0086, 0.0065, 0.0043, 0.0032])
def test_sphere_shell_filled(vz, flood, element):
    _same(vz, _cloud_at(_shell(0.05, 6000), 0.0008), element)


def test_sphere_shell_unfilled_and_open(vz, flood):
    _same(vz, _cloud_at(_shell(0.05, 6000), 0.0008), 0.005, fill=False)
    g = _same(vz, _cloud_at(_shell(0.05, 6000, 0.75), 0.0008), 0.005)
    assert vz.count_occupied(g) > 0


def test_rotated_anisotropic_capture(vz, flood):
    import vsim.scenes as sc

    cloud = sc.capture_cloud(60_000, 0.08, seed=11)
    _same(vz, cloud, 0.004)
    _same(vz, cloud, 0.0025, seal=3, sigma=1.0)
    _same(vz, cloud, 0.006, seal=0)


@pytest.mark.parametrize("large", [0.006, 0.0025])
def test_box_sizes_and_stamp_paths(vz, large):
    # Gaussians reaching ~6 cells each way (boxes of ~13^3 cells, over the
    # 64 a thread stamps inline, so a block each) or ~2.5 (boxes of 125-343
    # cells, also a block each, a few rounds of its threads), mixed with
    # small ones
    rng = np.random.default_rng(3)
    n = 400
    pos = rng.uniform(-0.1, 0.1, (n, 3)).astype(np.float32)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    scale = np.where(rng.random((n, 1)) < 0.5, large, 0.0004) * rng.uniform(0.5, 1.5, (n, 3))
    _same(vz, (pos, q.astype(np.float32), scale.astype(np.float32)), 0.002)
    long = _cloud_at([0, 0, 0], 1)
    long[2][:] = [0.05, 0.004, 0.004]
    long[1][:] = [0, 0, math.sqrt(0.5), math.sqrt(0.5)]
    g = _same(vz, long, 0.0125, fill=False)
    cell, _ = vz.locate(g.origin, g.h, g.dims, 0, 0.08, 0)
    assert g.occupancy[cell[0] + g.dims[0] * (cell[1] + g.dims[1] * cell[2])] == 1


def test_degenerate_gaussians(vz):
    # zero and denormal scales mixed in: their axes divide to inf or NaN and
    # test nothing, their centre cells are still marked
    rng = np.random.default_rng(5)
    pos, rot, scale = _cloud_at(_shell(0.04, 3000), 0.0008)
    scale[::7] = 0
    scale[3::11, 1] = 1e-40
    rot[5::13] = [0.5, -0.5, 0.5, 0.5]
    _same(vz, (pos, rot, scale), 0.004)
    flat = pos.copy()
    flat[:, 1] = 0.01  # a flat cloud: extent only from the ellipsoids on y
    _same(vz, (flat, rot, scale), 0.004)


@pytest.mark.parametrize("padding", [0, 1, 3])
def test_padding_edges(vz, flood, padding):
    # under two cells of padding the stamp's box can leave the grid, and the
    # reference's typed array ignores those indices
    rng = np.random.default_rng(9)
    pos = rng.uniform(-0.02, 0.02, (500, 3)).astype(np.float32)
    cloud = _cloud_at(pos, 0.002)
    _same(vz, cloud, 0.003, padding=padding)
    flat = pos.copy()
    flat[:, 2] = 0.0
    _same(vz, _cloud_at(flat, 0.0), 0.003, padding=padding)


def test_device_inputs(vz):
    import torch
    import vsim.scenes as sc

    cloud = sc.capture_cloud(20_000, 0.05, seed=2)
    host = vz.voxelize_cloud(*cloud, 0.003)
    dev = vz.voxelize_cloud_on_device(*[torch.from_numpy(a).cuda() for a in cloud], 0.003)
    assert dev.dims == host.dims and dev.origin == host.origin
    assert np.array_equal(dev.occupancy, host.occupancy)


def test_errors(vz):
    from vsim import _ffi

    with pytest.raises(_ffi.VsimError, match="no Gaussians"):
        vz.voxelize_cloud_on_device(*_cloud_at([], 0.01), 0.01)
    with pytest.raises(_ffi.VsimError, match="no extent"):
        vz.voxelize_cloud_on_device(*_cloud_at([0, 0, 0], 0), 0.01)
    nan = _cloud_at([[0, 0, 0], [np.nan, 0, 0]], 0.01)
    with pytest.raises(_ffi.VsimError, match="no extent"):
        vz.voxelize_cloud_on_device(*nan, 0.01)
    with pytest.raises(_ffi.VsimRangeError):
        vz.voxelize_cloud_on_device(*_cloud_at([0, 0, 0], 0.01), 0.0)
    with pytest.raises(_ffi.VsimRangeError):
        vz.voxelize_cloud_on_device(*_cloud_at([0, 0, 0], 0.01), float("inf"))


def test_samples_on_the_surface(vz):
    # Binary-exact layout: h = 1/4, centres on cell corners, radius one cell
    # (sigma 2 x scale 1/8), so samples one cell away along an axis give a
    # sum of exactly 1 (inside); scales one float ulp smaller put the same
    # samples just outside. The float test cannot call either; both go to
    # the double evaluation.
    rng = np.random.default_rng(12)
    pos = (rng.integers(-20, 20, (300, 3)) * 0.25).astype(np.float32)
    exact = _cloud_at(pos, 0.125)
    _same(vz, exact, 0.25, fill=False)
    below = _cloud_at(pos, float(np.nextafter(np.float32(0.125), np.float32(0))))
    _same(vz, below, 0.25, fill=False)
    mixed = (pos, exact[1], np.where(rng.random((300, 1)) < 0.5, exact[2], below[2]).astype(np.float32))
    _same(vz, mixed, 0.25)


def _cube_shell(half, spacing, hole_axis_sign, hole_half):
    """Points on the faces of a cube of half-size `half`, `spacing` apart,
    leaving a square hole of half-width `hole_half` in the middle of the
    face on x = hole_axis_sign * half."""
    t = np.arange(-half, half + spacing / 2, spacing)
    u, v = np.meshgrid(t, t, indexing="ij")
    u, v = u.ravel(), v.ravel()
    faces = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            p = np.zeros((u.size, 3))
            p[:, axis] = sign * half
            p[:, (axis + 1) % 3] = u
            p[:, (axis + 2) % 3] = v
            if axis == 0 and sign == hole_axis_sign:
                keep = ~((np.abs(u) < hole_half) & (np.abs(v) < hole_half))
                p = p[keep]
            faces.append(p)
    return np.unique(np.round(np.concatenate(faces), 9), axis=0)


@pytest.mark.parametrize("rounds", [24, 2, 1, 0])
def test_nested_shells_winding_path(vz, rounds):
    # An outer cube open on +x around an inner cube open on -x: the inner
    # cavity is outside only by a path that enters the gap, turns round the
    # inner cube and enters it from the far side, which the sweeps follow
    # over several rounds; with fewer rounds the union-find decides. A
    # closed third cube inside stays enclosed and is filled.
    pts = np.concatenate([_cube_shell(0.12, 0.003, 1.0, 0.02), _cube_shell(0.07, 0.003, -1.0, 0.02),
                          _cube_shell(0.025, 0.003, 1.0, 0.0)])
    cloud = _cloud_at(pts, 0.0016)
    before = vz.set_flood_rounds(rounds)
    try:
        g = _same(vz, cloud, 0.004)
    finally:
        vz.set_flood_rounds(before)
    # the innermost cube is filled; the cavity between it and the middle one is not
    cell, _ = vz.locate(g.origin, g.h, g.dims, 0.0, 0.0, 0.0)
    assert g.occupancy[cell[0] + g.dims[0] * (cell[1] + g.dims[1] * cell[2])] == 1
    for probe in ((0.0, 0.05, 0.0), (0.095, 0.0, 0.0), (-0.095, 0.0, 0.0)):
        cell, _ = vz.locate(g.origin, g.h, g.dims, *probe)
        assert g.occupancy[cell[0] + g.dims[0] * (cell[1] + g.dims[1] * cell[2])] == 0, probe


def _box_shell(half, spacing):
    """Points on the faces of an axis-aligned box of half-extents `half`."""
    axes = [np.arange(-h, h + spacing / 2, spacing) for h in half]
    pts = []
    for axis in range(3):
        u, v = np.meshgrid(axes[(axis + 1) % 3], axes[(axis + 2) % 3], indexing="ij")
        for sign in (-1.0, 1.0):
            p = np.zeros((u.size, 3))
            p[:, axis] = sign * half[axis]
            p[:, (axis + 1) % 3] = u.ravel()
            p[:, (axis + 2) % 3] = v.ravel()
            pts.append(p)
    return np.unique(np.round(np.concatenate(pts), 9), axis=0)


@pytest.mark.parametrize("nx", [8, 31, 32, 33, 64, 65])
def test_word_edges(vz, flood, nx):
    # The seal and the flood pack 32 cells to a word along x: rows one cell
    # short of, on and past a word's end, and shorter than a word.
    h, reach = 0.004, 0.0016
    extent = (nx - 4 - 0.5) * h  # padding 2 on both sides
    cloud = _cloud_at(_box_shell((extent / 2 - reach, 0.03, 0.02), 0.002), reach / 2)
    g = _same(vz, cloud, h)
    assert g.dims[0] == nx
    assert vz.count_occupied(g) > 0
