"""Pins of the host-side restatements: the reference's own tests of its
voxelisers, OBJ parser, pick and grip, ported (inputs and tolerances kept).
Paths are relative to the reference's packages/visionary-sim/test/unit/."""
import math

import numpy as np
import pytest

from vsim import voxelize as vz
from vsim import simulator as vs


# ---- voxelize.test.js ---------------------------------------------------------------

def _box_mesh(half):
    """voxelize.test.js:14-29."""
    p = np.array([-half, -half, -half, half, -half, -half, half, half, -half, -half, half, -half,
                  -half, -half, half, half, -half, half, half, half, half, -half, half, half], np.float32).reshape(-1, 3)
    i = np.array([0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4, 3, 7, 6, 3, 6, 2, 0, 4, 7, 0, 7, 3,
                  1, 2, 6, 1, 6, 5], np.uint32).reshape(-1, 3)
    return vz.Mesh(p, i)


def test_grid_lays_out_elements():
    # voxelize.test.js:32-37
    g = vz.grid_for_bounds(([0, 0, 0], [0.4, 0.2, 0.1]), 0.02, 2)
    assert g.dims == [24, 14, 9] and g.h == 0.02


def test_grid_rounds_partial_element_up():
    # voxelize.test.js:39-42
    assert vz.grid_for_bounds(([0, 0, 0], [0.41, 0.2, 0.1]), 0.02, 2).dims[0] == 25


def test_grid_ignores_float32_dust():
    # voxelize.test.js:44-52
    extent = float(np.float32(0.15))
    assert extent > 0.15
    assert vz.grid_for_bounds(([0, 0, 0], [extent] * 3), 0.0125, 2).dims == [16, 16, 16]


def test_grid_refuses_to_guess():
    # voxelize.test.js:54-61
    for bad in (0, -1, float("nan"), float("inf")):
        with pytest.raises(ValueError, match="element_size"):
            vz.grid_for_bounds(([0, 0, 0], [0.1] * 3), bad)


def test_grid_padding():
    # voxelize.test.js:63-68
    g = vz.grid_for_bounds(([-1, -1, -1], [1, 1, 1]), 0.25, 2)
    assert abs(g.origin[0] - (-1 - 2 * g.h)) < 1e-12 and vz.count_occupied(g) == 0


def test_sdf_sphere_volume():
    # voxelize.test.js:72-84
    r = 0.1
    g = vz.voxelize_sdf(vz.sphere(r), 2 * r / 32)
    ratio = vz.count_occupied(g) * g.h ** 3 / ((4 / 3) * math.pi * r ** 3)
    assert 1.0 < ratio < 1.16


def test_sdf_torus_hole():
    # voxelize.test.js:86-92
    g = vz.voxelize_sdf(vz.torus(0.08, 0.03), 0.22 / 28)
    c = [math.floor((0 - g.origin[a]) / g.h) for a in range(3)]
    assert g.occupancy[vz.cell_index(g, *c)] == 0 and vz.count_occupied(g) > 0


def test_mesh_box_volume():
    # voxelize.test.js:96-105
    m = _box_mesh(0.5)
    g = vz.voxelize_mesh(m, vz.mesh_bounds(m.positions), 1.0 / 20)
    ratio = vz.count_occupied(g) * g.h ** 3
    assert 0.95 < ratio < 1.35


def test_mesh_survives_a_hole():
    # voxelize.test.js:107-120: the -y face dropped
    m = _box_mesh(0.5)
    holed = vz.Mesh(m.positions, np.vstack([m.indices[:4], m.indices[6:]]))
    g = vz.voxelize_mesh(holed, vz.mesh_bounds(holed.positions), 1 / 16)
    assert vz.count_occupied(g) * g.h ** 3 > 0.7


def test_obj_parses_and_voxelises():
    # voxelize.test.js:122-137
    text = "\n".join(["v -0.5 -0.5 -0.5", "v 0.5 -0.5 -0.5", "v 0.5 0.5 -0.5", "v -0.5 0.5 -0.5",
                      "v -0.5 -0.5 0.5", "v 0.5 -0.5 0.5", "v 0.5 0.5 0.5", "v -0.5 0.5 0.5",
                      "f 1 3 2", "f 1 4 3", "f 5 6 7", "f 5 7 8", "f 1 2 6", "f 1 6 5", "f 4 8 7", "f 4 7 3",
                      "f 1 5 8", "f 1 8 4", "f 2 3 7", "f 2 7 6"])
    m = vz.parse_obj(text)
    assert m.positions.size == 24 and m.indices.size == 36
    g = vz.voxelize_mesh(m, vz.mesh_bounds(m.positions), 1 / 12)
    fill = vz.count_occupied(g) / g.occupancy.size
    assert 0.1 < fill < 0.75


def test_close_seals_a_pit():
    # voxelize.test.js:141-150
    g = vz.voxelize_sdf(vz.box([0.1, 0.1, 0.1]), 0.2 / 12)
    before = vz.count_occupied(g)
    pit = vz.cell_index(g, g.dims[0] // 2, g.dims[1] // 2, g.dims[2] // 2)
    g.occupancy[pit] = 0
    assert vz.count_occupied(g) == before - 1
    vz.morphological_close(g)
    assert g.occupancy[pit] == 1 and vz.count_occupied(g) == before


def test_obj_face_forms():
    # objLoader.js:41-60: "v", "v/vt", "v//vn", "v/vt/vn" and negative indices
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 1/1 2//2 3/3/3\nf -1 -2 -3 -4\n# comment\nvn 0 0 1"
    m = vz.parse_obj(text)
    assert m.indices.tolist() == [[0, 1, 2], [3, 2, 1], [3, 1, 0]]


# ---- pick.test.js -------------------------------------------------------------------

def _nodes(points):
    out = np.zeros((len(points), 4), np.float32)
    out[:, :3] = points
    return out


def _pick(points, masses=None, radius=0.1, static=None):
    masses = np.ones(len(points), np.float32) if masses is None else np.asarray(masses, np.float32)
    static = np.zeros(len(points), bool) if static is None else static
    return vs.nearest_node_to_ray(_nodes(points), masses, [0, 0, 0], [0, 0, 1], radius, static)


def test_pick_closest_to_ray():
    assert _pick([[1, 0, 1], [0.02, 0, 1], [0, 0.5, 1]]) == 1          # pick.test.js:28-30


def test_pick_nearer_of_two():
    assert _pick([[0, 0, 5], [0.05, 0, 1]]) == 1                        # pick.test.js:32-36


def test_pick_no_material():
    assert _pick([[0, 0, 1]], [0]) == -1                                # pick.test.js:38-43
    assert _pick([[0, 0, 1], [0, 0, 2]], [0, 1]) == 1


def test_pick_behind():
    assert _pick([[0, 0, -1]]) == -1                                    # pick.test.js:45-47


def test_pick_past_static():
    # pick.test.js:49-55
    pts, m = [[0, 0, 1], [0.05, 0, 2], [0.2, 0, 1.5]], [2, 3, 4]
    assert _pick(pts, m, static=np.array([True, False, False])) == 1
    assert _pick(pts, m, static=np.array([True, True, False])) == -1


def test_pick_reports_miss():
    assert _pick([[0.4, 0, 1], [0, 0.4, 2]]) == -1                      # pick.test.js:57-59


def test_body_of_node():
    # pick.test.js:62-71
    assert [vs.body_of_node([0, 10, 25], n) for n in (0, 9, 10, 24, 25, 99)] == [0, 0, 1, 1, 2, 2]
    assert vs.body_of_node([0], 7) == 0


# ---- grip.test.js -------------------------------------------------------------------

def _lattice(h, extent=0.12):
    """grip.test.js:30-52: a cube of nodes at spacing h, a node at the centre."""
    n = round(extent / h)
    per = n + 1
    pos = np.zeros((per ** 3, 4), np.float32)
    idx = 0
    for i in range(per):
        for j in range(per):
            for k in range(per):
                pos[idx, :3] = ((i - n / 2) * h, (j - n / 2) * h, (k - n / 2) * h)
                idx += 1
    half = n // 2
    return pos, np.ones(per ** 3, np.float32), [0], (half * per + half) * per + half


def _within(pos, m, anchor, radius, offsets, limit=10 ** 9, static=None):
    static = np.zeros(len(m), bool) if static is None else static
    return vs.within_radius(pos, m, anchor, radius, offsets, static, limit)


def test_grip_material_independent_of_resolution():
    # grip.test.js:64-88
    c_pos, c_m, c_off, c_c = _lattice(0.01)
    f_pos, f_m, f_off, f_c = _lattice(0.005)
    ball_c = len(_within(c_pos, c_m, c_c, 0.04, c_off)[0]) * 0.01 ** 3
    ball_f = len(_within(f_pos, f_m, f_c, 0.04, f_off)[0]) * 0.005 ** 3
    assert 0.9 < ball_f / ball_c < 1.1
    none = np.zeros(len(c_m), bool)
    one_c = len(vs.single_node(c_pos, c_m, c_c, none)[0]) * 0.01 ** 3
    one_f = len(vs.single_node(f_pos, f_m, f_c, np.zeros(len(f_m), bool))[0]) * 0.005 ** 3
    assert abs(one_f / one_c - 1 / 8) < 1e-9


def test_grip_hand_size_in_metres():
    # grip.test.js:90-104
    for h in (0.01, 0.005):
        pos, m, off, c = _lattice(h)
        _, offs, _ = _within(pos, m, c, 0.04, off)
        longest = max(math.hypot(*o) for o in offs.astype(np.float64))
        assert 0.04 - h < longest <= 0.04 + 1e-9


def test_single_node():
    # grip.test.js:107-118
    nodes, offs, found = vs.single_node(np.zeros((1, 4), np.float32), np.ones(1, np.float32), 0, np.zeros(1, bool))
    assert nodes == [0] and offs.tolist() == [[0, 0, 0]] and found == 1


def test_grip_static_filtered_before_counting():
    # grip.test.js:121-132
    pos = np.array([[0, 0, 0, 0], [0.01, 0, 0, 0], [0.02, 0, 0, 0], [-0.02, 0, 0, 0], [0.025, 0, 0, 0],
                    [0.04, 0, 0, 0], [0, 0, 0, 0]], np.float32)
    m = np.ones(7, np.float32)
    static = np.zeros(7, bool)
    static[1] = True
    nodes, _, found = _within(pos, m, 0, 0.03, [0, 6], limit=2, static=static)
    assert nodes == [0, 2] and found == 4
    assert _within(pos, m, 0, 0.03, [0, 6], limit=9, static=static)[0] == [0, 2, 3, 4]


def test_grip_rejects_static_or_empty_anchor():
    # grip.test.js:134-144
    pos = np.zeros((2, 4), np.float32)
    m = np.array([1, 0], np.float32)
    static = np.array([True, False])
    for anchor in (0, 1):
        assert _within(pos, m, anchor, 1, [0], static=static)[2] == 0
        assert vs.single_node(pos, m, anchor, static)[2] == 0


def test_grip_anchor_first_then_nearest_ties_by_index():
    # grip.test.js:146-166
    pos, m, off, c = _lattice(0.01)
    nodes, offs, _ = _within(pos, m, c, 0.03, off)
    assert nodes[0] == c and offs[0].tolist() == [0, 0, 0]
    nodes, offs, _ = _within(pos, m, c, 0.015, off)
    d = [math.hypot(*o) for o in offs.astype(np.float64)]
    assert all(d[i] >= d[i - 1] - 1e-12 for i in range(1, len(d)))
    assert nodes[1:7] == sorted(nodes[1:7])


def test_grip_excludes_no_material_and_other_bodies():
    # grip.test.js:168-190
    pos, m, off, c = _lattice(0.01)
    m[c + 1] = 0
    assert c + 1 not in _within(pos, m, c, 0.03, off)[0]
    pos, m, _, c = _lattice(0.01)
    extra = np.zeros((1, 4), np.float32)
    extra[0, 0] = 0.07
    both = np.vstack([pos, extra])
    assert len(pos) not in _within(both, np.ones(len(both), np.float32), c, 1.0, [0, len(pos)])[0]


def test_grip_truncates_and_counts():
    # grip.test.js:192-201
    pos, m, off, c = _lattice(0.01)
    full = _within(pos, m, c, 0.03, off)
    limited = _within(pos, m, c, 0.03, off, limit=5)
    assert limited[0] == full[0][:5] and limited[2] == len(full[0]) and len(limited[0]) == 5


def test_grip_radius_zero_is_single_node():
    # grip.test.js:203-209
    pos, m, off, c = _lattice(0.01)
    ball = _within(pos, m, c, 0.0, off)
    single = vs.single_node(pos, m, c, np.zeros(len(m), bool))
    assert ball[0] == single[0] and ball[2] == single[2] and ball[1].tolist() == single[1].tolist()


def test_default_grip_radius():
    # grip.test.js:218-226
    assert vs.DEFAULT_GRIPPED_PART_RADIUS > 0.02 and vs.DEFAULT_GRIPPED_PART_RADIUS * 2 < 0.15


# ---- cloudVolume.test.js -----------------------------------------------------------

def _cloud_at(points, radius):
    """cloudVolume.test.js:26-40: identical unrotated Gaussians."""
    pos = np.asarray(points, np.float32).reshape(-1, 3)
    rot = np.zeros((len(pos), 4), np.float32)
    rot[:, 3] = 1
    return pos, rot, np.full((len(pos), 3), radius, np.float32)


def _sphere_shell(radius, count, cover=1.0):
    """cloudVolume.test.js:52-66: a golden-angle spiral over the sphere, only
    the part from the south pole up to `cover`."""
    golden = math.pi * (3 - math.sqrt(5))
    points = []
    for i in range(count):
        y = 1 - (2 * (i + 0.5)) / count
        if y > 2 * cover - 1:
            continue
        ring = math.sqrt(max(0.0, 1 - y * y))
        theta = golden * i
        points += [math.cos(theta) * ring * radius, y * radius, math.sin(theta) * ring * radius]
    return points


def _occupancy_at(grid, point):
    """cloudVolume.test.js:73-76: asked through `locate`, as the render side asks."""
    cell, _ = vz.locate(grid.origin, grid.h, grid.dims, *point)
    return int(grid.occupancy[cell[0] + grid.dims[0] * (cell[1] + grid.dims[1] * cell[2])])


_RADIUS = 0.05
_SPREAD = 0.0008
_SHELL = _sphere_shell(_RADIUS, 6000)
_EXACT = 4 / 3 * math.pi * _RADIUS ** 3


def test_cloud_centres_in_solid_cells():
    # cloudVolume.test.js:84-109
    cloud = _cloud_at(_SHELL, _SPREAD)
    for element in (0.013, 0.0086, 0.0065, 0.0043, 0.0032):
        g = vz.voxelize_cloud(*cloud, element)
        outside = sum(_occupancy_at(g, p) == 0 for p in cloud[0].astype(np.float64).tolist())
        assert outside == 0, element


def test_cloud_shell_becomes_solid():
    # cloudVolume.test.js:111-130
    cloud = _cloud_at(_SHELL, _SPREAD)
    shell = vz.voxelize_cloud(*cloud, 0.005, fill=False)
    solid = vz.voxelize_cloud(*cloud, 0.005)
    assert vz.count_occupied(shell) * shell.h ** 3 / _EXACT < 0.7
    ratio = vz.count_occupied(solid) * solid.h ** 3 / _EXACT
    assert 1.15 < ratio < 1.45


def test_cloud_volume_converges():
    # cloudVolume.test.js:132-144
    cloud = _cloud_at(_SHELL, _SPREAD)

    def error(element):
        g = vz.voxelize_cloud(*cloud, element)
        return abs(vz.count_occupied(g) * g.h ** 3 - _EXACT) / _EXACT

    assert error(0.0037) < error(0.01) * 0.7


def test_cloud_open_capture_stays_hollow():
    # cloudVolume.test.js:146-156
    cloud = _cloud_at(_sphere_shell(_RADIUS, 6000, 0.75), _SPREAD)
    shell = vz.count_occupied(vz.voxelize_cloud(*cloud, 0.005, fill=False))
    filled = vz.count_occupied(vz.voxelize_cloud(*cloud, 0.005))
    assert filled < shell * 1.5


def test_cloud_padding_ring_clear():
    # cloudVolume.test.js:158-176
    g = vz.voxelize_cloud(*_cloud_at(_SHELL, _SPREAD), 0.0065)
    nx, ny, nz = g.dims
    occ = g.occupancy.reshape(nz, ny, nx)
    assert occ[0].sum() + occ[-1].sum() + occ[:, 0].sum() + occ[:, -1].sum() + occ[:, :, 0].sum() \
        + occ[:, :, -1].sum() == 0


def test_cloud_stamps_along_own_axes():
    # cloudVolume.test.js:178-190: a quarter turn about z puts the long axis on y
    pos, rot, scale = _cloud_at([0, 0, 0], 1)
    scale[:] = [0.05, 0.004, 0.004]
    rot[:] = [0, 0, math.sqrt(0.5), math.sqrt(0.5)]
    g = vz.voxelize_cloud(pos, rot, scale, 0.0125, fill=False)
    assert _occupancy_at(g, [0, 0.08, 0]) == 1
    assert _occupancy_at(g, [0.08, 0, 0]) == 0


def test_cloud_refuses_empty_and_flat():
    # cloudVolume.test.js:192-195
    with pytest.raises(ValueError, match="no Gaussians"):
        vz.voxelize_cloud(*_cloud_at([], 0.01), 0.01)
    with pytest.raises(ValueError, match="no extent"):
        vz.voxelize_cloud(*_cloud_at([0, 0, 0], 0), 0.01)


def test_quat_to_columns_quarter_turn():
    # cloudVolume.test.js:199-208: column k is where basis vector k lands
    m = vz.quat_to_columns([0, 0, math.sqrt(0.5), math.sqrt(0.5)])[0]
    assert np.allclose(m, [0, 1, 0, -1, 0, 0, 0, 0, 1], atol=1e-6)


def test_quat_to_columns_orthonormal():
    # cloudVolume.test.js:210-221
    q = np.array([0.3, -0.5, 0.2, 0.7])
    m = vz.quat_to_columns(q / np.linalg.norm(q))[0].astype(np.float64).reshape(3, 3)
    assert np.allclose(m @ m.T, np.eye(3), atol=1e-6)


def test_fill_enclosed_counts_the_cavity():
    # cloudVolume.js:321-375: a closed 5^3 box shell around a 3^3 cavity fills
    # exactly the cavity; a hole in one face lets the outside in.
    g = vz.grid_for_bounds(([0, 0, 0], [1, 1, 1]), 1 / 5)
    nx, ny, nz = g.dims
    occ = g.occupancy.reshape(nz, ny, nx)
    occ[2:7, 2:7, 2:7] = 1
    occ[3:6, 3:6, 3:6] = 0
    holed = vz.OccupancyGrid(g.dims, g.origin, g.h, g.occupancy.copy())
    holed.occupancy.reshape(nz, ny, nx)[4, 4, 2] = 0
    assert vz.fill_enclosed(g) == 27
    assert vz.count_occupied(g) == 125
    assert vz.fill_enclosed(holed) == 0


def test_js_hypot_matches_reference_cases():
    # V8's Math.hypot: zero, infinity before NaN, and the scaled sum
    assert vz.js_hypot(0.0, 0.0, 0.0) == 0.0
    assert vz.js_hypot(np.inf, np.nan, 1.0) == np.inf
    assert np.isnan(vz.js_hypot(np.nan, 1.0, 1.0))
    assert vz.js_hypot(3.0, 4.0, 12.0) == 13.0
    assert vz.js_hypot(1e300, 1e300, 0.0) == pytest.approx(math.sqrt(2) * 1e300)


def test_voxelize_source_dispatch():
    # voxelLattice.js:208-226: one table, three kinds, anything else refused
    cloud = _cloud_at(_SHELL, _SPREAD)
    assert np.array_equal(vz.voxelize_source("cloud", cloud, 0.01).occupancy,
                          vz.voxelize_cloud(*cloud, 0.01).occupancy)
    assert vz.count_occupied(vz.voxelize_source("shape", vz.sphere(0.05), 0.01)) > 0
    assert vz.count_occupied(vz.voxelize_source("mesh", _box_mesh(0.5), 1 / 8)) > 0
    with pytest.raises(ValueError, match='kind "points"'):
        vz.voxelize_source("points", cloud, 0.01)


def test_captured_cloud_scene_centres_in_cells():
    # cloudVolume.js:52-59: the body built from a capture holds every one of
    # its Gaussians' centres in a solid cell, where the splat deformation
    # reads them
    from vsim import scenes as sc

    scene = sc.captured_cloud(count=20_000, radius=0.06, element_size=0.008)
    body = scene.bodies[0]
    means = scene.splats[0][0]
    for p in means.astype(np.float64).tolist():
        cell, _ = vz.locate(body.origin, body.h, body.cell_dims, *p)
        assert body.occupancy[cell[0] + body.cell_dims[0] * (cell[1] + body.cell_dims[1] * cell[2])] == 1
    lowest = min(p[1] for p in means.tolist())
    assert lowest > scene.tank[0][1]
    assert 1.0 < body.cell_count * body.h ** 3 / (4 / 3 * math.pi * 0.06 ** 3) < 1.8


# ---- staticPrescription.test.js ---------------------------------------------------

def test_static_region_classifies_positions():
    # staticPrescription.test.js:11-22
    from vsim import scenes as sc

    positions = np.array([-1, 2, 3, 1, 2, 3, -1, 3, 3, -2, 1, 3], np.float32)
    region = lambda x, y, z: x < 0 and y <= 2 and z == 3  # noqa: E731
    assert sc.static_nodes_in_region(positions, region).tolist() == [0, 3]
    assert sc.static_nodes_in_region(positions).tolist() == []
    assert sc.static_nodes_in_region(positions, lambda x, y, z: True).tolist() == [0, 1, 2, 3]
    assert sc.static_nodes_in_region(np.zeros(0, np.float32), region).tolist() == []


def test_rest_positions_are_the_lattice_nodes():
    # lattice.js:171-179: float32 of origin + index * h, x fastest
    from vsim import scenes as sc

    body = sc.Body((2, 1, 1), (0.1, -0.2, 0.3), 0.016, np.ones(2, np.uint8))
    rest = sc.rest_positions(body)
    assert rest.dtype == np.float32 and rest.shape == (12, 3)
    assert rest[1].tolist() == [np.float32(0.1 + 0.016), np.float32(-0.2), np.float32(0.3)]
    assert rest[11].tolist() == [np.float32(0.1 + 2 * 0.016), np.float32(-0.2 + 0.016), np.float32(0.3 + 0.016)]
