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
