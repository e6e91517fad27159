"""Pins of the CPU oracle: the reference's own known-answer tests, ported.

The reference cannot run here (its step is WGSL on WebGPU and its unit-test
compute backend is a no-op), so these tests are what ties the oracle to it.
Each test names the reference test it ports, by file and line, and keeps that
test's inputs and tolerances. Paths are relative to the reference's
packages/visionary-sim/test/unit/.
"""
import ctypes as C
import math

import numpy as np

H = 0.03125                 # elastic.test.js:190
DT = 1 / (60 * 20)          # elastic.test.js:193
DEFAULT = dict(youngs_modulus=1.2e5, poisson_ratio=0.40, density=1000.0, friction=0.4, damping=0.6,
               relaxation=0.012, max_stretch=0.0)
RATIOS = [0.25, 0.3, 0.35, 0.45, 0.49]   # elastic.test.js:295
CORNERS = np.array([[(c >> a) & 1 for a in range(3)] for c in range(8)], float)


def lame(nu, e=1.2e5):
    nu = min(max(nu, 0.25), 0.49)
    e = max(e, 1.0)
    return e / (2 * (1 + nu)), (e * nu) / ((1 + nu) * (1 - 2 * nu))


def kuhn(oracle):
    tets = np.zeros(24, np.uint32)
    oracle.lib().vo_kuhn_tets(tets.ctypes.data_as(C.POINTER(C.c_uint32)))
    return tets.reshape(6, 4)


def inverses(oracle, h):
    out, p = oracle.f64(np.zeros(54))
    oracle.lib().vo_kuhn_rest_inverses(h, p)
    return out.reshape(6, 9)


def rest_tet(oracle, nu, tet=0):
    """elastic.test.js:202-225."""
    mu, lam = lame(nu)
    volume = H ** 3 / 6
    node_mass = 1000.0 * volume / 4
    tets = kuhn(oracle)
    return dict(p=CORNERS[tets[tet]] * H, B=inverses(oracle, H)[tet], w=np.full(4, 1 / node_mass),
                mu=mu, lam=lam, volume=volume, alpha_dev=1 / (mu * volume) / DT ** 2,
                alpha_hyd=1 / (lam * volume) / DT ** 2, gamma=1 + mu / lam)


def project(oracle, s, p, w=None, prev=None, relax=0.0):
    w = s["w"] if w is None else w
    prev = p if prev is None else prev
    pa, pp = oracle.f64(p)
    va, vp = oracle.f64(prev)
    wa, wp = oracle.f64(w)
    ba, bp = oracle.f64(s["B"])
    out, op = oracle.f64(np.zeros(12))
    oracle.lib().vo_project_tet_f64(pp, vp, wp, bp, s["alpha_dev"], s["alpha_hyd"], s["gamma"], relax, op)
    return out.reshape(4, 3)


def run(oracle, s, p, substeps, relax=0.0):
    pa, pp = oracle.f64(np.array(p, float).ravel())
    wa, wp = oracle.f64(s["w"])
    ba, bp = oracle.f64(s["B"])
    oracle.lib().vo_run_free_tet_f64(pp, wp, bp, s["alpha_dev"], s["alpha_hyd"], s["gamma"], relax, DT, substeps)
    return pa.reshape(4, 3)


def moved(a, b):
    return float(np.max(np.linalg.norm(np.asarray(b) - np.asarray(a), axis=1)))


def volume(p):
    return np.linalg.det(np.stack([p[1] - p[0], p[2] - p[0], p[3] - p[0]], axis=1)) / 6


# ---- elastic.test.js ---------------------------------------------------------

def test_rest_is_fixed_point_every_ratio(oracle):
    # elastic.test.js:298-317
    for nu in RATIOS:
        s = rest_tet(oracle, nu)
        assert moved(s["p"], project(oracle, s, s["p"])) < 1e-9, nu


def test_rest_fixed_point_every_tet(oracle):
    # elastic.test.js:319-326
    for t in range(6):
        s = rest_tet(oracle, 0.25, t)
        assert moved(s["p"], project(oracle, s, s["p"])) < 1e-9, t


def test_free_tet_holds_volume_for_a_second(oracle):
    # elastic.test.js:340-345 (coupled half)
    s = rest_tet(oracle, 0.25)
    assert abs(volume(run(oracle, s, s["p"], 1200)) / volume(s["p"]) - 1) < 5e-7


def test_squashed_tet_recovers(oracle):
    # elastic.test.js:347-356
    s = rest_tet(oracle, 0.25)
    ratio = volume(run(oracle, s, s["p"] * 0.9, 1200)) / volume(s["p"])
    assert 0.6 < ratio < 1.4


def test_momentum_conserved(oracle):
    # elastic.test.js:358-368
    s = rest_tet(oracle, 0.3)
    squashed = s["p"] * np.array([1, 0.7, 1])
    after = project(oracle, s, squashed)
    assert np.all(np.abs((after - squashed).sum(axis=0)) < 1e-12)


def test_collapsed_tet_stays_finite(oracle):
    # elastic.test.js:370-382
    s = rest_tet(oracle, 0.35)
    assert np.all(np.isfinite(project(oracle, s, np.zeros((4, 3)))))


def test_block_never_singular(oracle):
    # elastic.test.js:384-397
    for nu in RATIOS:
        s = rest_tet(oracle, nu)
        cd, ch = C.c_double(), C.c_double()
        gd, gdp = oracle.f64(np.zeros(12))
        gh, ghp = oracle.f64(np.zeros(12))
        pa, pp = oracle.f64(s["p"])
        ba, bp = oracle.f64(s["B"])
        oracle.lib().vo_tet_constraints_f64(pp, bp, s["gamma"], C.byref(cd), C.byref(ch), gdp, ghp)
        gd, gh = gd.reshape(4, 3), gh.reshape(4, 3)
        a00 = sum(s["w"][i] * gd[i] @ gd[i] for i in range(4)) + s["alpha_dev"]
        a01 = sum(s["w"][i] * gd[i] @ gh[i] for i in range(4))
        a11 = sum(s["w"][i] * gh[i] @ gh[i] for i in range(4)) + s["alpha_hyd"]
        assert a00 * a11 - a01 * a01 >= s["alpha_dev"] * s["alpha_hyd"]


def test_inert_corner(oracle):
    # elastic.test.js:400-438
    s = rest_tet(oracle, 0.3)
    squashed = s["p"] * np.array([1, 0.85, 1])
    driven = np.concatenate([[0.0], s["w"][1:]])
    prescribed = project(oracle, s, squashed, w=driven)
    assert moved(squashed[:1], prescribed[:1]) == 0
    discarded = project(oracle, s, squashed)
    for i in range(1, 4):
        assert moved(discarded[i:i + 1], prescribed[i:i + 1]) > 1e-9


RELAX = 0.04 / DT  # elastic.test.js:443


def test_kelvin_voigt_zero_relax_changes_nothing(oracle):
    # elastic.test.js:445-452
    s = rest_tet(oracle, 0.35)
    squashed = s["p"] * np.array([1, 0.8, 1])
    bare = project(oracle, s, squashed)
    damped = project(oracle, s, squashed, prev=s["p"], relax=0.0)
    assert moved(bare, damped) == 0


def test_kelvin_voigt_rest_stays(oracle):
    # elastic.test.js:454-465
    for nu in RATIOS:
        s = rest_tet(oracle, nu)
        assert moved(s["p"], project(oracle, s, s["p"], relax=RELAX)) < 1e-9


def test_kelvin_voigt_ignores_translation(oracle):
    # elastic.test.js:467-476
    s = rest_tet(oracle, 0.35)
    shifted = s["p"] + np.array([0.004, -0.011, 0.002])
    assert moved(shifted, project(oracle, s, shifted, prev=s["p"], relax=RELAX)) < 1e-9


def test_kelvin_voigt_ignores_spin(oracle):
    # elastic.test.js:478-502
    s = rest_tet(oracle, 0.35)
    a = 0.002
    x, y, z = s["p"].T
    spun = np.stack([x * math.cos(a) - y * math.sin(a), x * math.sin(a) + y * math.cos(a), z], axis=1)
    sheared = np.stack([x + y * a, y, z], axis=1)
    shear = moved(sheared, project(oracle, s, sheared, prev=s["p"], relax=RELAX))
    assert moved(spun, project(oracle, s, spun, prev=s["p"], relax=RELAX)) < shear / 100


def test_collapse_barrier_matches_closed_form(oracle, vsimlib):
    # elastic.test.js:539-569 (bisection over survival of a squashed tetrahedron)
    collapse = vsimlib.lib().vsim_collapse_scale
    for nu in [0.25, 0.3, 0.35]:
        s = rest_tet(oracle, nu)
        rest = volume(s["p"])

        def survives(f):
            r = volume(run(oracle, s, s["p"] * f, 3000)) / rest
            return 0.5 < r < 2

        ok, lost = 1.0, 0.05
        for _ in range(18):
            mid = (ok + lost) / 2
            if survives(mid):
                ok = mid
            else:
                lost = mid
        assert abs(ok - collapse(s["gamma"])) < 0.005, nu


def test_collapse_scale_values(vsimlib):
    # elastic.test.js:583-590
    cs = vsimlib.lib().vsim_collapse_scale
    assert abs(cs(4) - 1) < 5e-7
    assert abs(cs(2) - 0.5437) < 5e-4
    assert abs(cs(1)) < 5e-7
    assert cs(5) > 1


def test_compliance_identity(vsimlib):
    # elastic.test.js:593-604
    m = vsimlib.Material(**dict(DEFAULT, poisson_ratio=0.3))
    mu, lam = C.c_double(), C.c_double()
    vsimlib.lib().vsim_lame_parameters(C.byref(m), C.byref(mu), C.byref(lam))
    d, hh, g = C.c_double(), C.c_double(), C.c_double()
    vsimlib.lib().vsim_element_compliance(C.byref(m), H ** 3 / 6, C.byref(d), C.byref(hh), C.byref(g))
    assert abs((d.value * mu.value) / (hh.value * lam.value) - 1) < 5e-13
    assert abs(d.value * mu.value - 1 / (H ** 3 / 6)) < 5e-7 * (1 / (H ** 3 / 6))


# ---- kuhn.test.js ---------------------------------------------------------------

def test_kuhn_positive_and_fills(oracle):
    # kuhn.test.js:15-35
    h = 0.037
    a, p = oracle.f64(np.zeros(54))
    oracle.lib().vo_kuhn_rest_shapes(h, p)
    shapes = a.reshape(6, 3, 3).transpose(0, 2, 1)  # column-major -> rows
    vols = np.linalg.det(shapes) / 6
    assert np.all(vols > 0)
    assert np.all(np.abs(vols / (h ** 3 / 6) - 1) < 1e-6)
    assert abs(vols.sum() / h ** 3 - 1) < 1e-6


def test_kuhn_inverts(oracle):
    # kuhn.test.js:37-49
    h = 0.02
    a, p = oracle.f64(np.zeros(54))
    oracle.lib().vo_kuhn_rest_shapes(h, p)
    shapes = a.reshape(6, 3, 3).transpose(0, 2, 1)
    inv = inverses(oracle, h).reshape(6, 3, 3).transpose(0, 2, 1)
    for t in range(6):
        assert np.allclose(shapes[t] @ inv[t], np.eye(3), atol=5e-7)


def test_kuhn_conforms(oracle):
    # kuhn.test.js:57-90: 3x3x3 cells, boundary faces 6 * 9 * 2
    tets = kuhn(oracle)
    faces = {}
    nd = (4, 4, 4)
    for k in range(3):
        for j in range(3):
            for i in range(3):
                corners = [(i + ((c >> 0) & 1)) + nd[0] * ((j + ((c >> 1) & 1)) + nd[1] * (k + ((c >> 2) & 1)))
                           for c in range(8)]
                for tet in tets:
                    nodes = [corners[c] for c in tet]
                    for skip in range(4):
                        key = tuple(sorted(n for q, n in enumerate(nodes) if q != skip))
                        faces[key] = faces.get(key, 0) + 1
    assert sum(1 for v in faces.values() if v == 1) == 6 * 9 * 2
    assert all(v in (1, 2) for v in faces.values())


def test_library_kuhn_table_matches_oracle(oracle, vsimlib):
    lib_table = np.zeros(54, np.float32)
    vsimlib.lib().vsim_kuhn_rest_inverse(lib_table.ctypes.data_as(C.POINTER(C.c_float)))
    assert np.array_equal(lib_table, inverses(oracle, 1.0).ravel().astype(np.float32))


# ---- contact.test.js --------------------------------------------------------------

def node(**kw):
    d = dict(position=[0, 0, 0], previous=[0, 0, 0], inv_mass=1.0, radius=0.01, friction=0.0)
    d.update(kw)
    return np.array(list(d["position"]) + list(d["previous"]) + [d["inv_mass"], d["radius"], d["friction"]], float)


def pair(oracle, me, mate, mi=0, ji=1):
    a, ap = oracle.f64(me)
    b, bp = oracle.f64(mate)
    out, op = oracle.f64(np.zeros(3))
    hit = oracle.lib().vo_resolve_pair_f64(ap, bp, mi, ji, op)
    return out if hit else None


def test_contact_equal_split(oracle):
    # contact.test.js:257-269
    ov = 0.004
    a, b = node(), node(position=[0.02 - ov, 0, 0])
    fa, fb = pair(oracle, a, b, 0, 1), pair(oracle, b, a, 1, 0)
    assert abs(fa[0] + ov / 2) < 5e-13 and abs(fb[0] - ov / 2) < 5e-13
    assert np.all(fa + fb == 0)


def test_contact_mass_weighted(oracle):
    # contact.test.js:271-282
    ov = 0.004
    light, heavy = node(inv_mass=1), node(position=[0.02 - ov, 0, 0], inv_mass=0.1)
    assert abs(pair(oracle, light, heavy)[0] + ov / 1.1) < 5e-13
    assert abs(pair(oracle, heavy, light, 1, 0)[0] - ov * 0.1 / 1.1) < 5e-13


def test_contact_inert_node(oracle):
    # contact.test.js:284-290
    free, pinned = node(), node(position=[0.016, 0, 0], inv_mass=0)
    assert np.all(pair(oracle, pinned, free, 1, 0) == 0)
    assert abs(pair(oracle, free, pinned)[0] + 0.004) < 5e-13


def test_contact_merely_close(oracle):
    # contact.test.js:292-295
    assert pair(oracle, node(), node(position=[0.02, 0, 0])) is None
    assert pair(oracle, node(), node(position=[0.05, 0, 0])) is None


def test_contact_coincident(oracle):
    # contact.test.js:297-305: index-oriented normal, +y for the lower index
    c = pair(oracle, node(), node(), 0, 1)
    assert np.all(np.isfinite(c)) and abs(c[1] - 0.01) < 5e-13
    assert abs(pair(oracle, node(), node(), 1, 0)[1] + 0.01) < 5e-13


def test_contact_friction_cone(oracle):
    # contact.test.js:307-334
    ov = 0.004

    def contact(slide, friction):
        a = node(previous=[0, -slide, 0], friction=friction)
        b = node(position=[0.02 - ov, 0, 0], friction=friction)
        return pair(oracle, a, b)

    assert abs(contact(0.0002, 0.5)[1] + 0.0002 / 2) < 5e-13
    assert abs(contact(0.01, 0.5)[1] + 0.5 * ov / 2) < 5e-13
    free = contact(0.01, 0)
    assert abs(free[1]) < 5e-13 and abs(free[0] + ov / 2) < 5e-13


def test_contact_min_friction(oracle):
    # contact.test.js:336-345
    ov = 0.004
    a = node(previous=[0, -0.01, 0], friction=0.9)
    b = node(position=[0.02 - ov, 0, 0], friction=0.1)
    assert abs(pair(oracle, a, b)[1] + 0.1 * ov / 2) < 5e-13


def test_broadphase_grid_layout(oracle):
    # contact.test.js:101-147
    mn, mx, size = [-0.30, 0.0, -0.20], [0.30, 0.50, 0.20], 0.0142
    o, op = oracle.f64(np.zeros(3))
    e = C.c_double()
    dims = np.zeros(3, np.uint32)
    mna, mnp = oracle.f64(mn)
    mxa, mxp = oracle.f64(mx)
    oracle.lib().vo_broadphase_grid(mnp, mxp, size, op, C.byref(e), dims.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert np.allclose(o, np.array(mn) - size)
    assert np.all(o + dims * size >= np.array(mx))

    def bucket(point):
        pa, pp = oracle.f64(point)
        return oracle.lib().vo_bucket_of(op, e.value, dims.ctypes.data_as(C.POINTER(C.c_uint32)), pp)

    for i, j, k in [(0, 0, 0), (1, 2, 3), tuple(int(d) - 1 for d in dims)]:
        centre = o + (np.array([i, j, k]) + 0.5) * size
        assert bucket(centre) == i + dims[0] * (j + dims[1] * k)
    assert bucket([-100, -100, -100]) == 0
    assert bucket([100, 100, 100]) == int(np.prod(dims)) - 1
    # contact.test.js:139-147: an empty scene still has a finite grid
    oracle.lib().vo_broadphase_grid(mnp, mxp, 0.0, op, C.byref(e), dims.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert e.value > 0 and 0 < np.prod(dims.astype(float)) < 1e9

    # contact.test.js:149-187: pairs within one bucket never more than one apart
    oracle.lib().vo_broadphase_grid(mnp, mxp, size, op, C.byref(e), dims.ctypes.data_as(C.POINTER(C.c_uint32)))
    state = 12345

    def nxt():
        nonlocal state
        state = (state * 1103515245 + 12345) & 0x7FFFFFFF
        return state / 0x7FFFFFFF

    def coords(index):
        return np.array([index % dims[0], (index // dims[0]) % dims[1], index // (dims[0] * dims[1])])

    for _ in range(2000):
        point = [mn[a] + nxt() * (mx[a] - mn[a]) for a in range(3)]
        d = np.array([nxt() * 2 - 1, nxt() * 2 - 1, nxt() * 2 - 1])
        near = np.array(point) + d / max(np.linalg.norm(d), 1e-9) * size * 0.999 * nxt()
        assert np.all(np.abs(coords(bucket(point)).astype(int) - coords(bucket(near)).astype(int)) <= 1)


# ---- kinematicDrive.test.js ---------------------------------------------------------

def drive_hard(oracle, here, goal, velocity, dt):
    pos, pp = oracle.f64(np.zeros(3))
    vel, vp = oracle.f64(np.zeros(3))
    a, ap = oracle.f64(here)
    b, bp = oracle.f64(goal)
    c, cp = oracle.f64(velocity)
    oracle.lib().vo_drive_hard_f64(ap, bp, cp, dt, pp, vp)
    return pos, vel


def test_drive_hard(oracle):
    # kinematicDrive.test.js:69-118
    dt = 1 / 1200
    pos, _ = drive_hard(oracle, [0, 0, 0], [10, 0, 0], [1, 0, 0], dt)
    assert list(pos) == [1 * dt, 0, 0]
    goal = [0.001, -0.0002, 0]
    pos, _ = drive_hard(oracle, [0, 0, 0], goal, np.array(goal) * 1e6, dt)
    assert list(pos) == goal
    goal = np.array([0.012, -0.02, 0.005])
    here = np.zeros(3)
    for _ in range(20):
        here, _ = drive_hard(oracle, here, goal, goal / (20 * dt), dt)
    assert np.all(np.abs(here - goal) < 5e-13)
    _, vel = drive_hard(oracle, [0, 0, 0], [10, 10, 10], [0.3, -0.1, 0.2], dt)
    assert np.all(np.abs(vel - [0.3, -0.1, 0.2]) < 5e-10)
    pos, vel = drive_hard(oracle, [1, 2, 3], [1, 2, 3], [0, 0, 0], dt)
    assert list(pos) == [1, 2, 3] and list(vel) == [0, 0, 0]


def test_drive_compliant(oracle):
    # kinematicDrive.test.js:120-160: frac = dt^2 / (dt^2 + tau^2), mass-free
    dt, tau = 1 / 1200, 0.05
    out, op = oracle.f64(np.zeros(3))
    a, ap = oracle.f64([0, 0, 0])
    b, bp = oracle.f64([1, 0, 0])
    oracle.lib().vo_drive_compliant_f64(ap, bp, dt, tau, op)
    assert abs(out[0] - dt * dt / (dt * dt + tau * tau)) < 1e-15
    oracle.lib().vo_drive_compliant_f64(ap, bp, dt, 1e-12, op)
    assert abs(out[0] - 1) < 1e-9


# ---- stretch.test.js ------------------------------------------------------------------

def stretch(oracle, a, b, wa, wb, maximum):
    aa, ap = oracle.f64(a)
    bb, bp = oracle.f64(b)
    oracle.lib().vo_stretch_pair_f64(ap, bp, wa, wb, maximum)
    return aa, bb


def test_stretch_limit(oracle):
    # stretch.test.js:5-31
    a, b = stretch(oracle, [2, 3, 4], [2, 4, 4], 1, 1, 1.05)
    assert list(a) == [2, 3, 4] and list(b) == [2, 4, 4]
    a, b = stretch(oracle, [2, 3, 4], [2, 5, 4], 1, 1, 1.05)
    assert abs(a[1] - (3 + 0.475)) < 1e-12 and abs(b[1] - (5 - 0.475)) < 1e-12
    a, b = stretch(oracle, [0, 0, 0], [2, 0, 0], 0, 4, 1.05)
    assert a[0] == 0 and abs(b[0] - 1.05) < 1e-12
    a, b = stretch(oracle, [0, 0, 0], [2, 0, 0], 0, 0, 1.05)
    assert b[0] == 2
    a, b = stretch(oracle, [0, 0, 0], [2, 0, 0], 2, 1, 1.05)
    assert abs(b[0] - a[0] - 1.05) < 1e-12 and abs((a[0] / 2 + b[0]) / 1.5 - 2 / 1.5) < 1e-12
    edges, ep = oracle.f64(np.zeros(84))
    oracle.lib().vo_stretch_edges(ep)
    edges = edges.reshape(28, 3)
    assert len({(int(a), int(b)) for a, b, _ in edges}) == 28
    for a, b, length in edges:
        assert abs(length - np.linalg.norm(CORNERS[int(a)] - CORNERS[int(b)])) < 1e-12


# ---- sample.test.js / covariance.test.js ------------------------------------------------

def test_affine_field_reproduced(oracle):
    # sample.test.js:64-115: a 10 x 8 x 6 grid (the box voxelisation's bounds)
    # deformed by an affine map; the sampler reproduces it.
    A = np.array([1.13, 0.21, -0.07, -0.05, 0.94, 0.16, 0.09, -0.11, 1.27]).reshape(3, 3).T
    b = np.array([0.031, -0.017, 0.048])
    h = 0.012
    cd = np.array([10, 8, 6], np.uint32)
    nd = cd + 1
    origin = np.array([-0.06, -0.048, -0.036])
    k, j, i = np.meshgrid(np.arange(nd[2]), np.arange(nd[1]), np.arange(nd[0]), indexing="ij")
    rest = (origin + np.stack([i, j, k], -1).reshape(-1, 3) * h).astype(np.float32).astype(float)
    deformed = (rest @ A.T + b).astype(np.float32).astype(float)
    da, dp = oracle.f64(deformed)
    oa, op = oracle.f64(origin)
    for t in ([3.3, 2.7, 1.1], [5.9, 4.2, 3.8], [0.5, 0.5, 0.5]):
        point = origin + np.array(t) * h
        pa, pp = oracle.f64(point)
        pos, posp = oracle.f64(np.zeros(3))
        F, Fp = oracle.f64(np.zeros(9))
        oracle.lib().vo_deformation_at_f64(dp, nd.ctypes.data_as(C.POINTER(C.c_uint32)),
                                          cd.ctypes.data_as(C.POINTER(C.c_uint32)), op, h, pp, posp, Fp)
        assert np.all(np.abs(pos - (A @ point + b)) < 5e-6)
        assert np.all(np.abs(F.reshape(3, 3).T - A) < 5e-5)


def _cov_ref(q, s):
    x, y, z, w = q
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                  [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                  [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]]).T
    return r @ np.diag(np.asarray(s) ** 2) @ r.T


def cov(oracle, F, q, s):
    fa, fp = oracle.f64(np.asarray(F).T.ravel())
    qa, qp = oracle.f64(q)
    sa, sp = oracle.f64(s)
    out, op = oracle.f64(np.zeros(9))
    oracle.lib().vo_deformed_covariance_f64(fp, qp, sp, op)
    return out.reshape(3, 3).T


def test_covariance(oracle):
    # covariance.test.js:101-171
    q = np.array([0.3, -0.5, 0.2, 0.7])
    q /= np.linalg.norm(q)
    s = [0.02, 0.006, 0.0004]
    got = cov(oracle, np.eye(3), q, s)
    ref = _cov_ref(q, s)
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-9
    got = cov(oracle, np.diag([2, 3, 0.5]), [0, 0, 0, 1], [0.01, 0.02, 0.04])
    assert np.max(np.abs(got - np.diag([0.02 ** 2, 0.06 ** 2, 0.02 ** 2]))) / 0.06 ** 2 < 1e-9
    state = 20260810

    def nxt():
        nonlocal state
        state = (state * 1103515245 + 12345) % 2147483648
        return state / 2147483648

    for trial in range(2000):
        amp = [0.05, 0.4, 1.5][trial % 3]
        F = np.eye(3).T.ravel() + np.array([(nxt() * 2 - 1) * amp for _ in range(9)])
        F = F.reshape(3, 3).T
        q = np.array([nxt() * 2 - 1 for _ in range(4)])
        q /= np.linalg.norm(q)
        flat = trial % 4 == 0
        s = np.array([1, 0.3, 0.003 if flat else 0.1]) * np.array([(0.5 + nxt()) * 0.02 for _ in range(3)])
        got = cov(oracle, F, q, s)
        ref = F @ _cov_ref(q, s) @ F.T
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-9
        assert np.max(np.abs(got - got.T)) / np.max(np.abs(got)) < 1e-12


# ---- lattice.test.js --------------------------------------------------------------

def test_lone_cell_surface(oracle):
    # lattice.test.js:133-145
    cd = np.array([3, 3, 3], np.uint32)
    occ = np.zeros(27, np.uint8)
    occ[1 + 3 * (1 + 3 * 1)] = 1
    out = np.zeros(64, np.uint32)
    n = oracle.lib().vo_surface_nodes(cd.ctypes.data_as(C.POINTER(C.c_uint32)),
                                      occ.ctypes.data_as(C.POINTER(C.c_uint8)),
                                      out.ctypes.data_as(C.POINTER(C.c_uint32)))
    expect = sorted((1 + (c & 1)) + 4 * ((1 + ((c >> 1) & 1)) + 4 * (1 + ((c >> 2) & 1))) for c in range(8))
    assert n == 8 and list(out[:8]) == expect


def test_lattice_colours_mass_surface(oracle):
    # lattice.test.js:17-130 on a voxelised sphere (12 cells across)
    import vsim.scenes as sc

    n = 12
    c = (np.arange(n) + 0.5) - n / 2
    k, j, i = np.meshgrid(c, c, c, indexing="ij")
    occ = ((i * i + j * j + k * k) <= (n / 2) ** 2).astype(np.uint8).ravel()
    h = 0.2 / 12
    body = sc.Body((n, n, n), (-0.1, -0.1, -0.1), h, occ, dict(DEFAULT))
    o = oracle.Oracle(sc.Scene([body], ((-1, -1, -1), (1, 1, 1))))
    cells, counts = o.cells(0)
    nd = (n + 1, n + 1, n + 1)
    at = 0
    for colour in range(8):
        claimed = set()
        for cell in cells[at:at + counts[colour]]:
            ci, cj, ck = cell % n, (cell // n) % n, cell // (n * n)
            assert ((ci & 1) | ((cj & 1) << 1) | ((ck & 1) << 2)) == colour
            for corner in range(8):
                node = (ci + (corner & 1)) + nd[0] * ((cj + ((corner >> 1) & 1)) + nd[1] * (ck + ((corner >> 2) & 1)))
                assert node not in claimed
                claimed.add(node)
        at += counts[colour]
    assert len(set(cells.tolist())) == len(cells) == int(occ.sum())
    inv = o.inv_mass()
    lumped = float(np.sum(1.0 / inv[inv > 0].astype(np.float64)))
    mass = 1000 * h ** 3 * occ.sum()
    assert abs(lumped - mass) < 5e-7 * mass
    surface, _ = o.surface()
    assert 0 < surface.size < np.count_nonzero(inv)
    assert np.all(inv[surface] > 0) and np.all(np.diff(surface.astype(np.int64)) > 0)
    mid = (n // 2) + nd[0] * ((n // 2) + nd[1] * (n // 2))
    assert mid not in set(surface.tolist()) and 0 not in set(surface.tolist())


# ---- ellipsoid.test.js (apps/simulator/test/unit/ellipsoid.test.js) ---------------

def _stream(seed):
    """ellipsoid.test.js:95-98, in JavaScript's double arithmetic."""
    state = float(seed)

    def nxt():
        nonlocal state
        state = math.fmod(state * 1103515245.0 + 12345.0, 2147483648.0)
        return state / 2147483648.0

    return nxt


def _rotation(nxt):
    q = np.array([nxt() * 2 - 1 for _ in range(4)])
    return q / np.linalg.norm(q)


def _ellipsoid_cov(rot, scale):
    """R diag(s)^2 R^T (ellipsoid.test.js:55-64)."""
    x, y, z, w = rot
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    return r @ np.diag(np.asarray(scale) ** 2) @ r.T


def _six(m):
    return np.array([m[0, 0], m[1, 0], m[2, 0], m[1, 1], m[2, 1], m[2, 2]])


def _axes(m):
    import pyoracle

    return pyoracle.ellipsoid_axes_f64(_six(m))


def _close(actual, expected, tol):
    return np.max(np.abs(actual - expected)) / np.max(np.abs(expected)) < tol


def test_ellipsoid_identity(oracle):
    # ellipsoid.test.js:126-135: an undeformed ellipsoid comes back unchanged
    rest = _rotation(_stream(11))
    scale = [0.02, 0.006, 0.0004]
    rot, sc = _axes(_ellipsoid_cov(rest, scale))
    assert _close(_ellipsoid_cov(rot, sc), _ellipsoid_cov(rest, scale), 1e-9)


def test_ellipsoid_diagonal(oracle):
    # ellipsoid.test.js:137-146
    rot, sc = _axes(np.diag([0.0004, 0.0036, 0.0004]))
    assert np.allclose(np.sort(sc), [0.02, 0.02, 0.06], atol=5e-10, rtol=0)


def test_ellipsoid_reconstructs(oracle):
    # ellipsoid.test.js:148-166: 2000 carried covariances, flat splats included
    nxt = _stream(20260810)
    for trial in range(2000):
        amp = [0.05, 0.4, 1.5][trial % 3]
        g = np.eye(3).T.ravel() + np.array([(nxt() * 2 - 1) * amp for _ in range(9)])
        g = g.reshape(3, 3).T
        rot = _rotation(nxt)
        flat = trial % 4 == 0
        scale = [v * (0.5 + nxt()) * 0.02 for v in (1, 0.3, 0.003 if flat else 0.1)]
        expected = g @ _ellipsoid_cov(rot, scale) @ g.T
        r, s = _axes(expected)
        assert _close(_ellipsoid_cov(r, s), expected, 1e-9), f"trial {trial}"


def test_ellipsoid_unit_quaternion(oracle):
    # ellipsoid.test.js:168-181
    nxt = _stream(7)
    for trial in range(500):
        g = (np.eye(3).T.ravel() + np.array([(nxt() * 2 - 1) * 0.8 for _ in range(9)])).reshape(3, 3).T
        r, _ = _axes(g @ _ellipsoid_cov(_rotation(nxt), [0.02, 0.01, 0.0002]) @ g.T)
        assert abs(math.hypot(*r) - 1) < 5e-10, f"trial {trial}"


def test_ellipsoid_degenerate(oracle):
    # ellipsoid.test.js:183-196: a flattened ellipsoid loses an axis, not the splat
    flattening = np.array([[1, 0, 0], [0, 0, 0], [0, 0, 1]], float)
    m = flattening @ _ellipsoid_cov(_rotation(_stream(3)), [0.02, 0.01, 0.005]) @ flattening.T
    r, s = _axes(m)
    assert np.all(np.isfinite(s)) and np.all(np.isfinite(r))
    assert np.sort(s)[0] < 1e-9 and np.sort(s)[2] > 1e-3


def test_ellipsoid_float_evaluation_reconstructs(oracle):
    """The float evaluation (what the GPU computes) keeps f32-level accuracy
    on the same carried covariances."""
    import pyoracle

    nxt = _stream(20260810)
    covs, expected = [], []
    for trial in range(500):
        amp = [0.05, 0.4, 1.5][trial % 3]
        g = (np.eye(3).T.ravel() + np.array([(nxt() * 2 - 1) * amp for _ in range(9)])).reshape(3, 3).T
        rot = _rotation(nxt)
        scale = [v * (0.5 + nxt()) * 0.02 for v in (1, 0.3, 0.1)]
        e = g @ _ellipsoid_cov(rot, scale) @ g.T
        covs.append(_six(e))
        expected.append(e)
    rots, scales = pyoracle.ellipsoid_axes_f32(np.array(covs))
    for r, s, e in zip(rots.astype(np.float64), scales.astype(np.float64), expected):
        assert _close(_ellipsoid_cov(r, s), e, 1e-4)
