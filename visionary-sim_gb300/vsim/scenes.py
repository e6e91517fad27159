"""Seeded synthetic scenes of the solver's workloads.

The reference voxelises meshes, SDFs and Gaussian clouds into occupancy
grids (voxelize.js, cloudVolume.js); the workloads here are defined directly
as occupancy grids instead:

- ``single_box``: a 16 x 4 x 4-cell bar pinned at one end, no contact.
- ``noise_blob``: seeded 3-octave value noise on an n^3 grid, thresholded at
  0.5 and kept to its largest 6-connected component, resting above a ground
  plane, with self contact, plus Gaussian splats inside its occupied cells.
- ``box_batch``: many independent boxes with log-uniform sides, random
  materials and one random face pinned, on a ground plane.
- ``blob_and_sheet``: a large noise blob with a thin sheet above it.

Splat distributions: means uniform inside occupied cells, log-scales uniform
in [ln 1e-3, ln 1e-2] per axis, uniformly random unit quaternions, opacity
U(0.1, 1), RGB U(0, 1).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _ffi

DEFAULT_MATERIAL = dict(youngs_modulus=1.2e5, poisson_ratio=0.40, density=1000.0, friction=0.4,
                        damping=0.6, relaxation=0.012, max_stretch=0.0)
H = 0.016  # cell edge of every workload, metres


@dataclass
class Body:
    """One body as the C ABI takes it: an occupancy grid and a material."""
    cell_dims: tuple
    origin: tuple
    h: float
    occupancy: np.ndarray  # uint8, flattened with x fastest
    material: dict = field(default_factory=lambda: dict(DEFAULT_MATERIAL))
    static_nodes: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))

    @property
    def node_dims(self):
        return tuple(d + 1 for d in self.cell_dims)

    @property
    def node_count(self):
        nx, ny, nz = self.node_dims
        return nx * ny * nz

    @property
    def cell_count(self):
        return int(np.count_nonzero(self.occupancy))


@dataclass
class Scene:
    bodies: list
    tank: tuple  # ((min xyz), (max xyz))
    step_duration: float | None = None  # None: the CFL rule picks it
    substeps: int = 10
    iterations: int = 1
    contact: bool = True
    self_contact: bool = False
    isolated: bool = False  # bodies never touch each other (own contact grids)
    splats: dict = field(default_factory=dict)  # body -> (means, quats, scales, opacity, rgb)

    @property
    def cells(self):
        return sum(b.cell_count for b in self.bodies)


class Descs:
    """ctypes arrays for vsim_create (and the oracle) that keep the numpy
    buffers they point into alive."""

    def __init__(self, scene: Scene):
        self.keep = []
        n = len(scene.bodies)
        self.bodies = (_ffi.BodyDesc * max(n, 1))()
        for i, b in enumerate(scene.bodies):
            d = self.bodies[i]
            occ = np.ascontiguousarray(b.occupancy, dtype=np.uint8)
            st = np.ascontiguousarray(b.static_nodes, dtype=np.uint32)
            self.keep += [occ, st]
            d.cell_dims[:] = [int(v) for v in b.cell_dims]
            d.origin[:] = [float(v) for v in b.origin]
            d.h = float(b.h)
            d.occupancy = occ.ctypes.data_as(C.POINTER(C.c_uint8))
            for k, v in b.material.items():
                setattr(d.material, k, float(v))
            d.static_nodes = st.ctypes.data_as(C.POINTER(C.c_uint32)) if st.size else None
            d.static_count = int(st.size)
        self.count = n
        self.tank = _ffi.Tank()
        self.tank.min[:] = [float(v) for v in scene.tank[0]]
        self.tank.max[:] = [float(v) for v in scene.tank[1]]


def rest_positions(body: Body) -> np.ndarray:
    """lattice.js:171-179: every node's rest position, float32 (origin + (i,
    j, k) h in double, stored as the reference's Float32Array), (n, 3) in
    node order."""
    nx, ny, nz = body.node_dims
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    return (np.asarray(body.origin, np.float64) + ijk * body.h).astype(np.float32)


def static_nodes_in_region(positions, region=None) -> np.ndarray:
    """staticPrescription.js:9-20: the nodes whose rest position (x, y, z,
    float32 values) the body's declaration `region(x, y, z)` accepts, in
    node order, inactive nodes included; none without a declaration."""
    if region is None:
        return np.zeros(0, np.uint32)
    p = np.asarray(positions, np.float32).reshape(-1, 3).astype(np.float64)
    return np.asarray([n for n in range(len(p)) if region(p[n, 0], p[n, 1], p[n, 2])], np.uint32)


def with_static_region(body: Body, region) -> Body:
    """The body with its static nodes sampled from a declaration on its rest
    positions (simulator.js:64)."""
    return Body(body.cell_dims, body.origin, body.h, body.occupancy, dict(body.material),
                static_nodes_in_region(rest_positions(body), region))


def node_index(dims, i, j, k):
    nx, ny, _ = dims
    return i + nx * (j + ny * k)


def face_nodes(node_dims, axis: int, side: int) -> np.ndarray:
    """Body-local indices of the nodes on one face of the node grid."""
    nx, ny, nz = node_dims
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    coord = (i, j, k)[axis]
    last = node_dims[axis] - 1
    mask = coord == (0 if side == 0 else last)
    return np.sort((i + nx * (j + ny * k))[mask].astype(np.uint32))


def value_noise(n: int, seed: int, octaves: int = 3, base: int = 4) -> np.ndarray:
    """Seeded value noise in [0, 1] sampled at the centres of an n^3 grid
    (array indexed [k, j, i]): `octaves` octaves of smoothstep-interpolated
    random lattice values, frequencies base * 2^o, amplitudes 2^-o."""
    rng = np.random.default_rng(seed)
    coords = (np.arange(n) + 0.5) / n
    total = np.zeros((n, n, n))
    norm = 0.0
    for o in range(octaves):
        freq = base * 2 ** o
        amp = 0.5 ** o
        lattice = rng.random((freq + 1, freq + 1, freq + 1))
        x = coords * freq
        i0 = np.minimum(np.floor(x).astype(int), freq - 1)
        t = x - i0
        s = t * t * (3 - 2 * t)
        # trilinear over the 8 lattice corners, axes (k, j, i)
        acc = np.zeros((n, n, n))
        for dk in (0, 1):
            wk = (s if dk else 1 - s)[:, None, None]
            for dj in (0, 1):
                wj = (s if dj else 1 - s)[None, :, None]
                for di in (0, 1):
                    wi = (s if di else 1 - s)[None, None, :]
                    acc += wk * wj * wi * lattice[np.ix_(i0 + dk, i0 + dj, i0 + di)]
        total += amp * acc
        norm += amp
    return total / norm


def largest_component(mask: np.ndarray) -> np.ndarray:
    """The largest 6-connected component of a boolean grid."""
    from scipy import ndimage

    labels, count = ndimage.label(mask)
    if count == 0:
        return mask
    sizes = np.bincount(labels.ravel())
    sizes[0] = 0
    return labels == int(np.argmax(sizes))


def noise_occupancy(n: int, seed: int, threshold: float = 0.5) -> np.ndarray:
    """Occupancy (uint8, x fastest) of a seeded noise blob on an n^3 grid."""
    occ = largest_component(value_noise(n, seed) > threshold)
    return np.ascontiguousarray(occ.astype(np.uint8)).ravel()


def log_uniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size))


def splats_in(body: Body, count: int, seed: int):
    """`count` Gaussians inside the occupied cells of `body`."""
    rng = np.random.default_rng(seed)
    occ = np.flatnonzero(body.occupancy)
    cx, cy, _ = body.cell_dims
    cells = occ[rng.integers(0, occ.size, count)]
    ijk = np.stack([cells % cx, (cells // cx) % cy, cells // (cx * cy)], axis=1).astype(np.float64)
    means = (np.asarray(body.origin) + (ijk + rng.random((count, 3))) * body.h).astype(np.float32)
    quats = rng.normal(size=(count, 4))
    quats /= np.linalg.norm(quats, axis=1, keepdims=True)
    scales = np.exp(rng.uniform(math.log(1e-3), math.log(1e-2), (count, 3)))
    opacity = rng.uniform(0.1, 1.0, count)
    rgb = rng.random((count, 3))
    return (np.ascontiguousarray(means, np.float32), np.ascontiguousarray(quats, np.float32),
            np.ascontiguousarray(scales, np.float32), opacity.astype(np.float32), rgb.astype(np.float32))


# ---- the workloads ----------------------------------------------------------

def single_box() -> Scene:
    """16 x 4 x 4 cells (17 x 5 x 5 = 425 nodes), h = 0.016 m, E = 1e5 Pa,
    nu = 0.45, rho = 1000; the x = 0 face pinned; dt = 1/60 in 10 substeps;
    no contact and no ground (the tank is unbounded)."""
    dims = (16, 4, 4)
    mat = dict(DEFAULT_MATERIAL, youngs_modulus=1e5, poisson_ratio=0.45, density=1000.0)
    body = Body(dims, (0.0, 0.0, 0.0), H, np.ones(16 * 4 * 4, np.uint8), mat,
                face_nodes((17, 5, 5), 0, 0))
    inf = float("inf")
    return Scene([body], ((-inf, -inf, -inf), (inf, inf, inf)), step_duration=1 / 600, substeps=10,
                 contact=False)


def noise_blob(n: int = 64, seed: int = 1, splats: int = 1_000_000, lift_cells: int = 2) -> Scene:
    """A seeded noise blob on an n^3 grid (E log-uniform 1e4-1e6, nu = 0.45,
    rho = 1000) above a ground plane at y = 0, with self contact through the
    grid broadphase and `splats` Gaussians; dt = 1/60 in 10 substeps."""
    rng = np.random.default_rng(seed + 7919)
    occ = noise_occupancy(n, seed)
    e = float(log_uniform(rng, 1e4, 1e6))
    mat = dict(DEFAULT_MATERIAL, youngs_modulus=e, poisson_ratio=0.45, density=1000.0)
    half = n * H / 2
    body = Body((n, n, n), (-half, lift_cells * H, -half), H, occ, mat)
    margin = 0.1 * n * H + 4 * H
    tank = ((-half - margin, 0.0, -half - margin), (half + margin, n * H + lift_cells * H + margin,
                                                   half + margin))
    scene = Scene([body], tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True)
    if splats:
        scene.splats[0] = splats_in(body, splats, seed + 1)
    return scene


def box_batch(count: int = 256, seed: int = 2, splats_per_body: int = 0, spacing_cells: int = 52) -> Scene:
    """`count` independent boxes, sides log-uniform in [4, 48] cells per axis,
    E log-uniform 1e4-1e6, nu U(0.30, 0.49), rho U(500, 1500), one random face
    pinned each, resting above a ground plane; laid out on a square grid far
    enough apart never to touch (body contact off, the ground is the tank
    floor); dt = 1/60 in 10 substeps."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(math.sqrt(count)))
    bodies = []
    for b in range(count):
        dims = tuple(int(round(v)) for v in log_uniform(rng, 4, 48, 3))
        mat = dict(DEFAULT_MATERIAL,
                   youngs_modulus=float(log_uniform(rng, 1e4, 1e6)),
                   poisson_ratio=float(rng.uniform(0.30, 0.49)),
                   density=float(rng.uniform(500, 1500)))
        face = int(rng.integers(0, 6))
        gx, gz = b % side, b // side
        origin = (gx * spacing_cells * H, 2 * H, gz * spacing_cells * H)
        node_dims = tuple(d + 1 for d in dims)
        occ = np.ones(dims[0] * dims[1] * dims[2], np.uint8)
        bodies.append(Body(dims, origin, H, occ, mat, face_nodes(node_dims, face // 2, face % 2)))
    extent = side * spacing_cells * H
    tank = ((-1.0, 0.0, -1.0), (extent + 1.0, 2.0, extent + 1.0))
    scene = Scene(bodies, tank, step_duration=1 / 600, substeps=10, contact=False)
    for b, body in enumerate(bodies):
        if splats_per_body:
            scene.splats[b] = splats_in(body, splats_per_body, seed * 100003 + b)
    return scene


def surface_nodes(body: Body) -> np.ndarray:
    """Body-local boundary nodes: some but not all of the eight incident
    cells occupied (lattice.js:128-158)."""
    cx, cy, cz = body.cell_dims
    occ = np.zeros((cz + 2, cy + 2, cx + 2), np.int32)
    occ[1:-1, 1:-1, 1:-1] = body.occupancy.reshape(cz, cy, cx)
    filled = (occ[:-1, :-1, :-1] + occ[:-1, :-1, 1:] + occ[:-1, 1:, :-1] + occ[:-1, 1:, 1:] +
              occ[1:, :-1, :-1] + occ[1:, :-1, 1:] + occ[1:, 1:, :-1] + occ[1:, 1:, 1:])
    return np.flatnonzero((filled > 0) & (filled < 8)).astype(np.uint32)


def session_pool(count: int = 1000, seed: int = 3, min_n: int = 8, max_n: int = 64):
    """Serving sessions: seeded noise blobs on n^3 grids, n log-uniform in
    [min_n, max_n], materials as the single large body's (E log-uniform
    1e4-1e6, nu 0.45, rho 1000), each resting above the ground at the
    origin. Returns (bodies, tank)."""
    rng = np.random.default_rng(seed)
    bodies = []
    for s in range(count):
        n = int(round(float(log_uniform(rng, min_n, max_n))))
        occ = noise_occupancy(n, seed * 1_000_003 + s)
        mat = dict(DEFAULT_MATERIAL, youngs_modulus=float(log_uniform(rng, 1e4, 1e6)), poisson_ratio=0.45,
                   density=1000.0)
        half = n * H / 2
        bodies.append(Body((n, n, n), (-half, 2 * H, -half), H, occ, mat))
    extent = max_n * H
    tank = ((-extent, 0.0, -extent), (extent, 2 * extent, extent))
    return bodies, tank


def drag_request(body: Body, rng, speed: float = 0.5):
    """A drag: a random surface node of `body` pulled along a seeded cubic
    Bezier starting at the node's rest position, at `speed` m/s."""
    nodes = surface_nodes(body)
    node = int(nodes[rng.integers(0, nodes.size)])
    nx, ny, _ = body.node_dims
    ijk = np.array([node % nx, (node // nx) % ny, node // (nx * ny)], float)
    p0 = np.asarray(body.origin) + ijk * body.h
    steps = rng.normal(scale=0.05, size=(3, 3))
    control = np.vstack([p0, p0 + steps[0], p0 + steps[0] + steps[1], p0 + steps.sum(axis=0)])
    return node, control.astype(np.float32), speed


def blob_and_sheet(n: int = 192, seed: int = 4, splats: int = 20_000_000) -> Scene:
    """A seeded noise blob on an n^3 grid plus an n x n x 2-cell sheet a few
    cells above it (E = 5e5, nu = 0.48), ground plane, self and body contact;
    dt = 1/60 in 20 substeps of 2 Gauss-Seidel iterations; `splats` Gaussians
    in the blob."""
    occ = noise_occupancy(n, seed)
    mat = dict(DEFAULT_MATERIAL, youngs_modulus=5e5, poisson_ratio=0.48, density=1000.0)
    half = n * H / 2
    blob = Body((n, n, n), (-half, 2 * H, -half), H, occ, mat)
    sheet = Body((n, 2, n), (-half, (n + 6) * H, -half), H, np.ones(n * 2 * n, np.uint8), dict(mat))
    margin = 8 * H
    tank = ((-half - margin, 0.0, -half - margin), (half + margin, (n + 12) * H, half + margin))
    scene = Scene([blob, sheet], tank, step_duration=1 / 1200, substeps=20, iterations=2, contact=True,
                  self_contact=True)
    if splats:
        scene.splats[0] = splats_in(blob, splats, seed + 1)
    return scene


MATERIAL_KEYS = ("youngs_modulus", "poisson_ratio", "density", "friction", "damping", "relaxation", "max_stretch")


def tank_scene(fixture) -> Scene:
    """The reference's `tank` scene (apps/simulator/src/scene/tank.js:47-83):
    two meshes (spot, suzanne) and three analytic shapes (torus, sphere,
    cube) above a 0.6 x 0.5 x 0.4 m open-topped tank, each body's cells
    as the reference's voxelisers produce them (vsim.voxelize), read from
    `fixture` (an npz written by tests/golden/make_tank_fixture.py). The
    step duration is left to the CFL rule, contact between bodies is on,
    self contact off, as in the reference."""
    z = np.load(fixture) if not isinstance(fixture, dict) else fixture
    bodies = []
    for b in range(len(z["names"])):
        dims = tuple(int(v) for v in z[f"dims{b}"])
        occupancy = np.unpackbits(z[f"occupancy{b}"])[: dims[0] * dims[1] * dims[2]].astype(np.uint8)
        material = {k: float(v) for k, v in zip(MATERIAL_KEYS, z[f"material{b}"])}
        bodies.append(Body(dims, tuple(float(v) for v in z[f"origin{b}"]), float(z[f"h{b}"]), occupancy, material))
    tank = (tuple(float(v) for v in z["tank_min"]), tuple(float(v) for v in z["tank_max"]))
    return Scene(bodies, tank, step_duration=None, substeps=24, contact=True, self_contact=False)



def capture_cloud(count: int, radius: float, seed: int):
    """A synthetic capture: `count` Gaussians on the surface of a sphere of
    `radius` (golden-angle spiral, radial jitter N(0, (radius/200)^2)), with
    nothing behind the surface, as a scan gives. Scales log-uniform in
    [0.4, 1.6] x the sample spacing per axis, uniformly random unit
    quaternions (x, y, z, w). Returns float32 (positions, rotations,
    scales)."""
    rng = np.random.default_rng(seed)
    i = np.arange(count, dtype=np.float64)
    y = 1 - 2 * (i + 0.5) / count
    ring = np.sqrt(np.maximum(0.0, 1 - y * y))
    theta = math.pi * (3 - math.sqrt(5)) * i
    r = radius + rng.normal(scale=radius / 200, size=count)
    positions = np.stack([np.cos(theta) * ring * r, y * r, np.sin(theta) * ring * r], axis=1)
    spacing = math.sqrt(4 * math.pi * radius * radius / count)
    scales = log_uniform(rng, 0.4 * spacing, 1.6 * spacing, (count, 3))
    quats = rng.normal(size=(count, 4))
    quats /= np.linalg.norm(quats, axis=1, keepdims=True)
    return (positions.astype(np.float32), quats.astype(np.float32), scales.astype(np.float32))


def captured_cloud(count: int = 200_000, radius: float = 0.1, element_size: float = 0.008, seed: int = 5,
                   lift: float = 0.02) -> Scene:
    """A captured Gaussian cloud as a body, the reference's "cloud" rest
    geometry (voxelLattice.js:208-226): `capture_cloud`'s shell lifted so its
    lowest ellipsoid reach sits `lift` above the ground, voxelised by
    vsim.voxelize.voxelize_cloud (stamped, sealed, filled), the cloud's own
    Gaussians as the body's splats (each centre in a solid cell by
    construction). E = 2e5, nu = 0.45, rho = 1000; ground and self contact;
    dt = 1/60 in 10 substeps."""
    from . import voxelize

    positions, quats, scales = capture_cloud(count, radius, seed)
    grid = voxelize.voxelize_cloud(positions, quats, scales, element_size)
    drop = lift - (grid.origin[1] + voxelize.DEFAULT_PADDING * grid.h)
    positions = (positions.astype(np.float64) + [0.0, drop, 0.0]).astype(np.float32)
    grid = voxelize.voxelize_cloud(positions, quats, scales, element_size)
    mat = dict(DEFAULT_MATERIAL, youngs_modulus=2e5, poisson_ratio=0.45, density=1000.0)
    body = Body(tuple(grid.dims), tuple(grid.origin), grid.h, grid.occupancy, mat)
    hi = [grid.origin[a] + grid.dims[a] * grid.h for a in range(3)]
    margin = 0.5 * radius
    tank = ((grid.origin[0] - margin, 0.0, grid.origin[2] - margin), (hi[0] + margin, hi[1] + margin, hi[2] + margin))
    scene = Scene([body], tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True)
    rng = np.random.default_rng(seed + 1)
    scene.splats[0] = (positions, quats, scales, rng.uniform(0.1, 1.0, count).astype(np.float32),
                       rng.random((count, 3)).astype(np.float32))
    return scene
