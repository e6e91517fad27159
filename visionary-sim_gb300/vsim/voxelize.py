"""Rest geometry to occupancy grid: the reference's asset preparation and
voxelisers, restated on the host so that scenes built from meshes and
analytic shapes get exactly the reference's cells.

Follows, operation by operation in JavaScript's double arithmetic (mesh
vertices stored as float32, as the reference's Float32Array does):

- `apps/simulator/src/assets/objLoader.js:22-119` -- OBJ parsing, normalising
  to a size, translating;
- `packages/visionary-sim/src/body/restGeometry.js:31-43` -- mesh bounds;
- `apps/simulator/src/assets/shapes.js:29-172` -- torus, sphere and box
  signed distances, `translateShape`, `restOnGround` (the drawn surfaces are
  not needed here);
- `packages/visionary-sim/src/sim/discretize/lattice/voxelize.js:19-435` --
  `gridForBounds`, `voxelizeSdf`, `voxelizeMesh` (three-axis ray parity with a
  majority vote, edge marking, 6-neighbourhood close);
- `packages/visionary-sim/src/sim/discretize/lattice/cloudVolume.js:70-397`
  -- `voxelizeCloud`: a Gaussian cloud stamped as solid ellipsoids, sealed,
  flood-filled from the faces and eroded back (with `mat3FromQuat`,
  `mat3.js:71-87`, and `locate`, `sample.js:42-55`).

The result feeds `vsim_create` as a body's cell grid (cell_dims, origin, h,
occupancy).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable

import numpy as np


@dataclass
class Mesh:
    positions: np.ndarray  # float32, (n, 3)
    indices: np.ndarray    # uint32, (m, 3)


@dataclass
class Shape:
    sdf: Callable[[float, float, float], float]
    bounds: tuple           # (min xyz, max xyz), doubles


@dataclass
class OccupancyGrid:
    dims: list
    origin: list
    h: float
    occupancy: np.ndarray  # uint8, dims[0] * dims[1] * dims[2], x fastest


# ---- objLoader.js -------------------------------------------------------------

def parse_obj(text: str) -> Mesh:
    """objLoader.js:22-67: positions and fan-triangulated faces."""
    positions, indices = [], []
    for raw in text.split("\n"):
        line = raw.strip()
        if not line or line[0] == "#":
            continue
        if line.startswith("v "):
            parts = line.split()
            positions.append((float(parts[1]), float(parts[2]), float(parts[3])))
            continue
        if not line.startswith("f "):
            continue
        face = []
        count = len(positions)
        for token in line.split()[1:]:
            head = token.split("/")[0]
            try:
                index = int(head)
            except ValueError:
                continue
            face.append(index - 1 if index > 0 else count + index)
        for i in range(2, len(face)):
            indices.append((face[0], face[i - 1], face[i]))
    return Mesh(np.asarray(positions, np.float32).reshape(-1, 3), np.asarray(indices, np.uint32).reshape(-1, 3))


def mesh_bounds(positions: np.ndarray):
    """restGeometry.js:31-43."""
    p = positions.astype(np.float64)
    return [float(v) for v in p.min(axis=0)], [float(v) for v in p.max(axis=0)]


def normalize_mesh(mesh: Mesh, target_size: float) -> Mesh:
    """objLoader.js:86-103: the largest axis scaled to `target_size`, centred in
    x and z, base at y = 0; each result rounded to float32."""
    lo, hi = mesh_bounds(mesh.positions)
    extent = [hi[a] - lo[a] for a in range(3)]
    scale = target_size / max(extent)
    centre_x = (lo[0] + hi[0]) * 0.5
    centre_z = (lo[2] + hi[2]) * 0.5
    p = mesh.positions.astype(np.float64)
    out = np.empty_like(mesh.positions)
    out[:, 0] = ((p[:, 0] - centre_x) * scale).astype(np.float32)
    out[:, 1] = ((p[:, 1] - lo[1]) * scale).astype(np.float32)
    out[:, 2] = ((p[:, 2] - centre_z) * scale).astype(np.float32)
    return Mesh(out, mesh.indices)


def translate_mesh(mesh: Mesh, offset) -> Mesh:
    """objLoader.js:110-117."""
    p = mesh.positions.astype(np.float64) + np.asarray(offset, np.float64)
    return Mesh(p.astype(np.float32), mesh.indices)


def hypot_js(*values: float) -> float:
    """JavaScript's Math.hypot as V8 evaluates it (its published math
    builtin): infinity if any argument is infinite, else NaN if any is NaN,
    else 0 if all are 0; otherwise each magnitude is divided by the largest,
    the squares are summed in argument order with Kahan compensation, and
    the square root of the sum is multiplied by the largest. Python's
    math.hypot rounds differently in the last place."""
    mags = [abs(float(v)) for v in values]
    if any(math.isinf(m) for m in mags):
        return math.inf
    if any(math.isnan(m) for m in mags):
        return math.nan
    top = max(mags, default=0.0)
    if top == 0:
        return 0.0
    total = compensation = 0.0
    for m in mags:
        n = m / top
        summand = n * n - compensation
        preliminary = total + summand
        compensation = (preliminary - total) - summand
        total = preliminary
    return math.sqrt(total) * top


# ---- shapes.js ----------------------------------------------------------------

def torus(major_radius: float, minor_radius: float) -> Shape:
    """shapes.js:29-52 (a torus in the XZ plane)."""
    outer = major_radius + minor_radius

    def sdf(x, y, z):
        radial = hypot_js(x, z) - major_radius
        return hypot_js(radial, y) - minor_radius

    return Shape(sdf, ([-outer, -minor_radius, -outer], [outer, minor_radius, outer]))


def sphere(radius: float) -> Shape:
    """shapes.js:59-80."""
    return Shape(lambda x, y, z: hypot_js(x, y, z) - radius, ([-radius] * 3, [radius] * 3))


def box(half_extents) -> Shape:
    """shapes.js:87-115."""
    hx, hy, hz = half_extents

    def sdf(x, y, z):
        dx = abs(x) - hx
        dy = abs(y) - hy
        dz = abs(z) - hz
        outside = hypot_js(max(dx, 0), max(dy, 0), max(dz, 0))
        inside = min(max(dx, dy, dz), 0)
        return outside + inside

    return Shape(sdf, ([-hx, -hy, -hz], [hx, hy, hz]))


def translate_shape(shape: Shape, offset) -> Shape:
    """shapes.js:147-161."""
    dx, dy, dz = offset
    lo, hi = shape.bounds
    inner = shape.sdf
    return Shape(lambda x, y, z: inner(x - dx, y - dy, z - dz),
                 ([lo[0] + dx, lo[1] + dy, lo[2] + dz], [hi[0] + dx, hi[1] + dy, hi[2] + dz]))


def rest_on_ground(shape: Shape) -> Shape:
    """shapes.js:169-171: lowest point at y = 0."""
    return translate_shape(shape, [0, -shape.bounds[0][1], 0])


# ---- voxelize.js --------------------------------------------------------------

DEFAULT_PADDING = 2


def grid_for_bounds(bounds, element_size: float, padding: int = DEFAULT_PADDING) -> OccupancyGrid:
    """voxelize.js:40-67."""
    if not (element_size > 0 and math.isfinite(element_size)):
        raise ValueError(f"element_size must be a positive length in metres, got {element_size}")
    h = element_size
    lo, hi = bounds
    extent = [hi[a] - lo[a] for a in range(3)]
    dims = [max(1, math.ceil(e / h - 1e-6)) + 2 * padding for e in extent]
    origin = [v - h * padding for v in lo]
    return OccupancyGrid(dims, origin, h, np.zeros(dims[0] * dims[1] * dims[2], np.uint8))


def voxelize_sdf(shape: Shape, element_size: float, padding: int = DEFAULT_PADDING) -> OccupancyGrid:
    """voxelize.js:124-143 with anyCornerInside (:153-165): a cell is material
    when its centre is within half a cell of the surface or any corner is
    inside; the grid is shifted half a cell so centres land on the bounds."""
    grid = grid_for_bounds(shape.bounds, element_size, padding)
    h = grid.h
    origin = [v - h * 0.5 for v in grid.origin]
    grid.origin = origin
    threshold = h * 0.5
    nx, ny, nz = grid.dims
    sdf = shape.sdf
    occ = grid.occupancy
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                x = origin[0] + i * h
                y = origin[1] + j * h
                z = origin[2] + k * h
                if sdf(x + h * 0.5, y + h * 0.5, z + h * 0.5) < threshold or any(
                        sdf(x + (h if c & 1 else 0), y + (h if c & 2 else 0), z + (h if c & 4 else 0)) < 0
                        for c in range(8)):
                    occ[i + nx * (j + ny * k)] = 1
    return grid


def voxelize_mesh(mesh: Mesh, bounds, element_size: float, padding: int = DEFAULT_PADDING,
                  close: bool = True) -> OccupancyGrid:
    """voxelize.js:178-200."""
    grid = grid_for_bounds(bounds, element_size, padding)
    n = grid.occupancy.size
    votes = np.zeros(n, np.uint8)
    surface = np.zeros(n, np.uint8)
    for axis in range(3):
        _accumulate_axis(mesh, grid, axis, votes, surface)
    _mark_edge_cells(mesh, grid, surface)
    grid.occupancy[:] = ((votes >= 2) | (surface == 1)).astype(np.uint8)
    if close:
        morphological_close(grid)
    return grid


# ---- cloudVolume.js -----------------------------------------------------------

CLOUD_SIGMA = 2
CLOUD_SEAL = 2
# cloudVolume.js:86: a cell's eight corners (corners.js:12-21 order), then its centre.
_CELL_SAMPLES = [(c & 1, (c >> 1) & 1, (c >> 2) & 1) for c in range(8)] + [(0.5, 0.5, 0.5)]


def quat_to_columns(q) -> np.ndarray:
    """mat3.js:71-87 (mat3FromQuat) for quaternions (n, 4) in x, y, z, w
    order: column-major rotations (n, 9), each entry computed in double and
    stored as float32 like the reference's Float32Array."""
    q = np.asarray(q, np.float64).reshape(-1, 4)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    out = np.empty((len(q), 9), np.float32)
    out[:, 0] = 1 - 2 * (y * y + z * z)
    out[:, 1] = 2 * (x * y + z * w)
    out[:, 2] = 2 * (x * z - y * w)
    out[:, 3] = 2 * (x * y - z * w)
    out[:, 4] = 1 - 2 * (x * x + z * z)
    out[:, 5] = 2 * (y * z + x * w)
    out[:, 6] = 2 * (x * z + y * w)
    out[:, 7] = 2 * (y * z - x * w)
    out[:, 8] = 1 - 2 * (x * x + y * y)
    return out


def js_hypot(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """`hypot_js` of three arguments, elementwise over arrays."""
    v = np.abs(np.stack([np.asarray(a, np.float64), np.asarray(b, np.float64), np.asarray(c, np.float64)]))
    top = v.max(axis=0)
    safe = np.where(top > 0, top, 1.0)
    total = np.zeros_like(top)
    compensation = np.zeros_like(top)
    with np.errstate(invalid="ignore"):
        for r in range(3):
            n = v[r] / safe
            summand = n * n - compensation
            preliminary = total + summand
            compensation = (preliminary - total) - summand
            total = preliminary
        out = np.sqrt(total) * top
    out = np.where(top == 0, 0.0, out)
    out = np.where(np.isnan(v).any(axis=0), np.nan, out)
    return np.where(np.isinf(v).any(axis=0), np.inf, out)


def _ellipsoids(rotations, scales, sigma: float):
    """cloudVolume.js:195-210 (ellipsoidOf) for every Gaussian: the float32
    column-major rotations, the half-axes sigma * scale, and the reach along
    each world axis (the length of that row of R * diag(radius))."""
    columns = quat_to_columns(np.asarray(rotations, np.float32))
    radius = sigma * np.asarray(scales, np.float32).astype(np.float64).reshape(-1, 3)
    col = columns.astype(np.float64)
    half = np.stack([js_hypot(col[:, a] * radius[:, 0], col[:, 3 + a] * radius[:, 1], col[:, 6 + a] * radius[:, 2])
                     for a in range(3)], axis=1)
    return col, radius, half


def locate(origin, h: float, cell_dims, x: float, y: float, z: float):
    """sample.js:42-55: the cell holding a world point (clamped into the
    grid) and the point's local coordinates within it -- how the render side
    finds a Gaussian's cell."""
    cell, local = [0, 0, 0], [0.0, 0.0, 0.0]
    for a, p in enumerate((x, y, z)):
        g = (float(p) - origin[a]) / h
        index = min(max(math.floor(g), 0), cell_dims[a] - 1)
        cell[a] = index
        local[a] = g - index
    return cell, local


def voxelize_cloud(positions, rotations, scales, element_size: float, padding: int = DEFAULT_PADDING,
                   sigma: float = CLOUD_SIGMA, seal: int = CLOUD_SEAL, fill: bool = True,
                   stats: dict | None = None) -> OccupancyGrid:
    """cloudVolume.js:101-123 (voxelizeCloud): a Gaussian cloud (centres
    (n, 3), quaternions (n, 4) x-y-z-w, scales (n, 3), all float32 as the
    reference stores them) to an occupancy grid. Every Gaussian is stamped as
    a solid ellipsoid at `sigma` standard deviations, with the cell holding
    its centre always material; with `fill`, the shell is dilated `seal`
    times, every cell the outside cannot reach through face neighbours is
    filled, the result is eroded `seal` times and the stamp is put back.
    With `stats`, the occupied cells and the fill's count are stored in it."""
    pos = np.asarray(positions, np.float32).astype(np.float64).reshape(-1, 3)
    if len(pos) == 0:
        raise ValueError("voxelizeCloud: a cloud with no Gaussians has no volume")
    columns, radius, half = _ellipsoids(rotations, scales, sigma)
    # cloudVolume.js:219-234 (materialBounds)
    lo = [float(np.min(pos[:, a] - half[:, a])) for a in range(3)]
    hi = [float(np.max(pos[:, a] + half[:, a])) for a in range(3)]
    extent = [hi[a] - lo[a] for a in range(3)]
    # Math.max of the extents is NaN when any is, and the check then fails
    if any(math.isnan(e) for e in extent) or not (max(extent) > 0):
        raise ValueError("voxelizeCloud: a cloud with no extent has no volume")
    grid = grid_for_bounds((lo, hi), element_size, padding)
    _stamp_cloud(grid, pos, columns, radius, half)
    filled = _seal_and_fill(grid, seal) if fill else 0
    if stats is not None:
        stats.update(occupied=count_occupied(grid), filled=filled)
    return grid


def set_flood_rounds(rounds: int) -> int:
    """Caps the rounds of flood sweeps `voxelize_cloud_on_device`'s fill runs
    before its union-find decides (vsim_cloud_set_flood_rounds; 0: always the
    union-find), process-wide; returns the previous cap. Both paths give the
    flood's set; this is for testing each."""
    from . import _ffi

    return int(_ffi.lib().vsim_cloud_set_flood_rounds(int(rounds)))


def voxelize_cloud_on_device(positions, rotations, scales, element_size: float, padding: int = DEFAULT_PADDING,
                             sigma: float = CLOUD_SIGMA, seal: int = CLOUD_SEAL, fill: bool = True,
                             stats: dict | None = None) -> OccupancyGrid:
    """`voxelize_cloud` on the GPU through libvsim (`vsim_voxelize_cloud`,
    csrc/cloud_volume.cu): the same grid, cell for cell. `positions`,
    `rotations` and `scales` are host arrays, or CUDA torch tensors (then
    nothing is copied in). With `stats`, the occupied and filled cell counts
    are stored in it. Raises when the library is not built."""
    import ctypes as C

    from . import _ffi

    lib = _ffi.lib()
    opts = _ffi.CloudOptions(float(element_size), float(sigma), int(padding), int(seal), 1 if fill else 0)
    vol = C.c_void_p()
    if hasattr(positions, "data_ptr"):
        count = int(positions.numel() // 3)
        tensors = [t.contiguous().float() for t in (positions, rotations, scales)]
        _ffi.check(lib.vsim_voxelize_cloud_device(tensors[0].data_ptr(), tensors[1].data_ptr(), tensors[2].data_ptr(),
                                                  count, C.byref(opts), None, C.byref(vol)))
    else:
        arrays = [np.ascontiguousarray(np.asarray(a, np.float32)) for a in (positions, rotations, scales)]
        count = arrays[0].size // 3
        _ffi.check(lib.vsim_voxelize_cloud(_ffi.fptr(arrays[0]), _ffi.fptr(arrays[1]), _ffi.fptr(arrays[2]), count,
                                           C.byref(opts), C.byref(vol)))
    try:
        g = _ffi.CloudGrid()
        _ffi.check(lib.vsim_cloud_volume_grid(vol, C.byref(g)))
        dims = [int(v) for v in g.dims]
        occupancy = np.zeros(dims[0] * dims[1] * dims[2], np.uint8)
        _ffi.check(lib.vsim_cloud_volume_read(vol, occupancy.ctypes.data_as(C.POINTER(C.c_uint8)), occupancy.size))
        if stats is not None:
            stats.update(occupied=int(g.occupied), filled=int(g.filled))
        return OccupancyGrid(dims, [float(v) for v in g.origin], float(g.h), occupancy)
    finally:
        lib.vsim_cloud_volume_destroy(vol)


def _stamp_cloud(grid: OccupancyGrid, pos, columns, radius, half, budget: int = 1 << 22) -> None:
    """cloudVolume.js:138-178 (stampCloud) with cellMeetsEllipsoid (:252-276).
    Marking is an OR, so the Gaussians are taken in groups of equal box shape
    rather than one by one; each sample is the reference's double
    arithmetic in its order."""
    dims, origin, h = grid.dims, grid.origin, grid.h
    occ = grid.occupancy
    nx, ny = dims[0], dims[1]
    dims_a = np.asarray(dims)
    origin_a = np.asarray(origin, np.float64)
    # cloudVolume.js:384-386 (cellOf): the centre's cell, clamped into the grid
    centre_cell = np.clip(np.floor((pos - origin_a) / h), 0, dims_a - 1).astype(np.int64)
    occ[centre_cell[:, 0] + nx * (centre_cell[:, 1] + ny * centre_cell[:, 2])] = 1
    # cloudVolume.js:395-397 (offFace): the box, one cell inside both faces
    lo = np.clip(np.floor((pos - half - origin_a) / h), 1, dims_a - 2).astype(np.int64)
    hi = np.clip(np.floor((pos + half - origin_a) / h), 1, dims_a - 2).astype(np.int64)
    shape = np.maximum(hi - lo + 1, 0)
    shapes, group = np.unique(shape, axis=0, return_inverse=True)
    group = group.reshape(-1)
    for g, (bx, by, bz) in enumerate(shapes):
        cells = int(bx) * int(by) * int(bz)
        if cells == 0:
            continue
        members = np.nonzero(group == g)[0]
        kk, jj, ii = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
        offset = np.stack([ii.reshape(-1), jj.reshape(-1), kk.reshape(-1)], axis=1)
        step = max(1, budget // (cells * len(_CELL_SAMPLES)))
        for start in range(0, len(members), step):
            m = members[start:start + step]
            ijk = lo[m][:, None, :] + offset[None, :, :]                      # (g, cells, 3)
            hit = np.zeros(ijk.shape[:2], bool)
            c = columns[m][:, None, :]
            r = radius[m][:, None, :]
            centre = pos[m][:, None, :]
            with np.errstate(divide="ignore", invalid="ignore"):
                for sample in _CELL_SAMPLES:
                    d = [origin[a] + (ijk[..., a] + sample[a]) * h - centre[..., a] for a in range(3)]
                    total = np.zeros(ijk.shape[:2])
                    for a in range(3):
                        t = (c[..., 3 * a] * d[0] + c[..., 3 * a + 1] * d[1] + c[..., 3 * a + 2] * d[2]) / r[..., a]
                        total = total + t * t
                    hit |= total <= 1
            # the reference's cellIndex of the box coordinates; with padding
            # under two cells a box can leave the grid, and like its typed
            # array the grid ignores an index outside it
            index = ijk[..., 0] + nx * (ijk[..., 1] + ny * ijk[..., 2])
            hit &= (index >= 0) & (index < occ.size)
            occ[index[hit]] = 1


def _seal_and_fill(grid: OccupancyGrid, seal: int) -> int:
    """cloudVolume.js:291-306 (sealAndFill)."""
    stamp = grid.occupancy.copy()
    for _ in range(seal):
        grid.occupancy[:] = _neighbourhood_pass(grid, grid.occupancy, True)
    filled = fill_enclosed(grid)
    for _ in range(seal):
        grid.occupancy[:] = _neighbourhood_pass(grid, grid.occupancy, False)
    grid.occupancy |= stamp
    return filled


def fill_enclosed(grid: OccupancyGrid) -> int:
    """cloudVolume.js:321-375 (fillEnclosed): every empty cell that no
    face-connected path of empty cells joins to the grid's faces becomes
    material; returns how many. The flood from the faces is the set of
    6-connected empty components touching a face."""
    from scipy import ndimage

    nx, ny, nz = grid.dims
    empty = grid.occupancy.reshape(nz, ny, nx) == 0
    labels, _ = ndimage.label(empty, structure=ndimage.generate_binary_structure(3, 1))
    faces = np.concatenate([labels[0].ravel(), labels[-1].ravel(), labels[:, 0].ravel(), labels[:, -1].ravel(),
                            labels[:, :, 0].ravel(), labels[:, :, -1].ravel()])
    reached = np.isin(labels, np.unique(faces[faces > 0]))
    enclosed = (empty & ~reached).reshape(-1)
    grid.occupancy[enclosed] = 1
    return int(enclosed.sum())


def voxelize_source(kind: str, source, element_size: float) -> OccupancyGrid:
    """voxelLattice.js:208-226 (VOXELIZERS, proxyFor): rest geometry of kind
    "mesh" (a Mesh, laid out over its own bounds), "shape" (a Shape) or
    "cloud" (positions, rotations, scales) to its cell grid, cells
    `element_size` across; any other kind is refused."""
    if kind == "mesh":
        return voxelize_mesh(source, mesh_bounds(source.positions), element_size)
    if kind == "shape":
        return voxelize_sdf(source, element_size)
    if kind == "cloud":
        return voxelize_cloud(*source, element_size)
    raise ValueError(f'no way to discretise rest geometry of kind "{kind}"')


def cell_index(grid: OccupancyGrid, i: int, j: int, k: int) -> int:
    """voxelize.js:76-78."""
    return i + grid.dims[0] * (j + grid.dims[1] * k)


def count_occupied(grid: OccupancyGrid) -> int:
    """voxelize.js:84-90."""
    return int(grid.occupancy.sum())


def morphological_close(grid: OccupancyGrid) -> None:
    """voxelize.js:389-391: dilate then erode, in place."""
    grid.occupancy[:] = _neighbourhood_pass(grid, _neighbourhood_pass(grid, grid.occupancy, True), False)


def _cell(grid: OccupancyGrid, i: int, j: int, k: int) -> int:
    return i + grid.dims[0] * (j + grid.dims[1] * k)


def _mark_edge_cells(mesh: Mesh, grid: OccupancyGrid, surface: np.ndarray):
    """voxelize.js:214-248: every cell a triangle edge passes through."""
    dims, origin, h = grid.dims, grid.origin, grid.h
    step = h * 0.4
    pos = mesh.positions.astype(np.float64)
    for tri in mesh.indices:
        for e in range(3):
            a = pos[int(tri[e])]
            b = pos[int(tri[(e + 1) % 3])]
            dx = float(b[0]) - float(a[0])
            dy = float(b[1]) - float(a[1])
            dz = float(b[2]) - float(a[2])
            steps = max(1, math.ceil(hypot_js(dx, dy, dz) / step))
            ax, ay, az = float(a[0]), float(a[1]), float(a[2])
            for s in range(steps + 1):
                f = s / steps
                i = math.floor((ax + dx * f - origin[0]) / h)
                j = math.floor((ay + dy * f - origin[1]) / h)
                k = math.floor((az + dz * f - origin[2]) / h)
                if 0 <= i < dims[0] and 0 <= j < dims[1] and 0 <= k < dims[2]:
                    surface[_cell(grid, i, j, k)] = 1


def _accumulate_axis(mesh: Mesh, grid: OccupancyGrid, axis: int, votes: np.ndarray, surface: np.ndarray):
    """voxelize.js:265-360: one ray per cell column along `axis` (sampled a
    fixed sub-cell jitter off the centre); cells past an odd number of
    crossings vote interior, crossed cells hold surface."""
    dims, origin, h = grid.dims, grid.origin, grid.h
    u, v, w = (axis + 1) % 3, (axis + 2) % 3, axis
    crossings = {}
    jitter_u = h * 1.7e-4
    jitter_v = h * 0.9e-4
    pos = mesh.positions.astype(np.float64)
    for tri in mesh.indices:
        a, b, c = pos[int(tri[0])], pos[int(tri[1])], pos[int(tri[2])]
        au, av, aw = float(a[u]), float(a[v]), float(a[w])
        bu, bv, bw = float(b[u]), float(b[v]), float(b[w])
        cu, cv, cw = float(c[u]), float(c[v]), float(c[w])
        area2 = (bv - cv) * (au - cu) + (cu - bu) * (av - cv)
        if abs(area2) < 1e-20:
            continue
        inv_area2 = 1 / area2
        min_u, max_u = min(au, bu, cu), max(au, bu, cu)
        min_v, max_v = min(av, bv, cv), max(av, bv, cv)
        a0 = max(0, math.ceil((min_u - origin[u]) / h - 0.5))
        a1 = min(dims[u] - 1, math.floor((max_u - origin[u]) / h - 0.5))
        b0 = max(0, math.ceil((min_v - origin[v]) / h - 0.5))
        b1 = min(dims[v] - 1, math.floor((max_v - origin[v]) / h - 0.5))
        for cv2 in range(b0, b1 + 1):
            pv = origin[v] + (cv2 + 0.5) * h + jitter_v
            for cu2 in range(a0, a1 + 1):
                pu = origin[u] + (cu2 + 0.5) * h + jitter_u
                l0 = ((bv - cv) * (pu - cu) + (cu - bu) * (pv - cv)) * inv_area2
                if l0 < 0:
                    continue
                l1 = ((cv - av) * (pu - cu) + (au - cu) * (pv - cv)) * inv_area2
                if l1 < 0:
                    continue
                l2 = 1 - l0 - l1
                if l2 < 0:
                    continue
                crossings.setdefault(cu2 + dims[u] * cv2, []).append(l0 * aw + l1 * bw + l2 * cw)
    ijk = [0, 0, 0]
    for column, hits in crossings.items():
        hits.sort()
        ijk[u] = column % dims[u]
        ijk[v] = column // dims[u]
        for hit in hits:
            cw = math.floor((hit - origin[w]) / h)
            if 0 <= cw < dims[w]:
                ijk[w] = cw
                surface[_cell(grid, *ijk)] = 1
        nxt, inside = 0, False
        for cw in range(dims[w]):
            centre = origin[w] + (cw + 0.5) * h
            while nxt < len(hits) and hits[nxt] <= centre:
                inside = not inside
                nxt += 1
            if inside:
                ijk[w] = cw
                votes[_cell(grid, *ijk)] += 1


def _neighbourhood_pass(grid: OccupancyGrid, source: np.ndarray, dilate: bool) -> np.ndarray:
    """voxelize.js:402-435: 6-neighbourhood dilate or erode; outside the grid
    counts as empty."""
    nx, ny, nz = grid.dims
    s = source.reshape(nz, ny, nx).astype(bool)
    padded = np.pad(s, 1, constant_values=False)
    neighbours = [padded[1:-1, 1:-1, 2:], padded[1:-1, 1:-1, :-2], padded[1:-1, 2:, 1:-1],
                  padded[1:-1, :-2, 1:-1], padded[2:, 1:-1, 1:-1], padded[:-2, 1:-1, 1:-1]]
    if dilate:
        out = s | np.logical_or.reduce(neighbours)
    else:
        out = s & np.logical_and.reduce(neighbours)
    return out.reshape(-1).astype(np.uint8)
