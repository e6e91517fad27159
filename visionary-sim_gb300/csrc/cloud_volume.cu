// A Gaussian cloud to an occupancy grid on the device: voxelizeCloud
// (packages/visionary-sim/src/sim/discretize/lattice/cloudVolume.js:101-397),
// the reference's "cloud" rest geometry (voxelLattice.js:208-226).
//
// The reference runs it on the CPU in JavaScript doubles. Here every step is
// a kernel, in the same double arithmetic and order, so the grid is the same
// cell for cell:
//   1. bounds: each Gaussian's ellipsoid reach (materialBounds, :219-234),
//      reduced with order-preserving 64-bit keys;
//   2. the grid laid out on the host from the bounds (gridForBounds,
//      voxelize.js:40-67);
//   3. stamp: a thread per Gaussian marks its centre cell and tests the
//      cells of its box against the ellipsoid (stampCloud, :138-178); a box
//      of more than kInlineBoxCells cells is handed to a block instead;
//   4. seal and fill (:291-306): 6-neighbourhood dilations, the fill, as
//      many erosions, the stamp put back. The reference fills by flooding
//      the empty cells from the grid's faces (fillEnclosed, :321-375); the
//      cells a flood reaches are exactly the face-connected components of
//      empty cells that touch a face, found here by a concurrent union-find
//      (x runs seeded by warp ballots, links by atomicMin on roots, path
//      halving by plain stores) instead of a serial flood.
// Marking is an OR (a cell is set by any Gaussian that reaches it), and the
// components of a graph do not depend on the order edges are merged, so no
// step's result depends on thread timing.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include <math_constants.h>

#include "sim_internal.cuh"

struct vsim_cloud_volume {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t dims[3]{};
    double origin[3]{};
    double h = 0;
    uint64_t cells = 0;
    uint64_t occupied = 0;
    uint64_t filled = 0;
    uint8_t* occupancy = nullptr;
};

namespace vsim {
namespace {

constexpr uint32_t kCloudBlock = 256;
constexpr uint32_t kInlineBoxCells = 64;    // larger boxes are stamped by a block each
// Caps of the union-find loops. Labels strictly fall along every walk, so
// the loops end by themselves; the caps, and the shared flag the first
// thread to reach one raises (every walk polls it), only bound the kernels'
// time on an input no test has seen.
constexpr uint32_t kFindLimit = 1u << 22;
constexpr uint32_t kUniteLimit = 1u << 16;
constexpr uint32_t kPollEvery = 1024;

struct CloudInput {
    const float* pos;    // xyz per Gaussian
    const float* rot;    // quaternion x, y, z, w
    const float* scale;  // standard deviations per axis, metres
    uint32_t count;
    double sigma;
};

struct GridView {
    uint32_t dims[3];
    double origin[3];
    double h;
    uint32_t cells;
};

// One Gaussian as an ellipsoid (cloudVolume.js:195-210): the column-major
// rotation as the reference's Float32Array holds it, the half-axes in the
// Gaussian's frame, the reach along each world axis.
struct Ellipsoid {
    double col[9];
    double radius[3];
    double half[3];
};

// JavaScript's Math.hypot as V8 evaluates it (its published math builtin):
// infinity if any argument is infinite, else NaN if any is NaN, else 0 when
// all are 0; otherwise the magnitudes over the largest, squared and summed in
// argument order with Kahan compensation, square root times the largest.
__device__ double hypotV8(double a, double b, double c) {
    a = fabs(a);
    b = fabs(b);
    c = fabs(c);
    if (isinf(a) || isinf(b) || isinf(c)) return CUDART_INF;
    if (isnan(a) || isnan(b) || isnan(c)) return CUDART_NAN;
    const double top = fmax(a, fmax(b, c));
    if (top == 0.0) return 0.0;
    const double v[3] = {a, b, c};
    double total = 0.0, compensation = 0.0;
    for (int r = 0; r < 3; r++) {
        // x / x is exactly 1 and 0 / x exactly 0: those divisions are skipped
        const double n = v[r] == top ? 1.0 : v[r] == 0.0 ? 0.0 : v[r] / top;
        const double summand = n * n - compensation;
        const double preliminary = total + summand;
        compensation = (preliminary - total) - summand;
        total = preliminary;
    }
    return sqrt(total) * top;
}

// mat3.js:71-87 (mat3FromQuat), each entry rounded to float32 as its output
// array does, and the half-axes sigma * scale (cloudVolume.js:196-199).
__device__ void frameOf(const CloudInput& in, uint32_t i, Ellipsoid& e) {
    const double x = in.rot[4 * size_t(i)], y = in.rot[4 * size_t(i) + 1];
    const double z = in.rot[4 * size_t(i) + 2], w = in.rot[4 * size_t(i) + 3];
    e.col[0] = double(float(1.0 - 2.0 * (y * y + z * z)));
    e.col[1] = double(float(2.0 * (x * y + z * w)));
    e.col[2] = double(float(2.0 * (x * z - y * w)));
    e.col[3] = double(float(2.0 * (x * y - z * w)));
    e.col[4] = double(float(1.0 - 2.0 * (x * x + z * z)));
    e.col[5] = double(float(2.0 * (y * z + x * w)));
    e.col[6] = double(float(2.0 * (x * z + y * w)));
    e.col[7] = double(float(2.0 * (y * z - x * w)));
    e.col[8] = double(float(1.0 - 2.0 * (x * x + y * y)));
    for (int a = 0; a < 3; a++) e.radius[a] = in.sigma * double(in.scale[3 * size_t(i) + a]);
}

// cloudVolume.js:201-209: the reach along each world axis.
__device__ Ellipsoid ellipsoidOf(const CloudInput& in, uint32_t i) {
    Ellipsoid e;
    frameOf(in, i, e);
    for (int a = 0; a < 3; a++)
        e.half[a] = hypotV8(e.col[a] * e.radius[0], e.col[3 + a] * e.radius[1], e.col[6 + a] * e.radius[2]);
    return e;
}

// Doubles ordered as unsigned integers: the sign bit flipped on positives,
// every bit on negatives.
__device__ __forceinline__ unsigned long long orderedKey(double v) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

double fromOrderedKey(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

__device__ __forceinline__ unsigned long long warpMin64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ unsigned long long warpMax64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// cloudVolume.js:219-234 (materialBounds): keys[0..2] the smallest
// position - reach per axis, keys[3..5] the largest position + reach; a NaN
// anywhere raises *nan (Math.min and Math.max then give NaN). Each
// Gaussian's reach is stored in `reach` for the stamp.
__global__ void cloudBoundsKernel(CloudInput in, unsigned long long* __restrict__ keys, uint32_t* __restrict__ nan,
                                  double* __restrict__ reach) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
    bool sawNan = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < in.count; i += gridDim.x * blockDim.x) {
        const Ellipsoid e = ellipsoidOf(in, i);
        for (int a = 0; a < 3; a++) {
            reach[3 * size_t(i) + a] = e.half[a];  // kept for the stamp
            const double p = in.pos[3 * size_t(i) + a];
            const double l = p - e.half[a], u = p + e.half[a];
            sawNan |= isnan(l) || isnan(u);
            lo[a] = min(lo[a], orderedKey(l));
            hi[a] = max(hi[a], orderedKey(u));
        }
    }
    for (int a = 0; a < 3; a++) {
        lo[a] = warpMin64(lo[a]);
        hi[a] = warpMax64(hi[a]);
    }
    sawNan = __any_sync(0xffffffffu, sawNan);
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            atomicMin(keys + a, lo[a]);
            atomicMax(keys + 3 + a, hi[a]);
        }
        if (sawNan) atomicOr(nan, 1u);
    }
}

// cloudVolume.js:384-386 (cellOf) and :395-397 (offFace), on finite values.
__device__ __forceinline__ int64_t clampedCell(double v, double origin, double h, int64_t lo, int64_t hi) {
    const double f = floor((v - origin) / h);
    return static_cast<int64_t>(fmin(fmax(f, double(lo)), double(hi)));
}

// One of a cell's nine sample points (its eight corners in corners.js:12-21
// order, then its centre) tested against the ellipsoid in the reference's
// double arithmetic and order (cloudVolume.js:255-273).
__device__ __forceinline__ void sampleOffset(int s, double& ox, double& oy, double& oz) {
    ox = s == 8 ? 0.5 : double(s & 1);
    oy = s == 8 ? 0.5 : double((s >> 1) & 1);
    oz = s == 8 ? 0.5 : double((s >> 2) & 1);
}

__device__ bool sampleInside(const GridView& g, int64_t i, int64_t j, int64_t k, int s, const double c[3],
                             const Ellipsoid& e) {
    double ox, oy, oz;
    sampleOffset(s, ox, oy, oz);
    const double dx = g.origin[0] + (double(i) + ox) * g.h - c[0];
    const double dy = g.origin[1] + (double(j) + oy) * g.h - c[1];
    const double dz = g.origin[2] + (double(k) + oz) * g.h - c[2];
    double sum = 0.0;
    for (int a = 0; a < 3; a++) {
        const double t = (e.col[3 * a] * dx + e.col[3 * a + 1] * dy + e.col[3 * a + 2] * dz) / e.radius[a];
        sum += t * t;
    }
    return sum <= 1.0;
}

struct Box {
    int64_t lo[3], hi[3];
    __device__ int64_t extent(int a) const { return hi[a] - lo[a] + 1; }
    __device__ int64_t cells() const { return extent(0) * extent(1) * extent(2); }
};

// The sample test in float, with a bound on how far its sum of squares can
// be from the double evaluation's; a sample whose float sum is further than
// the bound from 1 is decided by it, every other one is evaluated in double.
// Same answers, far fewer double operations (a double division costs tens
// of float operations on this part). The bound, per Gaussian and box:
//   offset: float(base) + off * float(h), with base = origin + lo h - c (in
//     double) and off = i - lo + ox exact, against the double sequence
//     origin + (i + ox) h - c: within 2^-22 X + A, where X = |base| +
//     (extent + 1) h bounds |base|, off h and the offset, and A = 2^-50
//     (|origin| + |c| + (|lo| + extent + 1) h) the double sequence's own
//     rounding;
//   dot with column a (float entries, exact): the propagated offset errors
//     plus 2^-22 sum_k |col| X_k for its own three roundings;
//   t = dot / r: that over r (held x4 in `err`, a factor of 4 to spare),
//     plus 2^-23 |t| for the float reciprocal and product (taken x4);
//   sum of squares: sum_a (2|t_a| + e_a) e_a, plus 2^-21 s for its roundings,
//     plus a floor of 2^-20 so that 1 +- the bound is never rounded away.
// A Gaussian whose bound is not small (err >= 1e-3), whose half-axes or cell
// are outside [1e-30, 1e30], or whose box is wider than 2^20 cells is tested
// in double throughout.
struct FloatTest {
    float base[3];
    float h;
    float col[9];
    float inv[3];
    float err[3];
};

__device__ bool floatTestOf(const GridView& g, const Box& b, const double c[3], const Ellipsoid& e, FloatTest& f) {
    if (!(g.h > 1e-30 && g.h < 1e30)) return false;
    double X[3], ex[3];
    for (int a = 0; a < 3; a++) {
        if (b.extent(a) > (1 << 20)) return false;
        const double base = (g.origin[a] + double(b.lo[a]) * g.h) - c[a];
        const double span = double(b.extent(a) + 1) * g.h;
        X[a] = fabs(base) + span;
        ex[a] = 0x1p-22 * X[a] + 0x1p-50 * (fabs(g.origin[a]) + fabs(c[a]) + fabs(double(b.lo[a])) * g.h + span);
        f.base[a] = float(base);
    }
    f.h = float(g.h);
    for (int q = 0; q < 9; q++) f.col[q] = float(e.col[q]);
    for (int a = 0; a < 3; a++) {
        const double r = e.radius[a];
        if (!(r > 1e-30 && r < 1e30)) return false;
        // the float reciprocal of float(r): within 2^-23 of 1 / r, inside the
        // 2^-21 |t| allowance
        f.inv[a] = __frcp_rn(float(r));
        double dotErr = 0.0;
        for (int k = 0; k < 3; k++) dotErr += fabs(e.col[3 * a + k]) * (ex[k] + 0x1p-22 * X[k]);
        // above 4 dotErr / r: the reciprocal's error and every rounding of
        // this product are covered by the (1 + 2^-20)
        const double err = 4.0 * dotErr * double(f.inv[a]) * (1.0 + 0x1p-20);
        if (!(err < 1e-3)) return false;
        f.err[a] = float(err);
    }
    return true;
}

// 1 inside, 0 outside, -1 too close to call in float.
__device__ __forceinline__ int floatSample(const FloatTest& f, float ox, float oy, float oz) {
    const float dx = f.base[0] + ox * f.h, dy = f.base[1] + oy * f.h, dz = f.base[2] + oz * f.h;
    float sum = 0.0f, bound = 0.0f;
    for (int a = 0; a < 3; a++) {
        const float t = (f.col[3 * a] * dx + f.col[3 * a + 1] * dy + f.col[3 * a + 2] * dz) * f.inv[a];
        const float at = fabsf(t);
        const float et = f.err[a] + 0x1p-21f * at;
        sum += t * t;
        bound += (2.0f * at + et) * et;
    }
    bound += 0x1p-20f * sum + 0x1p-20f;
    if (sum > 1.0f + bound) return 0;
    if (sum < 1.0f - bound) return 1;
    return -1;
}

// cloudVolume.js:170-173 for one cell of a box: any sample inside. The index
// is the reference's cellIndex of the (possibly out-of-grid, when the
// padding is under two cells) coordinates, and like a typed array the grid
// ignores an index outside it. The double frame is rebuilt only for a sample
// the float test cannot call.
__device__ void stampCell(const CloudInput& in, uint32_t gaussian, const GridView& g, uint8_t* occ, const Box& b,
                          int64_t i, int64_t j, int64_t k, const double c[3], const FloatTest* f) {
    const int64_t cell = i + int64_t(g.dims[0]) * (j + int64_t(g.dims[1]) * k);
    if (cell < 0 || cell >= int64_t(g.cells) || occ[cell] != 0) return;
    Ellipsoid e;
    bool haveFrame = false;
    for (int s = 0; s < 9; s++) {
        double ox, oy, oz;
        sampleOffset(s, ox, oy, oz);
        int inside = -1;
        if (f)
            inside = floatSample(*f, float(i - b.lo[0]) + float(ox), float(j - b.lo[1]) + float(oy),
                                 float(k - b.lo[2]) + float(oz));
        if (inside < 0) {
            if (!haveFrame) {
                frameOf(in, gaussian, e);
                haveFrame = true;
            }
            inside = sampleInside(g, i, j, k, s, c, e) ? 1 : 0;
        }
        if (inside) {
            occ[cell] = 1;
            return;
        }
    }
}

__device__ Box boxOf(const GridView& g, const double c[3], const double* half) {
    Box b;
    for (int a = 0; a < 3; a++) {
        b.lo[a] = clampedCell(c[a] - half[a], g.origin[a], g.h, 1, int64_t(g.dims[a]) - 2);
        b.hi[a] = clampedCell(c[a] + half[a], g.origin[a], g.h, 1, int64_t(g.dims[a]) - 2);
    }
    return b;
}

// The Gaussian's box and its float test (false: test in double).
__device__ bool prepareStamp(const CloudInput& in, uint32_t i, const GridView& g, const double* __restrict__ reach,
                             const double c[3], Box& b, FloatTest& f) {
    const double half[3] = {reach[3 * size_t(i)], reach[3 * size_t(i) + 1], reach[3 * size_t(i) + 2]};
    b = boxOf(g, c, half);
    Ellipsoid e;
    frameOf(in, i, e);
    return floatTestOf(g, b, c, e, f);
}

// cloudVolume.js:147-177 for one Gaussian per thread: the centre's cell
// unconditionally, then the box; a box of more than kInlineBoxCells cells is
// listed for cloudStampBoxKernel.
__global__ void cloudStampKernel(CloudInput in, GridView g, const double* __restrict__ reach,
                                 uint8_t* __restrict__ occ, uint32_t* __restrict__ big,
                                 uint32_t* __restrict__ bigCount) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.count) return;
    const double c[3] = {in.pos[3 * size_t(i)], in.pos[3 * size_t(i) + 1], in.pos[3 * size_t(i) + 2]};
    int64_t at[3];
    for (int a = 0; a < 3; a++) at[a] = clampedCell(c[a], g.origin[a], g.h, 0, int64_t(g.dims[a]) - 1);
    occ[at[0] + int64_t(g.dims[0]) * (at[1] + int64_t(g.dims[1]) * at[2])] = 1;
    Box b;
    FloatTest f;
    const bool fast = prepareStamp(in, i, g, reach, c, b, f);
    if (b.cells() > kInlineBoxCells) {
        big[atomicAdd(bigCount, 1u)] = i;  // at most one slot per Gaussian: `big` holds count
        return;
    }
    for (int64_t k = b.lo[2]; k <= b.hi[2]; k++)
        for (int64_t j = b.lo[1]; j <= b.hi[1]; j++)
            for (int64_t i2 = b.lo[0]; i2 <= b.hi[0]; i2++) stampCell(in, i, g, occ, b, i2, j, k, c, fast ? &f : nullptr);
}

// The listed large boxes, a block each, its threads over the box's cells.
__global__ void cloudStampBoxKernel(CloudInput in, GridView g, const double* __restrict__ reach,
                                    uint8_t* __restrict__ occ, const uint32_t* __restrict__ big,
                                    const uint32_t* __restrict__ bigCount) {
    const uint32_t listed = *bigCount;
    for (uint32_t n = blockIdx.x; n < listed; n += gridDim.x) {
        const uint32_t i = big[n];
        const double c[3] = {in.pos[3 * size_t(i)], in.pos[3 * size_t(i) + 1], in.pos[3 * size_t(i) + 2]};
        Box b;
        FloatTest f;
        const bool fast = prepareStamp(in, i, g, reach, c, b, f);
        const int64_t ex = b.extent(0), exy = ex * b.extent(1), total = b.cells();
        for (int64_t t = threadIdx.x; t < total; t += blockDim.x) {
            const int64_t k = b.lo[2] + t / exy, r = t % exy;
            stampCell(in, i, g, occ, b, b.lo[0] + r % ex, b.lo[1] + r / ex, k, c, fast ? &f : nullptr);
        }
    }
}

struct Dims {
    uint32_t nx, ny, nz, cells;
};

// voxelize.js:402-435 (neighbourhoodPass): a clear cell with a set face
// neighbour becomes set (dilate), a set cell with a clear one becomes clear
// (erode); outside the grid counts as clear.
template <bool DILATE>
__global__ void neighbourhoodKernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, Dims d) {
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < d.cells; idx += gridDim.x * blockDim.x) {
        const uint32_t i = idx % d.nx, j = (idx / d.nx) % d.ny, k = idx / (d.nx * d.ny);
        bool result = src[idx] == 1;
        if (result != DILATE) {
            const uint32_t plane = d.nx * d.ny;
            const uint8_t n[6] = {i + 1 < d.nx ? src[idx + 1] : uint8_t(0), i > 0 ? src[idx - 1] : uint8_t(0),
                                  j + 1 < d.ny ? src[idx + d.nx] : uint8_t(0), j > 0 ? src[idx - d.nx] : uint8_t(0),
                                  k + 1 < d.nz ? src[idx + plane] : uint8_t(0), k > 0 ? src[idx - plane] : uint8_t(0)};
            for (int q = 0; q < 6; q++)
                if (DILATE ? n[q] == 1 : n[q] == 0) result = DILATE;
        }
        dst[idx] = result ? 1 : 0;
    }
}

// cloudVolume.js:302-304: the stamp put back on top.
__global__ void orKernel(uint8_t* __restrict__ occ, const uint8_t* __restrict__ stamp, uint32_t cells) {
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += gridDim.x * blockDim.x)
        occ[idx] |= stamp[idx];
}

// The root of a's tree. Labels only decrease along a path, so the walk ends;
// each step points a at its grandparent (path halving). A plain store is
// enough: the value written is an ancestor, and a link only ever lands on a
// root, which this never writes.
__device__ uint32_t findRoot(uint32_t* L, uint32_t a, uint32_t* err) {
    for (uint32_t step = 0; step < kFindLimit; step++) {
        const uint32_t p = __ldcg(L + a);
        if (p == a) return a;
        const uint32_t gp = __ldcg(L + p);
        if (gp != p) __stcg(L + a, gp);
        a = gp;
        if (step % kPollEvery == kPollEvery - 1 && *reinterpret_cast<volatile uint32_t*>(err)) return a;
    }
    atomicOr(err, 1u);
    return a;
}

// Joins the trees of a and b: the larger root is linked under the smaller
// with atomicMin; if it had been linked meanwhile, continue from its new
// parent. Every retry lowers a label, so it ends.
__device__ void unite(uint32_t* L, uint32_t a, uint32_t b, uint32_t* err) {
    for (uint32_t step = 0; step < kUniteLimit; step++) {
        a = findRoot(L, a, err);
        b = findRoot(L, b, err);
        if (a == b || *reinterpret_cast<volatile uint32_t*>(err)) return;
        if (a > b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicMin(L + b, a);
        if (old == b) return;
        b = old;
    }
    atomicOr(err, 1u);
}

// The labels seeded with x runs: a block takes kCloudBlock consecutive
// cells (a chunk starts at a multiple of kCloudBlock), and an empty cell
// whose -x neighbour is empty, in the same row and the same chunk, takes the
// label of its run's first cell (by ballot within a warp, then the last run
// start of the warps before it); every other cell labels itself. This joins
// the x edges inside a chunk without atomics.
__global__ void labelRunsKernel(const uint8_t* __restrict__ occ, uint32_t* __restrict__ L, Dims d) {
    __shared__ int lastStart[kCloudBlock / 32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = blockIdx.x * kCloudBlock; base < d.cells; base += gridDim.x * kCloudBlock) {
        const uint32_t idx = base + threadIdx.x;
        const bool empty = idx < d.cells && occ[idx] == 0;
        const bool linked = empty && threadIdx.x > 0 && occ[idx - 1] == 0 && idx % d.nx != 0;
        const uint32_t starts = __ballot_sync(0xffffffffu, !linked);
        if (lane == 31) lastStart[warp] = starts ? int(warp * 32 + 31 - __clz(starts)) : -1;
        __syncthreads();
        const uint32_t mine = starts & (0xffffffffu >> (31 - lane));
        int start = mine ? int(warp * 32 + 31 - __clz(mine)) : -1;
        for (int w = int(warp) - 1; start < 0 && w >= 0; w--) start = lastStart[w];
        // thread 0 is never linked, so every thread finds a start
        if (idx < d.cells) L[idx] = base + uint32_t(start);
        __syncthreads();
    }
}

// The remaining face-adjacent pairs of empty cells joined
// (cloudVolume.js:88-89, 359-364): an x edge across a chunk boundary; a y
// (z) edge unless the two cells' -x neighbours are both empty, in which case
// it is implied by edges already joined (cell ~ its -x neighbour ~ that
// one's -y (-z) neighbour ~ the cell's -y (-z) neighbour), so each stretch
// of overlapping runs is joined once, at its first cell.
__global__ void labelMergeKernel(const uint8_t* __restrict__ occ, uint32_t* L, Dims d, uint32_t* err) {
    const uint32_t plane = d.nx * d.ny;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < d.cells; idx += gridDim.x * blockDim.x) {
        if (occ[idx] != 0) continue;
        const uint32_t i = idx % d.nx, j = (idx / d.nx) % d.ny, k = idx / plane;
        const bool left = i > 0 && occ[idx - 1] == 0;
        if (left && idx % kCloudBlock == 0) unite(L, idx, idx - 1, err);
        if (j > 0 && occ[idx - d.nx] == 0 && !(left && occ[idx - 1 - d.nx] == 0)) unite(L, idx, idx - d.nx, err);
        if (k > 0 && occ[idx - plane] == 0 && !(left && occ[idx - 1 - plane] == 0)) unite(L, idx, idx - plane, err);
    }
}

// The roots of the empty cells on the grid's faces marked reached (the
// flood's seeds, cloudVolume.js:344-352). After the merge the trees are
// fixed: the walks here only shorten paths, never change a root.
__global__ void markFaceRootsKernel(const uint8_t* __restrict__ occ, uint32_t* L, uint8_t* __restrict__ reached, Dims d,
                                    uint32_t* err) {
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < d.cells; idx += gridDim.x * blockDim.x) {
        if (occ[idx] != 0) continue;
        const uint32_t i = idx % d.nx, j = (idx / d.nx) % d.ny, k = idx / (d.nx * d.ny);
        if (i == 0 || j == 0 || k == 0 || i == d.nx - 1 || j == d.ny - 1 || k == d.nz - 1)
            reached[findRoot(L, idx, err)] = 1;
    }
}

__device__ __forceinline__ unsigned long long blockSum(unsigned long long v) {
    __shared__ unsigned long long part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long total = 0;
    if (threadIdx.x == 0)
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) total += part[w];
    return total;
}

// cloudVolume.js:367-374: every empty cell whose tree the flood did not
// reach becomes material; *filled counts them. The root is walked to, not
// read from the cell's label: a concurrent path-halving store may leave a
// label at an ancestor short of the root.
__global__ void fillEnclosedKernel(uint8_t* __restrict__ occ, uint32_t* L, const uint8_t* __restrict__ reached,
                                   uint32_t cells, unsigned long long* __restrict__ filled, uint32_t* err) {
    unsigned long long mine = 0;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += gridDim.x * blockDim.x) {
        if (occ[idx] == 0 && !reached[findRoot(L, idx, err)]) {
            occ[idx] = 1;
            mine++;
        }
    }
    const unsigned long long total = blockSum(mine);
    if (threadIdx.x == 0 && total) atomicAdd(filled, total);
}

__global__ void countKernel(const uint8_t* __restrict__ occ, uint32_t cells, unsigned long long* __restrict__ count) {
    unsigned long long mine = 0;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += gridDim.x * blockDim.x)
        mine += occ[idx];
    const unsigned long long total = blockSum(mine);
    if (threadIdx.x == 0 && total) atomicAdd(count, total);
}

// Small device words of one run.
struct CloudScalars {
    unsigned long long keys[6];
    unsigned long long filled;
    unsigned long long occupied;
    uint32_t nan;
    uint32_t err;
    uint32_t bigCount;
    uint32_t pad;
};

// Scratch comes from a stream-ordered memory pool of this library's own, one
// per device, that keeps what a call frees for the next call instead of
// unmapping it: repeated voxelisations do not remap hundreds of megabytes.
// The pool holds the largest scratch any call needed until the process exits.
int scratchPool(int device, cudaMemPool_t* out) {
    static std::mutex lock;
    static cudaMemPool_t pools[64] = {};
    if (device < 0 || device >= 64) return fail(VSIM_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> hold(lock);
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        CK(cudaMemPoolCreate(&pools[device], &props), "memory pool");
        uint64_t keep = ~0ull;
        CK(cudaMemPoolSetAttribute(pools[device], cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
    }
    *out = pools[device];
    return VSIM_OK;
}

// A pool allocation freed, in stream order, when it goes out of scope.
struct DeviceBuffer {
    void* p = nullptr;
    cudaStream_t stream = nullptr;
    ~DeviceBuffer() {
        if (p) cudaFreeAsync(p, stream);
    }
};

#define POOL_ALLOC(buffer, bytes, pool, st, what)                                         \
    do {                                                                                   \
        (buffer).stream = (st);                                                            \
        CK(cudaMallocFromPoolAsync(&(buffer).p, (bytes), (pool), (st)), what);             \
    } while (0)

uint32_t streamGrid(uint64_t items, int sms) {
    const uint64_t want = (items + kCloudBlock - 1) / kCloudBlock;
    return uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(want, uint64_t(sms) * 8)));
}

int voxelizeCloud(vsim_cloud_volume* v, const CloudInput& in, const vsim_cloud_options& o) {
    cudaStream_t st = v->stream;
    int sms = 1;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, v->device), "device attributes");
    cudaMemPool_t pool;
    if (int rc = scratchPool(v->device, &pool)) return rc;

    // 1. bounds
    DeviceBuffer scalarsBuf;
    POOL_ALLOC(scalarsBuf, sizeof(CloudScalars), pool, st, "cloud scratch");
    auto* sc = static_cast<CloudScalars*>(scalarsBuf.p);
    CloudScalars init{};
    for (int a = 0; a < 3; a++) init.keys[a] = ~0ull;
    CK(cudaMemcpyAsync(sc, &init, sizeof init, cudaMemcpyHostToDevice, st), "cloud scratch");
    DeviceBuffer reachBuf;
    POOL_ALLOC(reachBuf, size_t(in.count) * 3 * sizeof(double), pool, st, "cloud scratch");
    auto* reach = static_cast<double*>(reachBuf.p);
    cloudBoundsKernel<<<streamGrid(in.count, sms), kCloudBlock, 0, st>>>(in, sc->keys, &sc->nan, reach);
    CK(cudaGetLastError(), "cloud bounds");
    CloudScalars got{};
    CK(cudaMemcpyAsync(&got, sc, sizeof got, cudaMemcpyDeviceToHost, st), "cloud bounds");
    CK(cudaStreamSynchronize(st), "cloud bounds");

    // cloudVolume.js:113-115, then 2. gridForBounds (voxelize.js:40-67)
    double lo[3], hi[3], extent[3];
    bool nan = got.nan != 0;
    for (int a = 0; a < 3; a++) {
        lo[a] = fromOrderedKey(got.keys[a]);
        hi[a] = fromOrderedKey(got.keys[3 + a]);
        extent[a] = hi[a] - lo[a];
        nan |= std::isnan(extent[a]);
    }
    if (nan || !(std::max(extent[0], std::max(extent[1], extent[2])) > 0))
        return fail(VSIM_ERR_INVALID, "voxelizeCloud: a cloud with no extent has no volume");
    const double h = o.element_size;
    if (!(h > 0 && std::isfinite(h)))
        return fail(VSIM_ERR_RANGE, "gridForBounds: elementSize must be a positive length in metres");
    double cells = 1;
    for (int a = 0; a < 3; a++) {
        const double n = std::max(1.0, std::ceil(extent[a] / h - 1e-6)) + 2.0 * o.padding;
        if (!(n < 4294967296.0)) return fail(VSIM_ERR_RANGE, "voxelizeCloud: the grid is too large");
        v->dims[a] = uint32_t(n);
        v->origin[a] = lo[a] - h * o.padding;
        cells *= n;
    }
    if (!(cells < 4294967296.0)) return fail(VSIM_ERR_RANGE, "voxelizeCloud: the grid has 2^32 cells or more");
    v->h = h;
    v->cells = uint64_t(cells);
    const uint32_t n = uint32_t(v->cells);
    const Dims d{v->dims[0], v->dims[1], v->dims[2], n};
    GridView g{};
    for (int a = 0; a < 3; a++) {
        g.dims[a] = v->dims[a];
        g.origin[a] = v->origin[a];
    }
    g.h = h;
    g.cells = n;

    CK(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&v->occupancy), n, pool, st), "cloud occupancy");
    CK(cudaMemsetAsync(v->occupancy, 0, n, st), "cloud occupancy");

    // 3. stamp
    DeviceBuffer bigBuf;
    POOL_ALLOC(bigBuf, size_t(in.count) * 4, pool, st, "cloud scratch");
    cloudStampKernel<<<(in.count + kCloudBlock - 1) / kCloudBlock, kCloudBlock, 0, st>>>(
        in, g, reach, v->occupancy, static_cast<uint32_t*>(bigBuf.p), &sc->bigCount);
    cloudStampBoxKernel<<<uint32_t(sms) * 4, kCloudBlock, 0, st>>>(
        in, g, reach, v->occupancy, static_cast<const uint32_t*>(bigBuf.p), &sc->bigCount);
    CK(cudaGetLastError(), "cloud stamp");

    // 4. seal and fill
    const uint32_t grid = streamGrid(n, sms);
    if (o.fill) {
        // stamp copy, a ping-pong buffer, labels, reached flags
        DeviceBuffer work;
        POOL_ALLOC(work, size_t(n) * 7 + 64, pool, st, "cloud fill scratch");
        auto* labels = static_cast<uint32_t*>(work.p);
        uint8_t* stamp = reinterpret_cast<uint8_t*>(labels + n);
        uint8_t* other = stamp + n;
        uint8_t* reached = other + n;
        CK(cudaMemcpyAsync(stamp, v->occupancy, n, cudaMemcpyDeviceToDevice, st), "cloud fill");
        uint8_t* cur = v->occupancy;
        for (uint32_t p = 0; p < o.seal; p++) {
            neighbourhoodKernel<true><<<grid, kCloudBlock, 0, st>>>(cur, other, d);
            std::swap(cur, other);
        }
        CK(cudaMemsetAsync(reached, 0, n, st), "cloud fill");
        labelRunsKernel<<<grid, kCloudBlock, 0, st>>>(cur, labels, d);
        labelMergeKernel<<<grid, kCloudBlock, 0, st>>>(cur, labels, d, &sc->err);
        markFaceRootsKernel<<<grid, kCloudBlock, 0, st>>>(cur, labels, reached, d, &sc->err);
        fillEnclosedKernel<<<grid, kCloudBlock, 0, st>>>(cur, labels, reached, n, &sc->filled, &sc->err);
        for (uint32_t p = 0; p < o.seal; p++) {
            neighbourhoodKernel<false><<<grid, kCloudBlock, 0, st>>>(cur, other, d);
            std::swap(cur, other);
        }
        if (cur != v->occupancy)
            CK(cudaMemcpyAsync(v->occupancy, cur, n, cudaMemcpyDeviceToDevice, st), "cloud fill");
        orKernel<<<grid, kCloudBlock, 0, st>>>(v->occupancy, stamp, n);
        CK(cudaGetLastError(), "cloud fill");
        countKernel<<<grid, kCloudBlock, 0, st>>>(v->occupancy, n, &sc->occupied);
        CK(cudaMemcpyAsync(&got, sc, sizeof got, cudaMemcpyDeviceToHost, st), "cloud fill");
        CK(cudaStreamSynchronize(st), "cloud fill");  // before `work` is freed
    } else {
        countKernel<<<grid, kCloudBlock, 0, st>>>(v->occupancy, n, &sc->occupied);
        CK(cudaMemcpyAsync(&got, sc, sizeof got, cudaMemcpyDeviceToHost, st), "cloud stamp");
        CK(cudaStreamSynchronize(st), "cloud stamp");
    }
    if (got.err) return fail(VSIM_ERR_TIMEOUT, "voxelizeCloud: the fill's union-find reached its iteration cap");
    v->filled = got.filled;
    v->occupied = got.occupied;
    return VSIM_OK;
}

int checkOptions(const vsim_cloud_options* o, uint64_t count) {
    if (!o) return fail(VSIM_ERR_INVALID, "options is NULL");
    if (count == 0) return fail(VSIM_ERR_INVALID, "voxelizeCloud: a cloud with no Gaussians has no volume");
    if (count > 0xffffffffull) return fail(VSIM_ERR_RANGE, "voxelizeCloud: at most 2^32 - 1 Gaussians");
    return VSIM_OK;
}

int newVolume(vsim_cloud_volume** out, vsim_cloud_volume** made) {
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    auto* v = new (std::nothrow) vsim_cloud_volume();
    if (!v) return fail(VSIM_ERR_NOMEM, "host allocation failed");
    CK(cudaGetDevice(&v->device), "current device");
    const cudaError_t e = cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete v;
        return cudaFail(e, "stream");
    }
    *made = v;
    return VSIM_OK;
}

void destroyVolume(vsim_cloud_volume* v) {
    if (!v) return;
    if (v->occupancy) cudaFreeAsync(v->occupancy, v->stream);
    if (v->stream) cudaStreamDestroy(v->stream);
    delete v;
}

}  // namespace
}  // namespace vsim

using namespace vsim;

extern "C" {

int vsim_voxelize_cloud_device(const float* d_positions, const float* d_rotations, const float* d_scales,
                               uint64_t count, const vsim_cloud_options* options, void* stream,
                               vsim_cloud_volume** out) {
    clearError();
    if (int rc = checkOptions(options, count)) return rc;
    if (!d_positions || !d_rotations || !d_scales) return fail(VSIM_ERR_INVALID, "NULL cloud array");
    vsim_cloud_volume* v = nullptr;
    if (int rc = newVolume(out, &v)) return rc;
    // the caller's work on the inputs finishes first
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    int rc = e == cudaSuccess ? VSIM_OK : cudaFail(e, "caller stream");
    if (!rc) rc = voxelizeCloud(v, CloudInput{d_positions, d_rotations, d_scales, uint32_t(count), options->sigma},
                                *options);
    if (rc) {
        cudaStreamSynchronize(v->stream);
        destroyVolume(v);
        return rc;
    }
    *out = v;
    return VSIM_OK;
}

namespace {

// Host inputs copied into pool memory on the volume's stream, then the device path.
int voxelizeHostCloud(vsim_cloud_volume* v, const float* positions, const float* rotations, const float* scales,
                      size_t n, const vsim_cloud_options& o) {
    cudaMemPool_t pool;
    if (int rc = scratchPool(v->device, &pool)) return rc;
    DeviceBuffer inputs;
    POOL_ALLOC(inputs, n * 40, pool, v->stream, "cloud inputs");
    auto* dPos = static_cast<float*>(inputs.p);
    float* dRot = dPos + 3 * n;
    float* dScale = dRot + 4 * n;
    CK(cudaMemcpyAsync(dPos, positions, n * 12, cudaMemcpyHostToDevice, v->stream), "cloud inputs");
    CK(cudaMemcpyAsync(dRot, rotations, n * 16, cudaMemcpyHostToDevice, v->stream), "cloud inputs");
    CK(cudaMemcpyAsync(dScale, scales, n * 12, cudaMemcpyHostToDevice, v->stream), "cloud inputs");
    return voxelizeCloud(v, CloudInput{dPos, dRot, dScale, uint32_t(n), o.sigma}, o);
}

}  // namespace

int vsim_voxelize_cloud(const float* positions, const float* rotations, const float* scales, uint64_t count,
                        const vsim_cloud_options* options, vsim_cloud_volume** out) {
    clearError();
    if (int rc = checkOptions(options, count)) return rc;
    if (!positions || !rotations || !scales) return fail(VSIM_ERR_INVALID, "NULL cloud array");
    vsim_cloud_volume* v = nullptr;
    if (int rc = newVolume(out, &v)) return rc;
    const int rc = voxelizeHostCloud(v, positions, rotations, scales, size_t(count), *options);
    if (rc) {
        cudaStreamSynchronize(v->stream);
        destroyVolume(v);
        return rc;
    }
    *out = v;
    return VSIM_OK;
}

int vsim_cloud_volume_grid(const vsim_cloud_volume* volume, vsim_cloud_grid* out) {
    clearError();
    if (!volume || !out) return fail(VSIM_ERR_INVALID, "NULL argument");
    for (int a = 0; a < 3; a++) {
        out->dims[a] = volume->dims[a];
        out->origin[a] = volume->origin[a];
    }
    out->h = volume->h;
    out->occupied = volume->occupied;
    out->filled = volume->filled;
    return VSIM_OK;
}

int vsim_cloud_volume_read(vsim_cloud_volume* volume, uint8_t* occupancy, size_t cells) {
    clearError();
    if (!volume || !occupancy) return fail(VSIM_ERR_INVALID, "NULL argument");
    if (cells < volume->cells) return fail(VSIM_ERR_CAPACITY, "occupancy buffer smaller than the grid");
    DeviceGuard guard(volume->device);
    CK(cudaMemcpyAsync(occupancy, volume->occupancy, volume->cells, cudaMemcpyDeviceToHost, volume->stream),
       "read occupancy");
    CK(cudaStreamSynchronize(volume->stream), "read occupancy");
    return VSIM_OK;
}

int vsim_cloud_volume_destroy(vsim_cloud_volume* volume) {
    clearError();
    if (!volume) return VSIM_OK;
    DeviceGuard guard(volume->device);
    destroyVolume(volume);
    return VSIM_OK;
}

}  // extern "C"
