// A Gaussian cloud to an occupancy grid on the device: voxelizeCloud
// (packages/visionary-sim/src/sim/discretize/lattice/cloudVolume.js:101-397),
// the reference's "cloud" rest geometry (voxelLattice.js:208-226).
//
// The reference runs it on the CPU in JavaScript doubles. Here every step is
// a kernel whose every decision equals the one the same double arithmetic
// and order would take, so the grid is the same cell for cell. Double
// arithmetic is slow on this part, so decisions are taken in float wherever
// a proven error bound shows float gives the same answer, and in double
// only where it cannot:
//   1. bounds: each Gaussian's ellipsoid reach (materialBounds, :219-234),
//      estimated in float with a relative bound; the extremes reduced with
//      order-preserving 64-bit keys, then evaluated exactly for the few
//      Gaussians whose bracket can hold an extreme;
//   2. the grid laid out on the host from the bounds (gridForBounds,
//      voxelize.js:40-67);
//   3. stamp: a thread per Gaussian marks its centre cell and tests the
//      cells of its box against the ellipsoid (stampCloud, :138-178), box
//      edges and samples decided in float unless too close to call; a box
//      of more than kInlineBoxCells cells is handed to a block instead;
//   4. seal and fill (:291-306) on the cells packed 32 to a word along x:
//      6-neighbourhood dilations, the fill, as many erosions, the stamp put
//      back, the words written out as bytes once. The reference fills by
//      flooding the empty cells from the grid's faces (fillEnclosed,
//      :321-375); here the flood's set is reached by rounds of sweeps over
//      the words (an occluded fill along x, warp scans along y and z) to a
//      round that adds nothing, or, past a cap of rounds, found as the
//      face-connected components of empty cells that touch a face by a
//      concurrent union-find (x runs seeded by warp ballots, links by
//      atomicMin on roots, path halving by plain stores).
// Marking is an OR (a cell is set by any Gaussian that reaches it), and the
// components of a graph do not depend on the order edges are merged, so no
// step's result depends on thread timing.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>

#include <math_constants.h>

#include "float_bounds.cuh"
#include "frame_rows.cuh"
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

using bounds::Box;
using bounds::Ellipsoid;
using bounds::floatCell;
using bounds::floatSample;
using bounds::floatTestOf;
using bounds::FloatTest;
using bounds::GridView;
using bounds::sampleInside;
using bounds::hypotV8;
using bounds::kReachSlack;
using bounds::reachEstimate;

constexpr uint32_t kCloudBlock = 256;
constexpr uint32_t kInlineBoxCells = 64;    // larger boxes are stamped by a block each
// Caps of the union-find loops. Labels strictly fall along every walk, so
// the loops end by themselves; the caps, and the shared flag the first
// thread to reach one raises (every walk polls it), only bound the kernels'
// time on an input no test has seen.
constexpr uint32_t kFindLimit = 1u << 22;
constexpr uint32_t kUniteLimit = 1u << 16;
constexpr uint32_t kPollEvery = 1024;
// Rounds of flood sweeps before the union-find takes over (a round that
// adds nothing ends the flood; each turn of a path the sweeps' axes cannot
// follow in one round costs a round).
constexpr uint32_t kFloodRounds = 24;
std::atomic<uint32_t> floodRounds{kFloodRounds};

struct CloudInput {
    const float* pos;    // xyz per Gaussian
    const float* rot;    // quaternion x, y, z, w
    const float* scale;  // standard deviations per axis, metres
    uint32_t count;
    double sigma;
    float sigmaF;        // float(sigma)
};




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

// The float side of the bounds and the stamp. For each Gaussian the bounds
// pass keeps, per world axis a, frames[3 i + a] = (row a of its frame as the
// float32 values frameOf rounds to, a float estimate of its reach along a);
// the estimate is NaN where it cannot be trusted, and only then is V8's
// hypot evaluated in double (FP64 runs at a small fraction of the float rate
// on this part: a double division costs about a hundred float operations).
//

// The radii float(sigma) * scale for the estimate (within 2^-23 of the
// double sigma * scale of cloudVolume.js:196-199), NaN where out of its
// range.
__device__ void radiiOf(const CloudInput& in, uint32_t i, float rf[3]) {
    for (int a = 0; a < 3; a++) rf[a] = bounds::radiusEstimate(in.sigmaF, in.scale[3 * size_t(i) + a]);
}

// Floats ordered as unsigned integers (as orderedKey for doubles).
__device__ __forceinline__ uint32_t orderedKey32(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u >> 31) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float fromOrderedKey32(uint32_t k) {
    return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}

// cloudVolume.js:219-234 (materialBounds), first pass: per axis the smallest
// float upper bound on position - reach (keys[0..2]) and the largest float
// lower bound on position + reach (keys[3..5]) over all Gaussians, from the
// reach estimates with directed roundings (the exact value rounded outwards
// where a Gaussian has no estimate). A NaN anywhere raises *nan (Math.min
// and Math.max then give NaN). Fills `frames`.
__global__ void cloudBoundsKernel(CloudInput in, uint32_t* __restrict__ keys, uint32_t* __restrict__ nan,
                                  float4* __restrict__ frames) {
    uint32_t lo[3] = {~0u, ~0u, ~0u}, hi[3] = {0, 0, 0};
    bool sawNan = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < in.count; i += gridDim.x * blockDim.x) {
        // The frame in float where every entry is certified to equal the
        // double path's float32 rounding (frame_rows.cuh), else in double.
        float col[9], rf[3];
        const float* q4 = in.rot + 4 * size_t(i);
        if (!frame::rowsInFloat(q4[0], q4[1], q4[2], q4[3], col)) {
            Ellipsoid full;
            frameOf(in, i, full);
            for (int q = 0; q < 9; q++) col[q] = float(full.col[q]);
        }
        // the double frame, when an exact reach is wanted: the float32
        // entries widened, exactly frameOf's
        Ellipsoid e;
        for (int q = 0; q < 9; q++) e.col[q] = col[q];
        for (int a = 0; a < 3; a++) e.radius[a] = in.sigma * double(in.scale[3 * size_t(i) + a]);
        radiiOf(in, i, rf);
        for (int a = 0; a < 3; a++) {
            const float p = in.pos[3 * size_t(i) + a];
            float hf = reachEstimate(col, rf, a);
            if (!isfinite(p)) hf = CUDART_NAN_F;
            frames[3 * size_t(i) + a] = make_float4(col[3 * a], col[3 * a + 1], col[3 * a + 2], hf);
            float l, u;
            if (isnan(hf)) {
                const double half = hypotV8(e.col[a] * e.radius[0], e.col[3 + a] * e.radius[1], e.col[6 + a] * e.radius[2]);
                const double ld = double(p) - half, ud = double(p) + half;
                sawNan |= isnan(ld) || isnan(ud);
                l = __double2float_ru(ld);
                u = __double2float_rd(ud);
            } else {
                const float narrow = __fmul_rd(hf, float(1.0 - kReachSlack));  // <= reach
                l = __fsub_ru(p, narrow);                                     // >= position - reach
                u = __fadd_rd(p, narrow);                                     // <= position + reach
            }
            lo[a] = min(lo[a], orderedKey32(l));
            hi[a] = max(hi[a], orderedKey32(u));
        }
    }
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
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

// The exact reach along axis a (cloudVolume.js:201-209).
__device__ double exactReach(const CloudInput& in, uint32_t i, int a) {
    Ellipsoid e;
    frameOf(in, i, e);
    return hypotV8(e.col[a] * e.radius[0], e.col[3 + a] * e.radius[1], e.col[6 + a] * e.radius[2]);
}

// Second pass: the exact extremes. Only a Gaussian whose position - reach can
// lie at or below the first pass's smallest upper bound can hold the minimum
// (every other one's exceeds it), and likewise for the maximum; those few get
// the exact reach and their exact bound into exact[0..5]. The test is in
// float, rounded outwards: position - reach >= RD(position - RU(hf (1 +
// slack))).
__global__ void cloudExtremesKernel(CloudInput in, const uint32_t* __restrict__ keys,
                                    const float4* __restrict__ frames, unsigned long long* __restrict__ exact) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
    float bound[6];
    for (int q = 0; q < 6; q++) bound[q] = fromOrderedKey32(keys[q]);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < in.count; i += gridDim.x * blockDim.x) {
        for (int a = 0; a < 3; a++) {
            const float p = in.pos[3 * size_t(i) + a];
            const float hf = frames[3 * size_t(i) + a].w;
            bool low = true, high = true;
            if (!isnan(hf)) {
                const float wide = __fmul_ru(hf, float(1.0 + kReachSlack));  // >= reach
                low = __fsub_rd(p, wide) <= bound[a];
                high = __fadd_ru(p, wide) >= bound[3 + a];
            }
            if (!(low || high)) continue;
            const double half = exactReach(in, i, a);
            if (low) lo[a] = min(lo[a], orderedKey(double(p) - half));
            if (high) hi[a] = max(hi[a], orderedKey(double(p) + half));
        }
    }
    for (int a = 0; a < 3; a++) {
        lo[a] = warpMin64(lo[a]);
        hi[a] = warpMax64(hi[a]);
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            if (lo[a] != ~0ull) atomicMin(exact + a, lo[a]);
            if (hi[a] != 0) atomicMax(exact + 3 + a, hi[a]);
        }
    }
}

// cloudVolume.js:384-386 (cellOf) and :395-397 (offFace), on finite values.
__device__ __forceinline__ int64_t clampedCell(double v, double origin, double h, int64_t lo, int64_t hi) {
    const double f = floor((v - origin) / h);
    return static_cast<int64_t>(fmin(fmax(f, double(lo)), double(hi)));
}

// The float test of Gaussian i's box (bounds::floatTestInFloat), from the
// cloud's scales.
__device__ bool floatTestInFloat(const CloudInput& in, uint32_t i, const GridView& g, const Box& b, const double c[3],
                                 const float cf[3], const float col[9], FloatTest& f) {
    const float scale[3] = {in.scale[3 * size_t(i)], in.scale[3 * size_t(i) + 1], in.scale[3 * size_t(i) + 2]};
    return bounds::floatTestInFloat(g, b, c, cf, col, in.sigma, in.sigmaF, scale, f);
}

// cloudVolume.js:170-173 for one cell of a box: any sample inside. The index
// is the reference's cellIndex of the (possibly out-of-grid, when the
// padding is under two cells) coordinates, and like a typed array the grid
// ignores an index outside it. The double frame is rebuilt only for a sample
// the float test cannot call.
//
// The float path converts nothing from double or 64-bit integers: on this
// part such conversions run on the FP64 pipe, and nine samples a cell made
// them the stamp's bottleneck. The cell's place in its box (under 2^20, so
// exact) is an int32 turned float once; the sample offsets are float
// constants.
__device__ void stampCell(const CloudInput& in, uint32_t gaussian, const GridView& g, uint8_t* occ, const int64_t lo[3],
                          int64_t i, int64_t j, int64_t k, const double c[3], const FloatTest* f) {
    const int64_t cell = i + int64_t(g.dims[0]) * (j + int64_t(g.dims[1]) * k);
    if (cell < 0 || cell >= int64_t(g.cells) || occ[cell] != 0) return;
    Ellipsoid e;
    bool haveFrame = false;
    const float fi = float(int32_t(i - lo[0])), fj = float(int32_t(j - lo[1])), fk = float(int32_t(k - lo[2]));
#pragma unroll
    for (int s = 0; s < 9; s++) {
        const float ox = s == 8 ? 0.5f : float(s & 1), oy = s == 8 ? 0.5f : float((s >> 1) & 1);
        const float oz = s == 8 ? 0.5f : float((s >> 2) & 1);
        int inside = -1;
        if (f) inside = floatSample(*f, fi + ox, fj + oy, fk + oz);
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


// Whether the float cells hold for a position on axis a (ranges that keep
// every term above a normal float's floor and below overflow).
__device__ __forceinline__ bool floatCellsHold(const GridView& g, float c, float reach) {
    return g.floatBound && g.invH > 0.0f && fabsf(c) <= 0x1p40f && reach <= 0x1p40f;
}

__device__ __forceinline__ int64_t clampCell(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : v > hi ? hi : v; }

// cloudVolume.js:384-386 for the centre: in float, else exact.
__device__ int64_t centreCell(const GridView& g, double c, int a) {
    const float cf = float(c);  // exact: c is a float position
    int64_t cell;
    if (floatCellsHold(g, cf, 0.0f)) {
        const float co = cf - g.originF[a];
        const float delta = bounds::cellDelta(g.originMag[a], cf, co, 0.0f, g.invH);
        if (floatCell(co, 0.0f, 0.0f, g.invH, delta, cell)) return clampCell(cell, 0, int64_t(g.dims[a]) - 1);
    }
    return clampedCell(c, g.origin[a], g.h, 0, int64_t(g.dims[a]) - 1);
}

// cloudVolume.js:147-160: the cells from position - reach to position +
// reach, within one cell of the faces. With a reach estimate hf the exact
// reach lies in [hf (1 - kReachSlack), hf (1 + kReachSlack)], also after
// those bounds are rounded to float (slack 2^-18 against the estimate's
// 2^-21), so each edge is the float cell of that interval; only an edge
// within delta of a cell boundary (or a Gaussian without an estimate)
// takes the exact reach and the double division.
__device__ Box boxOf(const CloudInput& in, uint32_t i, const GridView& g, const double c[3], const float hf[3]) {
    Box b;
    for (int a = 0; a < 3; a++) {
        const int64_t lo = 1, hi = int64_t(g.dims[a]) - 2;
        const float cf = float(c[a]);  // exact: c is a float position
        if (!isnan(hf[a]) && floatCellsHold(g, cf, hf[a])) {
            const float narrow = hf[a] * float(1.0 - kReachSlack), wide = hf[a] * float(1.0 + kReachSlack);
            const float co = cf - g.originF[a];
            const float delta = bounds::cellDelta(g.originMag[a], cf, co, wide, g.invH);
            int64_t l, u;
            if (floatCell(co, -wide, -narrow, g.invH, delta, l) && floatCell(co, narrow, wide, g.invH, delta, u)) {
                b.lo[a] = clampCell(l, lo, hi);
                b.hi[a] = clampCell(u, lo, hi);
                continue;
            }
        }
        const double half = exactReach(in, i, a);
        b.lo[a] = clampedCell(c[a] - half, g.origin[a], g.h, lo, hi);
        b.hi[a] = clampedCell(c[a] + half, g.origin[a], g.h, lo, hi);
    }
    return b;
}

// The Gaussian's box and its float test (false: test in double), from the
// frame rows and reach estimates the bounds pass kept; the frame's double
// values are the float rows widened, exactly frameOf's.
__device__ bool prepareStamp(const CloudInput& in, uint32_t i, const GridView& g, const float4* __restrict__ frames,
                             const double c[3], Box& b, FloatTest& f) {
    float col[9], hf[3], cf[3];
    for (int a = 0; a < 3; a++) {
        const float4 row = frames[3 * size_t(i) + a];
        col[3 * a] = row.x;
        col[3 * a + 1] = row.y;
        col[3 * a + 2] = row.z;
        hf[a] = row.w;
        cf[a] = in.pos[3 * size_t(i) + a];
    }
    b = boxOf(in, i, g, c, hf);
    return floatTestInFloat(in, i, g, b, c, cf, col, f);
}

// One Gaussian's stamp as the walk below needs it, in shared memory.
struct StampEntry {
    FloatTest f;
    int64_t lo[3];
    uint32_t ex, exy;  // the box's extent along x, and x times y
    uint32_t gaussian;
    uint32_t fast;
};

constexpr uint32_t kStampBlock = 128;

// cloudVolume.js:147-177. Each thread sets up one Gaussian: its centre's cell
// unconditionally, its box and float test; a box of more than
// kInlineBoxCells cells is listed for cloudStampBoxKernel. Then each warp
// walks its 32 Gaussians' boxes as one list of cells dealt to its lanes 32
// at a time (a lane finds the Gaussian owning its cell by a binary search
// over the warp's running offsets), so lanes are not idle while one
// Gaussian's box is longer than its neighbours'. Marking is an OR: which
// lane tests a cell, and when, changes nothing.
__global__ void __launch_bounds__(kStampBlock) cloudStampKernel(CloudInput in, GridView g,
                                                                const float4* __restrict__ frames,
                                                                uint8_t* __restrict__ occ, uint32_t* __restrict__ big,
                                                                uint32_t* __restrict__ bigCount) {
    constexpr unsigned kAll = 0xffffffffu;
    __shared__ StampEntry entries[kStampBlock];
    const uint32_t lane = threadIdx.x & 31;
    const StampEntry* warpEntries = entries + (threadIdx.x & ~31u);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = 0;
    if (i < in.count) {
        const double c[3] = {in.pos[3 * size_t(i)], in.pos[3 * size_t(i) + 1], in.pos[3 * size_t(i) + 2]};
        int64_t at[3];
        for (int a = 0; a < 3; a++) at[a] = centreCell(g, c[a], a);
        occ[at[0] + int64_t(g.dims[0]) * (at[1] + int64_t(g.dims[1]) * at[2])] = 1;
        Box b;
        StampEntry& mine = entries[threadIdx.x];
        const bool fast = prepareStamp(in, i, g, frames, c, b, mine.f);
        if (b.cells() > kInlineBoxCells) {
            big[atomicAdd(bigCount, 1u)] = i;  // at most one slot per Gaussian: `big` holds count
        } else {
            n = uint32_t(b.cells());
            for (int a = 0; a < 3; a++) mine.lo[a] = b.lo[a];
            mine.ex = uint32_t(b.extent(0));
            mine.exy = mine.ex * uint32_t(b.extent(1));
            mine.gaussian = i;
            mine.fast = fast ? 1u : 0u;
        }
    }
    // The warp's running offsets: lane l's cells are [off, off + n).
    uint32_t incl = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(kAll, incl, d);
        if (lane >= uint32_t(d)) incl += v;
    }
    const uint32_t off = incl - n;
    const uint32_t total = __shfl_sync(kAll, incl, 31);
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t t = base + lane;
        // the last lane whose offset is at or below t (offsets never fall)
        uint32_t owner = 0;
#pragma unroll
        for (uint32_t step = 16; step >= 1; step >>= 1) {
            const uint32_t probe = __shfl_sync(kAll, off, owner + step);
            if (probe <= t) owner += step;
        }
        const uint32_t first = __shfl_sync(kAll, off, owner);
        if (t >= total) continue;
        const StampEntry& e = warpEntries[owner];
        const uint32_t r = t - first, ex = e.ex, exy = e.exy;
        const uint32_t k = r / exy, rem = r - k * exy, j = rem / ex, i2 = rem - j * ex;
        const uint32_t gi = e.gaussian;
        const double c[3] = {in.pos[3 * size_t(gi)], in.pos[3 * size_t(gi) + 1], in.pos[3 * size_t(gi) + 2]};
        const int64_t lo[3] = {e.lo[0], e.lo[1], e.lo[2]};
        stampCell(in, gi, g, occ, lo, lo[0] + i2, lo[1] + j, lo[2] + k, c, e.fast ? &e.f : nullptr);
    }
}

// The listed large boxes, a block each, its threads over the box's cells.
__global__ void cloudStampBoxKernel(CloudInput in, GridView g, const float4* __restrict__ frames,
                                    uint8_t* __restrict__ occ, const uint32_t* __restrict__ big,
                                    const uint32_t* __restrict__ bigCount) {
    const uint32_t listed = *bigCount;
    for (uint32_t n = blockIdx.x; n < listed; n += gridDim.x) {
        const uint32_t i = big[n];
        const double c[3] = {in.pos[3 * size_t(i)], in.pos[3 * size_t(i) + 1], in.pos[3 * size_t(i) + 2]};
        Box b;
        FloatTest f;
        const bool fast = prepareStamp(in, i, g, frames, c, b, f);
        const int64_t ex = b.extent(0), exy = ex * b.extent(1), total = b.cells();
        for (int64_t t = threadIdx.x; t < total; t += blockDim.x) {
            const int64_t k = b.lo[2] + t / exy, r = t % exy;
            stampCell(in, i, g, occ, b.lo, b.lo[0] + r % ex, b.lo[1] + r / ex, k, c, fast ? &f : nullptr);
        }
    }
}

struct Dims {
    uint32_t nx, ny, nz, cells;
};


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
// ---------------------------------------------------------------- flood --
// The same set fillEnclosed's flood reaches (cloudVolume.js:321-375): the
// empty cells joined to an empty face cell by a path of face-adjacent empty
// cells. The grid's empty cells are packed 32 to a word along x (rows of
// nw words; bits past nx are clear, so never entered), the face cells seed
// `reached`, and sweeps spread it: along x within each row (an occluded
// fill, words carried into their neighbours, up then down), along y and z
// 32 columns at a time (a word takes its neighbour's reached bits where it
// is empty, then fills along x within itself). Every step only adds empty
// cells adjacent to reached ones, and a round of the three sweeps that adds
// nothing leaves a set closed under adjacency: the flood's set exactly. The
// rounds are capped; past the cap the union-find below decides instead.

struct Words {
    uint32_t nw;    // words per row
    uint32_t rows;  // ny * nz
    uint32_t ny, nz;
};

// Seeds g spread through the set bits of p towards higher (Up) or lower
// (Down) bit positions: Kogge-Stone occluded fill.
__device__ __forceinline__ uint32_t fillUp(uint32_t g, uint32_t p) {
    g |= p & (g << 1);
    p &= p << 1;
    g |= p & (g << 2);
    p &= p << 2;
    g |= p & (g << 4);
    p &= p << 4;
    g |= p & (g << 8);
    p &= p << 8;
    return g | (p & (g << 16));
}

__device__ __forceinline__ uint32_t fillDown(uint32_t g, uint32_t p) {
    g |= p & (g >> 1);
    p &= p >> 1;
    g |= p & (g >> 2);
    p &= p >> 2;
    g |= p & (g >> 4);
    p &= p >> 4;
    g |= p & (g >> 8);
    p &= p >> 8;
    return g | (p & (g >> 16));
}

// The valid bits of word `word` of a row (cells past nx are clear).
__device__ __forceinline__ uint32_t validBits(const Dims& d, uint32_t word) {
    const uint32_t count = min(32u, d.nx - word * 32);
    return count == 32 ? 0xffffffffu : (1u << count) - 1u;
}

// A thread per word: bit b of word w of a row set where cell 32 w + b is.
__global__ void packCellsKernel(const uint8_t* __restrict__ occ, Dims d, Words w, uint32_t* __restrict__ bits) {
    const uint32_t total = w.rows * w.nw;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t row = t / w.nw, word = t - row * w.nw;
        const uint32_t first = word * 32, count = min(32u, d.nx - first);
        const uint8_t* cells = occ + size_t(row) * d.nx + first;
        uint32_t m = 0;
        for (uint32_t b = 0; b < count; b++) m |= uint32_t(cells[b] != 0) << b;
        bits[t] = m;
    }
}

// voxelize.js:402-435 (neighbourhoodPass) on packed words, a thread per
// word: a clear cell with a set face neighbour becomes set (dilate), a set
// cell with a clear one becomes clear (erode); outside the grid counts as
// clear. The x neighbours are the word shifted by one, the edge bits taken
// from the neighbouring words of the row.
template <bool DILATE>
__global__ void neighbourhoodWordsKernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, Dims d, Words w) {
    const uint32_t total = w.rows * w.nw, plane = w.nw * d.ny;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t row = t / w.nw, word = t - row * w.nw;
        const uint32_t j = row % d.ny, k = row / d.ny;
        const uint32_t c = src[t];
        const uint32_t left = word > 0 ? src[t - 1] : 0u, right = word + 1 < w.nw ? src[t + 1] : 0u;
        const uint32_t n[6] = {(c << 1) | (left >> 31), (c >> 1) | (right << 31), j > 0 ? src[t - w.nw] : 0u,
                               j + 1 < d.ny ? src[t + w.nw] : 0u, k > 0 ? src[t - plane] : 0u,
                               k + 1 < d.nz ? src[t + plane] : 0u};
        uint32_t out = c;
        for (int q = 0; q < 6; q++) out = DILATE ? (out | n[q]) : (out & n[q]);
        dst[t] = out & validBits(d, word);
    }
}

// A thread per word: the empty cells of the sealed grid, and as reached
// those on a face of the grid (the flood's seeds, cloudVolume.js:344-352).
__global__ void seedFloodKernel(const uint32_t* __restrict__ cur, Dims d, Words w, uint32_t* __restrict__ empty,
                                uint32_t* __restrict__ reached) {
    const uint32_t total = w.rows * w.nw;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t row = t / w.nw, word = t - row * w.nw;
        const uint32_t j = row % d.ny, k = row / d.ny;
        const uint32_t e = ~cur[t] & validBits(d, word);
        uint32_t face = (j == 0 || k == 0 || j == d.ny - 1 || k == d.nz - 1) ? 0xffffffffu : 0u;
        if (word == 0) face |= 1u;
        if (word == w.nw - 1) face |= 1u << ((d.nx - 1) % 32);
        empty[t] = e;
        reached[t] = e & face;
    }
}

// Along x: a thread per row, up then down, the edge bit carried between
// neighbouring words.
__global__ void sweepXKernel(Words w, const uint32_t* __restrict__ empty, uint32_t* __restrict__ reached,
                             uint32_t* __restrict__ changed) {
    bool grew = false;
    for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < w.rows; row += gridDim.x * blockDim.x) {
        uint32_t* r = reached + size_t(row) * w.nw;
        const uint32_t* e = empty + size_t(row) * w.nw;
        uint32_t carry = 0;
        for (uint32_t q = 0; q < w.nw; q++) {
            const uint32_t was = r[q], p = e[q];
            const uint32_t g = fillUp(was | (carry & p & 1u), p);
            carry = g >> 31;
            if (g != was) {
                r[q] = g;
                grew = true;
            }
        }
        carry = 0;
        for (uint32_t q = w.nw; q-- > 0;) {
            const uint32_t was = r[q], p = e[q];
            const uint32_t g = fillDown(was | ((carry << 31) & p), p);
            carry = g & 1u;
            if (g != was) {
                r[q] = g;
                grew = true;
            }
        }
    }
    if (__any_sync(0xffffffffu, grew) && (threadIdx.x & 31) == 0) atomicOr(changed, 1u);
}

// Along y (a line per word column of an xz plane: stride nw, lines nz) or
// z (a line per word column of an xy row: stride nw ny, lines ny), a warp per
// line. Along a line a word takes its predecessor's reached bits where it
// is empty, x -> r | (e & x): maps of that form compose associatively,
// (a2, b2) after (a1, b1) = (a2 | (b2 & a1), b2 & b1), so each lane folds its
// segment of the line into one map, a warp scan gives every lane the
// reached bits entering its segment, and a second walk applies them, each
// word also filled along x within itself. Up the line, then down.
__device__ void sweepLineWay(bool up, uint32_t lane, uint32_t length, uint32_t seg, size_t base, uint32_t stride,
                             const uint32_t* __restrict__ empty, uint32_t* __restrict__ reached, bool& grew) {
    constexpr unsigned kAll = 0xffffffffu;
    // lane l holds steps [l seg, (l + 1) seg), walked upwards or downwards;
    // the lanes come in lane order up, in reverse lane order down
    const uint32_t s0 = min(lane * seg, length), s1 = min(s0 + seg, length);
    auto at = [&](uint32_t s) { return base + size_t(s) * stride; };
    uint32_t a = 0, b = ~0u;
    if (up) {
        for (uint32_t s = s0; s < s1; s++) {
            const uint32_t e = empty[at(s)];
            a = reached[at(s)] | (e & a);
            b &= e;
        }
    } else {
        for (uint32_t s = s1; s-- > s0;) {
            const uint32_t e = empty[at(s)];
            a = reached[at(s)] | (e & a);
            b &= e;
        }
    }
    // inclusive scan in walk order (lane order up, reverse lane order down)
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t pa = up ? __shfl_up_sync(kAll, a, d) : __shfl_down_sync(kAll, a, d);
        const uint32_t pb = up ? __shfl_up_sync(kAll, b, d) : __shfl_down_sync(kAll, b, d);
        if (up ? lane >= d : lane + d < 32) {
            a |= b & pa;
            b &= pb;
        }
    }
    const uint32_t before = up ? __shfl_up_sync(kAll, a, 1) : __shfl_down_sync(kAll, a, 1);
    uint32_t carry = (up ? lane > 0 : lane < 31) ? before : 0u;
    auto apply = [&](uint32_t s) {
        const uint32_t was = reached[at(s)], e = empty[at(s)];
        const uint32_t g = fillDown(fillUp(was | (e & carry), e), e);
        carry = g;
        if (g != was) {
            reached[at(s)] = g;
            grew = true;
        }
    };
    if (up) {
        for (uint32_t s = s0; s < s1; s++) apply(s);
    } else {
        for (uint32_t s = s1; s-- > s0;) apply(s);
    }
}

__global__ void sweepLineKernel(Words w, uint32_t lines, uint32_t length, uint32_t stride, uint32_t lineStride,
                                const uint32_t* __restrict__ empty, uint32_t* __restrict__ reached,
                                uint32_t* __restrict__ changed) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t seg = (length + 31) / 32;
    bool grew = false;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < lines * w.nw; t += warps) {
        const uint32_t line = t / w.nw, word = t - line * w.nw;
        const size_t base = size_t(line) * lineStride + word;
        sweepLineWay(true, lane, length, seg, base, stride, empty, reached, grew);
        __syncwarp();
        sweepLineWay(false, lane, length, seg, base, stride, empty, reached, grew);
        __syncwarp();
    }
    if (__any_sync(0xffffffffu, grew) && lane == 0) atomicOr(changed, 1u);
}

// cloudVolume.js:367-374 on the words: every empty cell not reached becomes
// material; *filled counts them. A thread per word.
__global__ void encloseWordsKernel(uint32_t* __restrict__ cur, Words w, const uint32_t* __restrict__ empty,
                                   const uint32_t* __restrict__ reached, unsigned long long* __restrict__ filled) {
    unsigned long long mine = 0;
    const uint32_t total = w.rows * w.nw;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t enclosed = empty[t] & ~reached[t];
        if (!enclosed) continue;
        mine += __popc(enclosed);
        cur[t] |= enclosed;
    }
    const unsigned long long sum = blockSum(mine);
    if (threadIdx.x == 0 && sum) atomicAdd(filled, sum);
}

// The cells of a | b as bytes (0 or 1) into occ, a thread per 16 cells of
// the byte grid (one 16-byte store where occ is 16-byte aligned, bytes
// otherwise); *occupied counts them when given.
__global__ void unpackCellsKernel(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, Dims d, Words w,
                                  uint8_t* __restrict__ occ, unsigned long long* __restrict__ occupied) {
    unsigned long long mine = 0;
    const uint32_t chunks = (d.cells + 15) / 16;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < chunks; q += gridDim.x * blockDim.x) {
        const uint32_t first = q * 16, count = min(16u, d.cells - first);
        uint32_t row = first / d.nx, i = first - row * d.nx;
        uint32_t at = ~0u, m = 0;
        uint32_t packed[4] = {0, 0, 0, 0};
#pragma unroll
        for (uint32_t c = 0; c < 16; c++) {
            if (c < count) {
                const uint32_t word = row * w.nw + (i >> 5);
                if (word != at) {
                    at = word;
                    m = a[word] | (b ? b[word] : 0u);
                }
                const uint32_t bit = (m >> (i & 31)) & 1u;
                packed[c >> 2] |= bit << (8 * (c & 3));
                mine += bit;
                if (++i == d.nx) {
                    i = 0;
                    row++;
                }
            }
        }
        if (count == 16 && (reinterpret_cast<uintptr_t>(occ) & 15u) == 0) {
            *reinterpret_cast<uint4*>(occ + first) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        } else {
            for (uint32_t c = 0; c < count; c++) occ[first + c] = uint8_t((packed[c >> 2] >> (8 * (c & 3))) & 1u);
        }
    }
    if (occupied) {
        const unsigned long long sum = blockSum(mine);
        if (threadIdx.x == 0 && sum) atomicAdd(occupied, sum);
    }
}

struct CloudScalars {
    unsigned long long exact[6];  // the exact extremes
    uint32_t keys[6];             // the bounds' first pass, float keys
    unsigned long long filled;
    unsigned long long occupied;
    uint32_t nan;
    uint32_t err;
    uint32_t bigCount;
    uint32_t changed;  // a flood round added cells
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
    for (int a = 0; a < 3; a++) {
        init.keys[a] = ~0u;
        init.exact[a] = ~0ull;
    }
    CK(cudaMemcpyAsync(sc, &init, sizeof init, cudaMemcpyHostToDevice, st), "cloud scratch");
    DeviceBuffer framesBuf;
    POOL_ALLOC(framesBuf, size_t(in.count) * 3 * sizeof(float4), pool, st, "cloud scratch");
    auto* frames = static_cast<float4*>(framesBuf.p);
    cloudBoundsKernel<<<streamGrid(in.count, sms), kCloudBlock, 0, st>>>(in, sc->keys, &sc->nan, frames);
    cloudExtremesKernel<<<streamGrid(in.count, sms), kCloudBlock, 0, st>>>(in, sc->keys, frames, sc->exact);
    CK(cudaGetLastError(), "cloud bounds");
    CloudScalars got{};
    CK(cudaMemcpyAsync(&got, sc, sizeof got, cudaMemcpyDeviceToHost, st), "cloud bounds");
    CK(cudaStreamSynchronize(st), "cloud bounds");

    // cloudVolume.js:113-115, then 2. gridForBounds (voxelize.js:40-67)
    double lo[3], hi[3], extent[3];
    bool nan = got.nan != 0;
    for (int a = 0; a < 3; a++) {
        lo[a] = fromOrderedKey(got.exact[a]);
        hi[a] = fromOrderedKey(got.exact[3 + a]);
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
    // float(1 / h) for the float cell estimate, which wants every quotient
    // it forms a normal float (quotients from 2^-60 / 2^40 up)
    const float invH = float(1.0 / h);
    g.invH = invH >= 0x1p-40f && invH <= 0x1p40f ? invH : 0.0f;
    g.hF = float(h);
    g.floatBound = h >= 0x1p-30 && h <= 0x1p30;
    for (int a = 0; a < 3; a++) {
        g.originF[a] = float(g.origin[a]);
        g.originMag[a] = std::max(std::fabs(g.originF[a]), 0x1p-100f);
        g.floatBound = g.floatBound && std::fabs(g.origin[a]) <= 0x1p40;
    }
    g.cells = n;

    CK(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&v->occupancy), n, pool, st), "cloud occupancy");
    CK(cudaMemsetAsync(v->occupancy, 0, n, st), "cloud occupancy");

    // 3. stamp
    DeviceBuffer bigBuf;
    POOL_ALLOC(bigBuf, size_t(in.count) * 4, pool, st, "cloud scratch");
    cloudStampKernel<<<(in.count + kStampBlock - 1) / kStampBlock, kStampBlock, 0, st>>>(
        in, g, frames, v->occupancy, static_cast<uint32_t*>(bigBuf.p), &sc->bigCount);
    cloudStampBoxKernel<<<uint32_t(sms) * 4, kCloudBlock, 0, st>>>(
        in, g, frames, v->occupancy, static_cast<const uint32_t*>(bigBuf.p), &sc->bigCount);
    CK(cudaGetLastError(), "cloud stamp");

    // 4. seal and fill
    const uint32_t grid = streamGrid(n, sms);
    if (o.fill) {
        // The seal and fill on the cells packed 32 to a word along x: the
        // stamp packed once, `seal` dilations, the flood, the enclosed cells
        // set, `seal` erosions, the stamp put back as the words are written
        // out as bytes once.
        const Words W{(d.nx + 31) / 32, d.ny * d.nz, d.ny, d.nz};
        const size_t words = size_t(W.rows) * W.nw;
        DeviceBuffer wordsBuf;
        POOL_ALLOC(wordsBuf, words * 5 * sizeof(uint32_t), pool, st, "cloud fill scratch");
        uint32_t* stampW = static_cast<uint32_t*>(wordsBuf.p);
        uint32_t* cur = stampW + words;
        uint32_t* other = cur + words;
        uint32_t* emptyW = other + words;
        uint32_t* reachedW = emptyW + words;
        const uint32_t wordGrid = streamGrid(words, sms);
        packCellsKernel<<<wordGrid, kCloudBlock, 0, st>>>(v->occupancy, d, W, stampW);
        const uint32_t* src = stampW;
        for (uint32_t p = 0; p < o.seal; p++) {
            neighbourhoodWordsKernel<true><<<wordGrid, kCloudBlock, 0, st>>>(src, cur, d, W);
            src = cur;
            std::swap(cur, other);
        }
        if (src != stampW) std::swap(cur, other);  // cur: the sealed grid
        else CK(cudaMemcpyAsync(cur, stampW, words * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st), "cloud fill");
        // The flood by sweeps, to a round that adds nothing; past the cap of
        // rounds the union-find decides.
        seedFloodKernel<<<wordGrid, kCloudBlock, 0, st>>>(cur, d, W, emptyW, reachedW);
        // a warp per line, four to a block
        auto lineBlocks = [](uint64_t lines) { return uint32_t(std::max<uint64_t>(1, (lines + 3) / 4)); };
        bool converged = false;
        const uint32_t rounds = floodRounds.load();
        for (uint32_t round = 0; round < rounds && !converged; round++) {
            CK(cudaMemsetAsync(&sc->changed, 0, sizeof(uint32_t), st), "cloud flood");
            sweepXKernel<<<uint32_t((W.rows + 127) / 128), 128, 0, st>>>(W, emptyW, reachedW, &sc->changed);
            sweepLineKernel<<<lineBlocks(uint64_t(d.nz) * W.nw), 128, 0, st>>>(W, d.nz, d.ny, W.nw, W.nw * d.ny,
                                                                                emptyW, reachedW, &sc->changed);
            sweepLineKernel<<<lineBlocks(uint64_t(d.ny) * W.nw), 128, 0, st>>>(W, d.ny, d.nz, W.nw * d.ny, W.nw,
                                                                                emptyW, reachedW, &sc->changed);
            CK(cudaGetLastError(), "cloud flood");
            uint32_t changed = 1;
            CK(cudaMemcpyAsync(&changed, &sc->changed, sizeof changed, cudaMemcpyDeviceToHost, st), "cloud flood");
            CK(cudaStreamSynchronize(st), "cloud flood");
            converged = changed == 0;
        }
        if (converged) {
            encloseWordsKernel<<<wordGrid, kCloudBlock, 0, st>>>(cur, W, emptyW, reachedW, &sc->filled);
        } else {
            // the sealed grid as bytes, filled by the union-find, packed back
            DeviceBuffer work;
            const size_t sealedAt = (size_t(n) * 4 + 15) / 16 * 16;
            POOL_ALLOC(work, sealedAt + size_t(n) * 2 + 64, pool, st, "cloud fill scratch");
            auto* labels = static_cast<uint32_t*>(work.p);
            uint8_t* sealed = static_cast<uint8_t*>(work.p) + sealedAt;
            uint8_t* reached = sealed + n;
            unpackCellsKernel<<<streamGrid((n + 15) / 16, sms), kCloudBlock, 0, st>>>(cur, nullptr, d, W, sealed,
                                                                                       nullptr);
            CK(cudaMemsetAsync(reached, 0, n, st), "cloud fill");
            labelRunsKernel<<<grid, kCloudBlock, 0, st>>>(sealed, labels, d);
            labelMergeKernel<<<grid, kCloudBlock, 0, st>>>(sealed, labels, d, &sc->err);
            markFaceRootsKernel<<<grid, kCloudBlock, 0, st>>>(sealed, labels, reached, d, &sc->err);
            fillEnclosedKernel<<<grid, kCloudBlock, 0, st>>>(sealed, labels, reached, n, &sc->filled, &sc->err);
            packCellsKernel<<<wordGrid, kCloudBlock, 0, st>>>(sealed, d, W, cur);
            CK(cudaStreamSynchronize(st), "cloud fill");  // before `work` is freed
        }
        for (uint32_t p = 0; p < o.seal; p++) {
            neighbourhoodWordsKernel<false><<<wordGrid, kCloudBlock, 0, st>>>(cur, other, d, W);
            std::swap(cur, other);
        }
        unpackCellsKernel<<<streamGrid((n + 15) / 16, sms), kCloudBlock, 0, st>>>(cur, stampW, d, W, v->occupancy,
                                                                                   &sc->occupied);
        CK(cudaGetLastError(), "cloud fill");
        CK(cudaMemcpyAsync(&got, sc, sizeof got, cudaMemcpyDeviceToHost, st), "cloud fill");
        CK(cudaStreamSynchronize(st), "cloud fill");  // before the words are freed
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
    if (!rc) rc = voxelizeCloud(v, CloudInput{d_positions, d_rotations, d_scales, uint32_t(count), options->sigma, float(options->sigma)},
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
    return voxelizeCloud(v, CloudInput{dPos, dRot, dScale, uint32_t(n), o.sigma, float(o.sigma)}, o);
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

uint32_t vsim_cloud_set_flood_rounds(uint32_t rounds) { return floodRounds.exchange(rounds); }

}  // extern "C"
