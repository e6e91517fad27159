// Gaussian-splat deformation (sample.wgsl:40-80 with covariance.wgsl:18-42)
// and the stable LSD radix sort behind the depth order.
#include <algorithm>
#include <mutex>
#include <string>

#include "kernels.cuh"

namespace vsim {

// ------------------------------------------------------------- splats --

// Back-to-front draw key: ascending key order is descending depth.
__device__ __forceinline__ uint32_t depthKey(float depth) {
    const uint32_t bits = __float_as_uint(depth);
    const uint32_t ordered = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
    return ~ordered;
}

// One thread per splat: trilinear position and gradient F from the cell's
// eight live nodes, then Sigma' = (F R S)(F R S)^T, then the depth key. The
// embedding (cell corner node, local coordinates) was computed at bind time
// with sample.wgsl:45-51's arithmetic.
// ellipsoid.wgsl:20-91: a covariance (xx, xy, xz, yy, yz, zz) as a unit
// quaternion xyzw and three axis lengths, by four sweeps of cyclic Jacobi.
// inverseSqrt is 1 / sqrt and normalize is q / sqrt(|q|^2) with |q|^2 fused
// as dot is; every other operation rounds once -- the CPU restatement's
// evaluation, so the two agree bit for bit.
__device__ __forceinline__ void ellipsoidAxes(const float cov[6], float4& rotation, float4& scale) {
    float a[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
    float q[4] = {0.0f, 0.0f, 0.0f, 1.0f};
#pragma unroll
    for (int sweep = 0; sweep < 4; sweep++) {
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const int r = (p + 1) % 3, other = (p + 2) % 3;
            const float apr = a[r * 3 + p];
            if (apr == 0.0f) continue;
            const float app = a[p * 3 + p];
            const float arr = a[r * 3 + r];
            const float theta = (arr - app) / (2.0f * apr);
            const float sign = theta >= 0.0f ? 1.0f : -1.0f;
            const float tangent = sign / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
            const float cosine = 1.0f / sqrtf(tangent * tangent + 1.0f);
            const float sine = tangent * cosine;
            const float apo = a[other * 3 + p];
            const float aro = a[other * 3 + r];
            const float turnedP = cosine * apo - sine * aro;
            const float turnedR = sine * apo + cosine * aro;
            a[p * 3 + p] = app - tangent * apr;
            a[r * 3 + r] = arr + tangent * apr;
            a[r * 3 + p] = 0.0f;
            a[p * 3 + r] = 0.0f;
            a[other * 3 + p] = turnedP;
            a[p * 3 + other] = turnedP;
            a[other * 3 + r] = turnedR;
            a[r * 3 + other] = turnedR;
            const float half = -(sine / (1.0f + cosine));
            float b[4] = {0.0f, 0.0f, 0.0f, 1.0f};
            b[other] = half;
            const float prod[4] = {q[3] * b[0] + q[0] * b[3] + q[1] * b[2] - q[2] * b[1],
                                   q[3] * b[1] - q[0] * b[2] + q[1] * b[3] + q[2] * b[0],
                                   q[3] * b[2] + q[0] * b[1] - q[1] * b[0] + q[2] * b[3],
                                   q[3] * b[3] - q[0] * b[0] - q[1] * b[1] - q[2] * b[2]};
            const float length =
                sqrtf(fmaf(prod[3], prod[3], fmaf(prod[2], prod[2], fmaf(prod[1], prod[1], prod[0] * prod[0]))));
#pragma unroll
            for (int c = 0; c < 4; c++) q[c] = prod[c] / length;
        }
    }
    rotation = make_float4(q[0], q[1], q[2], q[3]);
    scale = make_float4(sqrtf(fmaxf(a[0], 0.0f)), sqrtf(fmaxf(a[4], 0.0f)), sqrtf(fmaxf(a[8], 0.0f)), 0.0f);
}

template <bool AXES>
__global__ void __launch_bounds__(256) splatDeformKernel(const float4* __restrict__ embed,
                                                         const float4* __restrict__ quat,
                                                         const float4* __restrict__ scaleBody,
                                                         const SplatBody* __restrict__ bodies,
                                                         const float4* __restrict__ pos, uint32_t n, float vx,
                                                         float vy, float vz, float4* __restrict__ meanDepth,
                                                         float2* __restrict__ cov, uint32_t* __restrict__ keys,
                                                         uint32_t* __restrict__ order,
                                                         float4* __restrict__ axesRotation,
                                                         float4* __restrict__ axesScale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // The splat's embedding, scale and rotation do not change between
    // frames: loaded before waiting for the frame that moves the nodes.
    // The splat streams are read and written once, marked evict-first
    // (.cs), so that the node positions the corner gathers hit stay in L2.
    const float4 e = __ldcs(embed + i);
    const float4 sb = __ldcs(scaleBody + i);
    const float4 q4 = __ldcs(quat + i);
    const SplatBody B = bodies[__float_as_uint(sb.w)];
    pdlWait();
    pdlLaunchNext();
    const uint32_t node0 = __float_as_uint(e.w);
    const float local[3] = {e.x, e.y, e.z};
    const float inv = B.inv;
    V position = mk(0.0f, 0.0f, 0.0f);
    V col0 = mk(0.0f, 0.0f, 0.0f), col1 = col0, col2 = col0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
        const float fx = cx ? local[0] : 1.0f - local[0];
        const float fy = cy ? local[1] : 1.0f - local[1];
        const float fz = cz ? local[2] : 1.0f - local[2];
        const float dx = cx ? 1.0f : -1.0f, dy = cy ? 1.0f : -1.0f, dz = cz ? 1.0f : -1.0f;
        const V p = xyz(pos[node0 + cx + B.nx * cy + B.nxy * cz]);
        position = position + p * (fx * fy * fz);
        const V g = mk(dx * fy * fz, dy * fx * fz, dz * fx * fy) * inv;
        col0 = col0 + p * g.x;
        col1 = col1 + p * g.y;
        col2 = col2 + p * g.z;
    }
    const M F{{col0, col1, col2}};
    const float x = q4.x, y = q4.y, z = q4.z, w = q4.w;
    const V r0 = mk(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w));
    const V r1 = mk(2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w));
    const V r2 = mk(2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y));
    const V a0 = mul(F, r0) * sb.x;
    const V a1 = mul(F, r1) * sb.y;
    const V a2 = mul(F, r2) * sb.z;
    // (A A^T)(row, col) = a0[row] a0[col] + a1[row] a1[col] + a2[row] a2[col],
    // column col of A times row col of A^T, fused as M * v is.
    const float xx = fmaf(a2.x, a2.x, fmaf(a1.x, a1.x, a0.x * a0.x));
    const float xy = fmaf(a2.y, a2.x, fmaf(a1.y, a1.x, a0.y * a0.x));
    const float xz = fmaf(a2.z, a2.x, fmaf(a1.z, a1.x, a0.z * a0.x));
    const float yy = fmaf(a2.y, a2.y, fmaf(a1.y, a1.y, a0.y * a0.y));
    const float yz = fmaf(a2.z, a2.y, fmaf(a1.z, a1.y, a0.z * a0.y));
    const float zz = fmaf(a2.z, a2.z, fmaf(a1.z, a1.z, a0.z * a0.z));
    const float depth = position.x * vx + position.y * vy + position.z * vz;
    __stcs(meanDepth + i, make_float4(position.x, position.y, position.z, depth));
    __stcs(cov + 3 * i, make_float2(xx, xy));
    __stcs(cov + 3 * i + 1, make_float2(xz, yy));
    __stcs(cov + 3 * i + 2, make_float2(yz, zz));
    keys[i] = depthKey(depth);
    (void)order;
    if (AXES) {
        const float c6[6] = {xx, xy, xz, yy, yz, zz};
        ellipsoidAxes(c6, axesRotation[i], axesScale[i]);
    }
}

cudaError_t launchSplatDeform(cudaStream_t st, const SplatState& s, const float4* pos, uint32_t n, float vx, float vy,
                              float vz, bool axes) {
    if (n == 0) return cudaSuccess;
    // Programmatic dependent launch: the constant loads above overlap the
    // tail of the frame's last kernel.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((n + 255) / 256);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (axes)
        return cudaLaunchKernelEx(&cfg, splatDeformKernel<true>, (const float4*)s.embed, (const float4*)s.quat,
                                  (const float4*)s.scaleBody, (const SplatBody*)s.bodies, pos, n, vx, vy, vz,
                                  s.meanDepth, s.cov, s.keys, s.order, s.axesRotation, s.axesScale);
    return cudaLaunchKernelEx(&cfg, splatDeformKernel<false>, (const float4*)s.embed, (const float4*)s.quat,
                              (const float4*)s.scaleBody, (const SplatBody*)s.bodies, pos, n, vx, vy, vz, s.meanDepth,
                              s.cov, s.keys, s.order, (float4*)nullptr, (float4*)nullptr);
}

// --------------------------------------------------------- radix sort --
//
// Least-significant-digit radix sort, 8-bit digits, one sweep of the keys
// per pass -- the single-pass scan with decoupled look-back (Merrill and
// Garland, 2016) applied to radix sorting as Adinets and Merrill's
// "Onesweep" (2022) does:
//
// - one launch counts every pass's digits over all the keys at once (a
//   pass's digit totals do not depend on the order earlier passes leave);
// - then one launch per pass. Each block takes the next tile from a ticket,
//   so tiles start in order; it ranks its 4096 keys per digit (every warp
//   its 512 with __match_any_sync) and publishes the tile's count of each
//   digit in a status word (count and a flag packed in 32 bits, so one store
//   carries both). Then each digit's thread walks back over the tiles before
//   it, adding their counts until it meets a word that already holds an
//   inclusive prefix, and publishes the tile's own. A tile waits only on
//   tiles that started before it, which publish their counts without
//   waiting on anything, so every walk ends. With the digit's global start
//   (the histogram, scanned) the block writes the tile out in runs that are
//   contiguous per digit.
//
// Tiles and ranks follow input order, so each pass -- and the sort -- is
// stable. The status words, digit totals and tickets are cleared by one
// memset at the start of a sort; every other scratch word is written before
// it is read.

constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortItems = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // 4096 keys
constexpr uint32_t kWarps = kSortThreads / 32;
constexpr uint32_t kSortMaxPasses = 4;
constexpr uint32_t kStatusCount = 1u << 30;     // the word holds the tile's own count
constexpr uint32_t kStatusPrefix = 2u << 30;    // the word holds the inclusive prefix
constexpr uint32_t kStatusValue = (1u << 30) - 1u;
constexpr uint32_t kLookbackSpinLimit = 1u << 22;

namespace {
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr uint32_t tilesOf(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }
// Cleared at the start of a sort: per pass, a status word per (tile, digit);
// the digit totals of every pass; a ticket per pass and the failure word.
constexpr size_t sortStatusBytes(uint32_t n) { return align256(size_t(kSortMaxPasses) * tilesOf(n) * 256 * 4); }
constexpr size_t sortClearedBytes(uint32_t n) {
    return sortStatusBytes(n) + align256(kSortMaxPasses * 256 * 4) + 256;
}
constexpr size_t sortTempBytes(uint32_t n) { return 4 * align256(size_t(n) * 4) + sortClearedBytes(n); }
}  // namespace

size_t radixSortTempBytes(uint32_t n) { return sortTempBytes(n); }

uint32_t radixSortLaunches(uint32_t n, uint32_t keyBits) {
    if (n == 0) return 0;
    return 1 + (keyBits + 7) / 8;  // the digit counts, then one launch per pass
}

__device__ __forceinline__ uint32_t loadRelaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void storeRelaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Every pass's digit counts over all keys: per block in shared memory, then
// added into totals[pass * 256 + digit].
__global__ void __launch_bounds__(kSortThreads) sortDigitCountKernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                     uint32_t keyBits,
                                                                     uint32_t* __restrict__ totals) {
    __shared__ uint32_t bins[kSortMaxPasses * 256];
    for (uint32_t i = threadIdx.x; i < kSortMaxPasses * 256; i += kSortThreads) bins[i] = 0;
    pdlWait();  // the keys come from the kernel before
    pdlLaunchNext();
    __syncthreads();
    const uint32_t passes = (keyBits + 7) / 8;
    auto count = [&](uint32_t k) {
#pragma unroll
        for (uint32_t p = 0; p < kSortMaxPasses; p++) {
            if (p >= passes) break;
            const uint32_t bits = keyBits - 8 * p < 8 ? keyBits - 8 * p : 8;
            atomicAdd(&bins[p * 256 + ((k >> (8 * p)) & ((1u << bits) - 1u))], 1u);
        }
    };
    const uint32_t stride = gridDim.x * kSortThreads;
    // four keys per load where the keys start on a 16-byte boundary
    const uint32_t quads = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0 ? n / 4 : 0;
    const uint4* k4 = reinterpret_cast<const uint4*>(keys);
    for (uint32_t i = blockIdx.x * kSortThreads + threadIdx.x; i < quads; i += stride) {
        const uint4 q = k4[i];
        count(q.x);
        count(q.y);
        count(q.z);
        count(q.w);
    }
    for (uint32_t i = 4 * quads + blockIdx.x * kSortThreads + threadIdx.x; i < n; i += stride) count(keys[i]);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * 256; i += kSortThreads)
        if (bins[i]) atomicAdd(&totals[i], bins[i]);
}

// Block-wide exclusive scan of one value per thread (256 threads); returns
// the block total through `total`.
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* warpSums, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= uint32_t(d)) incl += u;
    }
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t s = lane < kWarps ? warpSums[lane] : 0;
        uint32_t sc = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, sc, d);
            if (lane >= uint32_t(d)) sc += u;
        }
        if (lane < kWarps) warpSums[lane] = sc - s;
        if (lane == kWarps - 1) warpSums[kWarps] = sc;
    }
    __syncthreads();
    total = warpSums[kWarps];
    const uint32_t out = warpSums[warp] + incl - v;
    __syncthreads();
    return out;
}

// One pass: rank a tile, find its digits' global offsets by decoupled
// look-back, scatter. `status` is this pass's (tile, digit) words, `totals`
// its 256 digit counts over all keys.
__device__ __forceinline__ void sortPass(const uint32_t* __restrict__ keysIn, const uint32_t* __restrict__ valsIn,
                                         uint32_t n, uint32_t shift, uint32_t mask,
                                         const uint32_t* __restrict__ totals, uint32_t* __restrict__ status,
                                         uint32_t* __restrict__ ticket, uint32_t* __restrict__ error,
                                         uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut) {
    __shared__ uint32_t sKeys[kSortTile];
    __shared__ uint32_t sVals[kSortTile];
    __shared__ uint32_t warpHist[kWarps][256];
    __shared__ uint32_t digitStart[256];
    __shared__ uint32_t globalStart[256];
    __shared__ uint32_t warpSums[kWarps + 1];
    __shared__ uint32_t sTile;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // The ticket counter was cleared before the sort's first launch, which
    // this one follows in stream order: safe to take before the wait.
    if (threadIdx.x == 0) sTile = atomicAdd(ticket, 1u);
    for (uint32_t i = threadIdx.x; i < kWarps * 256; i += kSortThreads) (&warpHist[0][0])[i] = 0;
    pdlWait();  // the keys and totals come from the kernels before
    pdlLaunchNext();
    __syncthreads();
    const uint32_t tile = sTile;
    const uint32_t tileBase = tile * kSortTile;
    const uint32_t warpBase = tileBase + warp * 32 * kSortItems;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
    for (uint32_t r = 0; r < kSortItems; r++) {
        const uint32_t idx = warpBase + r * 32 + lane;
        const bool valid = idx < n;
        key[r] = valid ? keysIn[idx] : 0u;
        val[r] = valid ? (valsIn ? valsIn[idx] : idx) : 0u;
        const uint32_t digit = valid ? (key[r] >> shift) & mask : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t before = valid ? warpHist[warp][digit] : 0u;
        __syncwarp();
        if (valid && (peers & lt) == 0) warpHist[warp][digit] = before + __popc(peers);
        __syncwarp();
        rank[r] = before + __popc(peers & lt);
    }
    __syncthreads();
    {
        const uint32_t d = threadIdx.x;
        // Per digit: exclusive prefix over warps, and the tile's count.
        uint32_t count = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; w++) {
            const uint32_t c = warpHist[w][d];
            warpHist[w][d] = count;
            count += c;
        }
        uint32_t* mine = status + size_t(tile) * 256 + d;
        storeRelaxed(mine, (tile == 0 ? kStatusPrefix : kStatusCount) | count);
        // Decoupled look-back over the tiles before this one.
        uint32_t before = 0;
        if (tile > 0) {
            uint32_t j = tile - 1, polls = 0;
            while (true) {
                const uint32_t word = loadRelaxed(status + size_t(j) * 256 + d);
                if ((word & ~kStatusValue) == 0) {  // tile j has not published yet
                    if (++polls > kLookbackSpinLimit) {
                        atomicOr(error, 1u);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                before += word & kStatusValue;
                if ((word & ~kStatusValue) == kStatusPrefix || j == 0) break;
                j--;
            }
            storeRelaxed(mine, kStatusPrefix | (before + count));
        }
        uint32_t total;
        digitStart[d] = blockExclusiveScan(count, warpSums, total);
        const uint32_t digitBase = blockExclusiveScan(totals[d], warpSums, total);
        globalStart[d] = digitBase + before;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kSortItems; r++) {
        const uint32_t idx = warpBase + r * 32 + lane;
        if (idx < n) {
            const uint32_t digit = (key[r] >> shift) & mask;
            const uint32_t slot = digitStart[digit] + warpHist[warp][digit] + rank[r];
            sKeys[slot] = key[r];
            sVals[slot] = val[r];
        }
    }
    __syncthreads();
    const uint32_t count = n - tileBase < kSortTile ? n - tileBase : kSortTile;
    for (uint32_t j = threadIdx.x; j < count; j += kSortThreads) {
        const uint32_t k = sKeys[j];
        const uint32_t digit = (k >> shift) & mask;
        const uint32_t out = globalStart[digit] + (j - digitStart[digit]);
        if (keysOut) keysOut[out] = k;
        valsOut[out] = sVals[j];
    }
}

// The pass as two kernels: sortPassKernel at the registers the compiler
// picks (86: two blocks an SM), sortPassWideKernel squeezed to 80 so that
// three fit. The second is faster once the tiles take several waves (20M
// keys: 27.4 against 23.6 G keys/s), slower within one wave, where each
// tile's latency is the pass (1M keys: 0.096 against 0.080 ms a sort).
__global__ void __launch_bounds__(kSortThreads) sortPassKernel(const uint32_t* __restrict__ keysIn,
                                                               const uint32_t* __restrict__ valsIn, uint32_t n,
                                                               uint32_t shift, uint32_t mask,
                                                               const uint32_t* __restrict__ totals,
                                                               uint32_t* __restrict__ status,
                                                               uint32_t* __restrict__ ticket,
                                                               uint32_t* __restrict__ error,
                                                               uint32_t* __restrict__ keysOut,
                                                               uint32_t* __restrict__ valsOut) {
    sortPass(keysIn, valsIn, n, shift, mask, totals, status, ticket, error, keysOut, valsOut);
}

__global__ void __launch_bounds__(kSortThreads, 3) sortPassWideKernel(const uint32_t* __restrict__ keysIn,
                                                                      const uint32_t* __restrict__ valsIn,
                                                                      uint32_t n, uint32_t shift, uint32_t mask,
                                                                      const uint32_t* __restrict__ totals,
                                                                      uint32_t* __restrict__ status,
                                                                      uint32_t* __restrict__ ticket,
                                                                      uint32_t* __restrict__ error,
                                                                      uint32_t* __restrict__ keysOut,
                                                                      uint32_t* __restrict__ valsOut) {
    sortPass(keysIn, valsIn, n, shift, mask, totals, status, ticket, error, keysOut, valsOut);
}

namespace {
// A sort kernel launched with programmatic dependent launch: its blocks may
// start while the kernel before finishes, and wait (pdlWait) before reading.
template <class... KArgs, class... Args>
cudaError_t pdl(void (*kernel)(KArgs...), uint32_t grid, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSortThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
}  // namespace

cudaError_t radixSortU32(const uint32_t* keys, uint32_t* order, uint32_t n, uint32_t keyBits, void* temp,
                         size_t tempBytes, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (tempBytes < radixSortTempBytes(n) || n > kStatusValue || keyBits < 1 || keyBits > 32)
        return cudaErrorInvalidValue;
    const uint32_t tiles = tilesOf(n);
    char* p = static_cast<char*>(temp);
    const size_t vec = align256(size_t(n) * 4);
    uint32_t* keysA = reinterpret_cast<uint32_t*>(p);
    uint32_t* keysB = reinterpret_cast<uint32_t*>(p + vec);
    uint32_t* valsA = reinterpret_cast<uint32_t*>(p + 2 * vec);
    uint32_t* valsB = reinterpret_cast<uint32_t*>(p + 3 * vec);
    char* cleared = p + 4 * vec;
    uint32_t* status = reinterpret_cast<uint32_t*>(cleared);
    uint32_t* totals = reinterpret_cast<uint32_t*>(cleared + sortStatusBytes(n));
    uint32_t* tickets = reinterpret_cast<uint32_t*>(cleared + sortStatusBytes(n) + align256(kSortMaxPasses * 256 * 4));
    uint32_t* error = tickets + kSortMaxPasses;
    const uint32_t passes = (keyBits + 7) / 8;
    cudaError_t e;
    if ((e = cudaMemsetAsync(cleared, 0, sortClearedBytes(n), st))) return e;
    int device = 0, sms = 0;
    if ((e = cudaGetDevice(&device)) || (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)))
        return e;
    const uint32_t countGrid = std::min<uint32_t>(tiles, 2u * uint32_t(sms));
    if ((e = pdl(sortDigitCountKernel, countGrid, st, keys, n, keyBits, totals))) return e;
    const uint32_t* kin = keys;
    const uint32_t* vin = nullptr;
    for (uint32_t pass_ = 0; pass_ < passes; pass_++) {
        const uint32_t shift = 8 * pass_;
        const uint32_t bits = keyBits - shift < 8 ? keyBits - shift : 8;
        const uint32_t mask = (1u << bits) - 1u;
        const bool last = pass_ + 1 == passes;
        uint32_t* kout = last ? nullptr : (pass_ % 2 == 0 ? keysA : keysB);
        uint32_t* vout = last ? order : (pass_ % 2 == 0 ? valsA : valsB);
        auto pass = [&](auto kernel) {
            return pdl(kernel, tiles, st, kin, vin, n, shift, mask, (const uint32_t*)(totals + 256 * pass_),
                       status + size_t(pass_) * tiles * 256, tickets + pass_, error, kout, vout);
        };
        if ((e = tiles > 2u * uint32_t(sms) ? pass(sortPassWideKernel) : pass(sortPassKernel))) return e;
        kin = kout;
        vin = vout;
    }
    return cudaSuccess;
}

}  // namespace vsim

// ------------------------------------------------- sort without allocating --
//
// Some callers cannot allocate device memory: a host engine that owns every
// byte of the GPU through its own pool and forbids libraries to allocate
// behind its back, a real-time frame loop that may not risk cudaMalloc's
// implicit device synchronisation or an allocation stall mid-frame, or a thin
// binding handed nothing but raw device pointers. For them the sort below
// takes its scratch from a fixed array compiled into this library instead of
// from the caller: it allocates nothing and frees nothing.
//
// The array holds the scratch of kNoAllocMaxKeys keys (about 17 MiB) and lives
// on every GPU that loads the library until the process exits. Every call
// shares it, so calls whose work overlaps on the GPU -- on two streams, or from
// two threads -- race and corrupt each other's results; serialise them. The
// array keeps the last call's contents: each call first clears (with a memset
// on its stream) the words that must start at zero -- the look-back status
// words, digit totals and tile tickets -- and writes every other word before
// reading it.

namespace vsim {
namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
constexpr size_t kNoAllocScratchBytes = sortTempBytes(kNoAllocMaxKeys);

__device__ __align__(256) static unsigned char g_sortScratch[kNoAllocScratchBytes];

// In host code `g_sortScratch` names a host-side stand-in, not device memory:
// the device address comes from cudaGetSymbolAddress, looked up with the
// device current and cached per device together with the identity of the
// context it was looked up in. A device reset (cudaDeviceReset, or a primary
// context torn down and made again) reloads the module and may move the
// array; the next call sees a new context and looks the address up again.
constexpr int kMaxDevices = 64;
std::mutex g_scratchLock;
struct ScratchEntry {
    void* ptr;
    unsigned long long context;  // 0: unknown, never trusted
};
ScratchEntry g_scratchAddress[kMaxDevices] = {};

// The unique id of the calling thread's current context (cuCtxGetId), 0 when
// there is none or the driver cannot say. Reached through the runtime's
// driver entry points, so the library does not link libcuda itself.
unsigned long long currentContextId() {
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent getCurrent = nullptr;
    static GetId getId = nullptr;
    static std::once_flag found;
    std::call_once(found, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getCurrent = reinterpret_cast<GetCurrent>(fn);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getId = reinterpret_cast<GetId>(fn);
    });
    if (!getCurrent || !getId) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (getCurrent(&ctx) != 0 || !ctx || getId(ctx, &id) != 0) return 0;
    return id;
}

cudaError_t scratchAddress(void** out) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> hold(g_scratchLock);
    ScratchEntry& entry = g_scratchAddress[device];
    const unsigned long long context = currentContextId();
    if (!entry.ptr || context == 0 || entry.context != context) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_sortScratch);  // makes the device's context current if none was
        if (e != cudaSuccess) return e;
        entry.ptr = ptr;
        entry.context = context ? context : currentContextId();
    }
    *out = entry.ptr;
    return cudaSuccess;
}


}  // namespace

}  // namespace vsim

extern "C" int vsim_radix_sort_u32_noalloc(const uint32_t* d_keys, uint32_t* d_order, uint32_t n, uint32_t key_bits,
                                           void* stream) {
    using namespace vsim;
    clearError();
    if (key_bits < 1 || key_bits > 32) return fail(VSIM_ERR_RANGE, "key_bits must be in [1, 32]");
    if (n > kNoAllocMaxKeys)
        return fail(VSIM_ERR_CAPACITY, "vsim_radix_sort_u32_noalloc sorts at most 1048576 keys; use "
                                       "vsim_radix_sort_u32 with caller-provided scratch for more");
    if (n == 0) return VSIM_OK;
    if (!d_keys || !d_order) return fail(VSIM_ERR_INVALID, "keys or order is NULL");
    if (wordRangesOverlap(d_keys, d_order, n)) return fail(VSIM_ERR_INVALID, "keys and order overlap");
    void* scratch = nullptr;
    cudaError_t e = scratchAddress(&scratch);
    if (e != cudaSuccess) return fail(VSIM_ERR_CUDA, std::string("scratch address: ") + cudaGetErrorString(e));
    e = radixSortU32(d_keys, d_order, n, key_bits, scratch, kNoAllocScratchBytes, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(VSIM_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    return VSIM_OK;
}

