// Gaussian-splat deformation (sample.wgsl:40-80 with covariance.wgsl:18-42)
// and the stable LSD radix sort behind the depth order.
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
    const float4 e = embed[i];
    const float4 sb = scaleBody[i];
    const float4 q4 = quat[i];
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
    meanDepth[i] = make_float4(position.x, position.y, position.z, depth);
    cov[3 * i] = make_float2(xx, xy);
    cov[3 * i + 1] = make_float2(xz, yy);
    cov[3 * i + 2] = make_float2(yz, zz);
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
// Least-significant-digit radix sort, 8-bit digits, reduce-then-scan per
// pass (no waits between blocks): a per-tile digit histogram, one
// device-wide exclusive scan of the (digit, tile) counts, then a scatter in
// which every warp ranks its 512 consecutive keys with __match_any_sync,
// the block stages the tile in shared memory in digit order, and the tile
// is written out in runs that are contiguous per digit. Tiles and ranks
// follow input order, so each pass -- and the sort -- is stable.

constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortItems = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // 4096 keys
constexpr uint32_t kWarps = kSortThreads / 32;
constexpr uint32_t kScanChunk = 4096;  // elements per block of the scan
constexpr uint32_t kScanMaxChunks = 4096;
constexpr uint32_t kFoldChunks = 64;  // chunks a down-sweep block sums itself

namespace {
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr uint32_t tilesOf(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }
constexpr size_t sortTempBytes(uint32_t n) {
    return 4 * align256(size_t(n) * 4) + align256(256 * size_t(tilesOf(n)) * 4) + align256(kScanMaxChunks * 4);
}
}  // namespace

size_t radixSortTempBytes(uint32_t n) { return sortTempBytes(n); }

uint32_t radixSortLaunches(uint32_t n, uint32_t keyBits) {
    if (n == 0) return 0;
    const uint32_t chunks = (256 * tilesOf(n) + kScanChunk - 1) / kScanChunk;
    return (keyBits + 7) / 8 * (chunks <= kFoldChunks ? 4u : 5u);  // the scan's middle level folded in
}

__global__ void __launch_bounds__(kSortThreads) sortHistKernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                               uint32_t shift, uint32_t mask, uint32_t tiles,
                                                               uint32_t* __restrict__ hist) {
    pdlWait();  // the keys and counts come from the kernel before
    pdlLaunchNext();
    __shared__ uint32_t bins[256];
    bins[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
    for (uint32_t r = 0; r < kSortItems; r++) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&bins[(keys[idx] >> shift) & mask], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = bins[threadIdx.x];
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

// Scan, level 1: each block sums its chunk.
__global__ void __launch_bounds__(kSortThreads) scanReduceKernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                 uint32_t* __restrict__ partial) {
    pdlWait();  // the keys and counts come from the kernel before
    pdlLaunchNext();
    __shared__ uint32_t warpSums[kWarps + 1];
    const uint32_t base = blockIdx.x * kScanChunk;
    uint32_t sum = 0;
    for (uint32_t r = 0; r < kScanChunk / kSortThreads; r++) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) sum += in[idx];
    }
    uint32_t total;
    blockExclusiveScan(sum, warpSums, total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// Scan, level 2: one block scans the chunk sums (at most kScanMaxChunks).
__global__ void __launch_bounds__(kSortThreads) scanPartialKernel(uint32_t* __restrict__ partial, uint32_t chunks) {
    pdlWait();  // the keys and counts come from the kernel before
    pdlLaunchNext();
    __shared__ uint32_t warpSums[kWarps + 1];
    constexpr uint32_t per = kScanMaxChunks / kSortThreads;
    uint32_t v[per];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        const uint32_t idx = threadIdx.x * per + i;
        v[i] = idx < chunks ? partial[idx] : 0;
        sum += v[i];
    }
    uint32_t total;
    uint32_t run = blockExclusiveScan(sum, warpSums, total);
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        const uint32_t idx = threadIdx.x * per + i;
        if (idx < chunks) partial[idx] = run;
        run += v[i];
    }
}

// Scan, level 3: each block scans its chunk from its offset, in place.
__global__ void __launch_bounds__(kSortThreads) scanDownKernel(uint32_t* __restrict__ data, uint32_t n,
                                                               const uint32_t* __restrict__ partial) {
    pdlWait();  // the keys and counts come from the kernel before
    pdlLaunchNext();
    __shared__ uint32_t warpSums[kWarps + 1];
    constexpr uint32_t per = kScanChunk / kSortThreads;
    const uint32_t base = blockIdx.x * kScanChunk + threadIdx.x * per;
    uint32_t v[per];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        v[i] = base + i < n ? data[base + i] : 0;
        sum += v[i];
    }
    uint32_t total;
    uint32_t run = blockExclusiveScan(sum, warpSums, total) + partial[blockIdx.x];
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        if (base + i < n) data[base + i] = run;
        run += v[i];
    }
}

// Scan, levels 2 and 3 in one launch when the chunks are few (at most
// kFoldChunks): each block sums the chunk totals before its own (one per
// thread at most) instead of reading them scanned by scanPartialKernel.

__global__ void __launch_bounds__(kSortThreads) scanDownFoldKernel(uint32_t* __restrict__ data, uint32_t n,
                                                                   const uint32_t* __restrict__ partial) {
    pdlWait();  // the counts and chunk totals come from the kernels before
    pdlLaunchNext();
    __shared__ uint32_t warpSums[kWarps + 1];
    uint32_t before;
    blockExclusiveScan(threadIdx.x < blockIdx.x ? partial[threadIdx.x] : 0u, warpSums, before);
    constexpr uint32_t per = kScanChunk / kSortThreads;
    const uint32_t base = blockIdx.x * kScanChunk + threadIdx.x * per;
    uint32_t v[per];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        v[i] = base + i < n ? data[base + i] : 0;
        sum += v[i];
    }
    uint32_t total;
    uint32_t run = blockExclusiveScan(sum, warpSums, total) + before;
#pragma unroll
    for (uint32_t i = 0; i < per; i++) {
        if (base + i < n) data[base + i] = run;
        run += v[i];
    }
}

__global__ void __launch_bounds__(kSortThreads) sortScatterKernel(const uint32_t* __restrict__ keysIn,
                                                                  const uint32_t* __restrict__ valsIn, uint32_t n,
                                                                  uint32_t shift, uint32_t mask, uint32_t tiles,
                                                                  const uint32_t* __restrict__ offsets,
                                                                  uint32_t* __restrict__ keysOut,
                                                                  uint32_t* __restrict__ valsOut) {
    pdlWait();  // the keys and counts come from the kernel before
    pdlLaunchNext();
    __shared__ uint32_t sKeys[kSortTile];
    __shared__ uint32_t sVals[kSortTile];
    __shared__ uint32_t warpHist[kWarps][256];
    __shared__ uint32_t digitStart[256];
    __shared__ uint32_t globalStart[256];
    __shared__ uint32_t warpSums[kWarps + 1];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t i = threadIdx.x; i < kWarps * 256; i += kSortThreads) (&warpHist[0][0])[i] = 0;
    __syncthreads();

    const uint32_t tileBase = blockIdx.x * kSortTile;
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
    // Per digit: exclusive prefix over warps, then over digits.
    {
        const uint32_t d = threadIdx.x;
        uint32_t running = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; w++) {
            const uint32_t c = warpHist[w][d];
            warpHist[w][d] = running;
            running += c;
        }
        uint32_t total;
        digitStart[d] = blockExclusiveScan(running, warpSums, total);
        globalStart[d] = offsets[d * tiles + blockIdx.x];
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

namespace {
// A sort kernel launched with programmatic dependent launch: its blocks may
// start while the kernel before finishes, and wait (pdlWait) before reading.
template <class... KArgs, class... Args>
void pdl(void (*kernel)(KArgs...), uint32_t grid, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSortThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
}  // namespace

cudaError_t radixSortU32(const uint32_t* keys, uint32_t* order, uint32_t n, uint32_t keyBits, void* temp,
                         size_t tempBytes, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (tempBytes < radixSortTempBytes(n)) return cudaErrorInvalidValue;
    const uint32_t tiles = tilesOf(n);
    const uint32_t histCount = 256 * tiles;
    const uint32_t chunks = (histCount + kScanChunk - 1) / kScanChunk;
    if (chunks > kScanMaxChunks) return cudaErrorInvalidValue;
    char* p = static_cast<char*>(temp);
    const size_t vec = align256(size_t(n) * 4);
    uint32_t* keysA = reinterpret_cast<uint32_t*>(p);
    uint32_t* keysB = reinterpret_cast<uint32_t*>(p + vec);
    uint32_t* valsA = reinterpret_cast<uint32_t*>(p + 2 * vec);
    uint32_t* valsB = reinterpret_cast<uint32_t*>(p + 3 * vec);
    uint32_t* hist = reinterpret_cast<uint32_t*>(p + 4 * vec);
    uint32_t* partial = reinterpret_cast<uint32_t*>(p + 4 * vec + align256(size_t(histCount) * 4));
    const uint32_t passes = (keyBits + 7) / 8;
    const uint32_t* kin = keys;
    const uint32_t* vin = nullptr;
    for (uint32_t pass = 0; pass < passes; pass++) {
        const uint32_t shift = 8 * pass;
        const uint32_t bits = keyBits - shift < 8 ? keyBits - shift : 8;
        const uint32_t mask = (1u << bits) - 1u;
        const bool last = pass + 1 == passes;
        uint32_t* kout = last ? nullptr : (pass % 2 == 0 ? keysA : keysB);
        uint32_t* vout = last ? order : (pass % 2 == 0 ? valsA : valsB);
        pdl(sortHistKernel, tiles, st, kin, n, shift, mask, tiles, hist);
        pdl(scanReduceKernel, chunks, st, (const uint32_t*)hist, histCount, partial);
        if (chunks <= kFoldChunks) {
            pdl(scanDownFoldKernel, chunks, st, hist, histCount, (const uint32_t*)partial);
        } else {
            pdl(scanPartialKernel, 1u, st, partial, chunks);
            pdl(scanDownKernel, chunks, st, hist, histCount, (const uint32_t*)partial);
        }
        pdl(sortScatterKernel, tiles, st, kin, vin, n, shift, mask, tiles, (const uint32_t*)hist, kout, vout);
        kin = kout;
        vin = vout;
    }
    return cudaGetLastError();
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
// The array holds the scratch of kNoAllocMaxKeys keys (about 16 MiB) and lives
// on every GPU that loads the library until the process exits. Every call
// shares it, so calls whose work overlaps on the GPU -- on two streams, or from
// two threads -- race and corrupt each other's results; serialise them. Each
// call writes every scratch word it reads before reading it, so nothing has
// to be cleared between calls.

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

