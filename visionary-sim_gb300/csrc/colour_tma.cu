// The large colour pass with tensor-memory-accelerator brick tiles: each
// block takes bricks of one colour's cells -- 8 x 4 x 4 cells, the colour's
// cells of a 16 x 8 x 8 region of its body -- whose 8 corners are exactly
// one 16 x 8 x 8 box of nodes, a box no other brick of the colour touches.
// A 4-D tensor map per body over (float component, x, y, z) of the node
// arrays brings the box of positions and the box of previous positions into
// shared memory with two bulk copies, the block solves its cells there, and
// one bulk copy writes the position box back (nodes of empty cells go back
// as they came). Two stages: the next brick's boxes load while this one is
// solved. The innermost coordinate is always 0, so every copy starts on a
// 16-byte boundary whatever the brick; boxes that reach past a body's node
// grid load zeros there and store nothing there.
//
// Arithmetic: solveCell on the same corners in the same order as the other
// colour passes (step_device.cuh), so results are equal bit for bit.
// Every mbarrier wait has an iteration limit; a block whose copies do not
// arrive records a fault, waits (bounded) for what it has in flight, and
// leaves.
#include <cuda.h>

#include <vector>

#include "sim_internal.cuh"
#include "step_device.cuh"

namespace vsim {

namespace {

constexpr uint32_t kBoxX = 16, kBoxY = 8, kBoxZ = 8;  // nodes of a brick's box
constexpr uint32_t kBoxNodes = kBoxX * kBoxY * kBoxZ;
constexpr uint32_t kBoxBytes = kBoxNodes * 16;
constexpr uint32_t kStageBytes = 2 * kBoxBytes;  // positions, previous positions
constexpr uint32_t kStages = 2;
constexpr uint32_t kTmaSmem = kStages * kStageBytes + 64;
constexpr uint32_t kTmaBlocksPerSm = 3;  // 3 x 64 KB of shared memory, 3 x 128 threads at ~127 registers
constexpr uint32_t kWaitLimit = 1u << 22;
static_assert(kTmaBlock == (kBoxX / 2) * (kBoxY / 2) * (kBoxZ / 2), "a thread per cell of a brick");

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void barrierInit(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(bar)) : "memory");
}

__device__ __forceinline__ void expectBytes(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}

// Waits for the barrier's phase `parity` to complete, at most kWaitLimit
// tries; false when the limit ran out.
__device__ __forceinline__ bool waitPhase(uint64_t* bar, uint32_t parity) {
    for (uint32_t n = 0; n < kWaitLimit; n++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smemAddr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void loadBox(void* dst, const CUtensorMap* map, const int (&c)[4], uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smemAddr(dst)),
        "l"(map), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(smemAddr(bar))
        : "memory");
}

__device__ __forceinline__ void storeBox(const CUtensorMap* map, const int (&c)[4], const void* src) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(map),
                 "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(smemAddr(src))
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

struct TmaMaps {
    CUtensorMap pos[kTmaBodies];
    CUtensorMap prev[kTmaBodies];
};

// bricks[2 n] = (body, brick x, y, z), bricks[2 n + 1] = the brick's 128
// occupancy bits for this colour (bit mx + 8 (my + 4 mz)).
__global__ void __launch_bounds__(kTmaBlock) elasticTmaKernel(const __grid_constant__ TmaMaps maps,
                                                              const uint4* __restrict__ bricks, uint32_t count,
                                                              uint32_t colour, const DevBody* __restrict__ bodies,
                                                              const uint32_t* __restrict__ bodyActive,
                                                              StretchLengths lens, uint32_t* __restrict__ fault) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    const uint32_t t = threadIdx.x;
    const int ci = int(colour & 1), cj = int((colour >> 1) & 1), ck = int((colour >> 2) & 1);
    auto coords = [&](uint4 e, int (&c)[4]) {
        c[0] = 0;
        c[1] = int(kBoxX * e.y) + ci;
        c[2] = int(kBoxY * e.z) + cj;
        c[3] = int(kBoxZ * e.w) + ck;
    };
    if (t == 0) {
        for (uint32_t s = 0; s < kStages; s++) barrierInit(&full[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // The node arrays are written by the pass before: wait for it.
    pdlWait();
    pdlLaunchNext();
    bool inFlight[kStages] = {false, false};  // thread 0's copies issued and not yet consumed
    auto issue = [&](uint32_t brick, uint32_t s) {
        const uint4 e = bricks[2 * brick];
        int c[4];
        coords(e, c);
        unsigned char* stage = smem + s * kStageBytes;
        expectBytes(&full[s], kStageBytes);
        loadBox(stage, &maps.pos[e.x], c, &full[s]);
        loadBox(stage + kBoxBytes, &maps.prev[e.x], c, &full[s]);
        inFlight[s] = true;
    };
    if (t == 0)
        for (uint32_t s = 0; s < kStages; s++)
            if (blockIdx.x + s * gridDim.x < count) issue(blockIdx.x + s * gridDim.x, s);
    uint32_t phase[kStages] = {0, 0};
    bool failed = false;
    const uint32_t mx = t & 7, my = (t >> 3) & 3, mz = t >> 5;
    uint32_t it = 0;
    for (uint32_t brick = blockIdx.x; brick < count; brick += gridDim.x, it++) {
        const uint32_t s = it & 1;
        const uint4 e = bricks[2 * brick], m = bricks[2 * brick + 1];
        const bool arrived = waitPhase(&full[s], phase[s]);
        if (__syncthreads_or(!arrived)) {
            failed = true;
            break;
        }
        inFlight[s] = false;
        phase[s] ^= 1;
        float4* P = reinterpret_cast<float4*>(smem + s * kStageBytes);
        const float4* Q = P + kBoxNodes;
        const uint32_t word = t < 32 ? m.x : t < 64 ? m.y : t < 96 ? m.z : m.w;
        if (((word >> (t & 31)) & 1u) && bodyActive[e.x]) {
            uint32_t at[8];
#pragma unroll
            for (int c = 0; c < 8; c++)
                at[c] = ((2 * mz + ((c >> 2) & 1)) * kBoxY + (2 * my + ((c >> 1) & 1))) * kBoxX + 2 * mx + (c & 1);
            V p[8], prev[8];
            float w[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const float4 a = P[at[c]];
                p[c] = xyz(a);
                w[c] = a.w;
                prev[c] = xyz(Q[at[c]]);
            }
            solveCell<false>(p, prev, w, cellConsts(bodies + e.x), lens);
#pragma unroll
            for (int c = 0; c < 8; c++) P[at[c]] = withW(p[c], w[c]);
        }
        // The block's writes to the box, visible to the bulk copy.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            int c[4];
            coords(e, c);
            storeBox(&maps.pos[e.x], c, P);
            const uint32_t next = brick + kStages * gridDim.x;
            if (next < count) {
                // The store must have read the stage before the next load overwrites it.
                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                issue(next, s);
            }
        }
    }
    if (t == 0) {
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        if (failed) {
            atomicExch(fault, 1u);
            for (uint32_t s = 0; s < kStages; s++)
                if (inFlight[s]) waitPhase(&full[s], phase[s]);
        }
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

// A body's node array as a 4-D tensor (float component, x, y, z).
bool encodeNodes(CUtensorMap* map, float4* base, const uint32_t nodeDims[3]) {
    EncodeTiled enc = encoder();
    if (!enc) return false;
    const cuuint64_t dims[4] = {4, nodeDims[0], nodeDims[1], nodeDims[2]};
    const cuuint64_t strides[3] = {16, 16ull * nodeDims[0], 16ull * nodeDims[0] * nodeDims[1]};
    const cuuint32_t box[4] = {4, kBoxX, kBoxY, kBoxZ};
    const cuuint32_t step[4] = {1, 1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, step, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int buildTmaPass(vsim_sim* s) {
    TmaPass& t = s->tma;
    t.ready = false;
    if (s->lat.size() > kTmaBodies || s->lat.empty()) return VSIM_OK;  // the pass keeps its other forms
    auto* maps = new (std::nothrow) TmaMaps();
    if (!maps) return fail(VSIM_ERR_NOMEM, "out of host memory");
    for (size_t b = 0; b < s->lat.size(); b++) {
        const Lattice& L = s->lat[b];
        if (!encodeNodes(&maps->pos[b], s->d.pos + s->offsets[b], L.nodeDims) ||
            !encodeNodes(&maps->prev[b], s->d.prev + s->offsets[b], L.nodeDims)) {
            delete maps;
            return fail(VSIM_ERR_CUDA, "encode the node tensor maps");
        }
    }
    // Per colour, the bricks holding its cells, with their occupancy bits.
    std::vector<uint4> list;
    for (int c = 0; c < 8; c++) {
        t.first[c] = uint32_t(list.size() / 2);
        const uint32_t ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
        for (size_t b = 0; b < s->lat.size(); b++) {
            const Lattice& L = s->lat[b];
            const uint32_t bx = (L.cellDims[0] + 2 * (kBoxX / 2) - 1) / (2 * (kBoxX / 2));
            const uint32_t by = (L.cellDims[1] + 2 * (kBoxY / 2) - 1) / (2 * (kBoxY / 2));
            const uint32_t bz = (L.cellDims[2] + 2 * (kBoxZ / 2) - 1) / (2 * (kBoxZ / 2));
            std::vector<uint32_t> bits(size_t(bx) * by * bz * 4, 0);
            for (uint32_t cell : L.cellsByColor[c]) {
                const uint32_t i = cell % L.cellDims[0], j = (cell / L.cellDims[0]) % L.cellDims[1],
                               k = cell / (L.cellDims[0] * L.cellDims[1]);
                const uint32_t mi = (i - ci) / 2, mj = (j - cj) / 2, mk = (k - ck) / 2;
                const size_t brick = (mi / (kBoxX / 2)) + size_t(bx) * ((mj / (kBoxY / 2)) + size_t(by) * (mk / (kBoxZ / 2)));
                const uint32_t bit = (mi % (kBoxX / 2)) + (kBoxX / 2) * ((mj % (kBoxY / 2)) + (kBoxY / 2) * (mk % (kBoxZ / 2)));
                bits[4 * brick + bit / 32] |= 1u << (bit % 32);
            }
            for (uint32_t z = 0; z < bz; z++)
                for (uint32_t y = 0; y < by; y++)
                    for (uint32_t x = 0; x < bx; x++) {
                        const size_t brick = x + size_t(bx) * (y + size_t(by) * z);
                        const uint32_t* w = &bits[4 * brick];
                        if (!(w[0] | w[1] | w[2] | w[3])) continue;
                        list.push_back(make_uint4(uint32_t(b), x, y, z));
                        list.push_back(make_uint4(w[0], w[1], w[2], w[3]));
                    }
        }
        t.count[c] = uint32_t(list.size() / 2) - t.first[c];
    }
    if (t.bricks) cudaFree(t.bricks);
    t.bricks = nullptr;
    if (!t.fault) CK(allocN(&t.fault, 1), "allocate the pass's fault word");
    CK(cudaMemsetAsync(t.fault, 0, 4, s->stream), "clear the pass's fault word");
    CK(allocN(&t.bricks, list.size()), "allocate brick lists");
    CK(cudaMemcpyAsync(t.bricks, list.data(), list.size() * 16, cudaMemcpyHostToDevice, s->stream), "upload bricks");
    CK(cudaStreamSynchronize(s->stream), "upload bricks");
    delete static_cast<TmaMaps*>(t.maps);
    t.maps = maps;
    static bool sized = false;
    if (!sized) {
        CK(cudaFuncSetAttribute(elasticTmaKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmem)),
           "size the pass's shared memory");
        sized = true;
    }
    t.ready = true;
    return VSIM_OK;
}

void freeTmaPass(TmaPass& t) {
    if (t.bricks) cudaFree(t.bricks);
    if (t.fault) cudaFree(t.fault);
    delete static_cast<TmaMaps*>(t.maps);
    t = TmaPass{};
}

cudaError_t launchElasticTma(const LaunchCtx& c, const vsim_sim* s, int colour, const StretchLengths& lens) {
    const TmaPass& t = s->tma;
    const uint32_t count = t.count[colour];
    if (count == 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(std::min(count, kTmaBlocksPerSm * c.sms));
    cfg.blockDim = dim3(kTmaBlock);
    cfg.dynamicSmemBytes = kTmaSmem;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = c.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, elasticTmaKernel, *static_cast<const TmaMaps*>(t.maps),
                              (const uint4*)(t.bricks + 2 * size_t(t.first[colour])), count, uint32_t(colour),
                              (const DevBody*)s->d.bodies, (const uint32_t*)s->d.bodyActive, lens, t.fault);
}

}  // namespace vsim
