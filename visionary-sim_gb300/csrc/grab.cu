// Grabbing on the device: Simulator.grab (simulator.js:383-425) picks the
// node a ray hits and grips a set of nodes around it. The reference reads
// every node position back and does both on the CPU; here the scans run on
// the device, in double precision as the reference's JavaScript computes,
// and only the anchor and the candidates within the grip radius come back.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sim_internal.cuh"

namespace vsim {
namespace {

// pick.js:14-16 (isGrabbableNode): material inverse mass above zero and not
// static -- exactly baseW > 0, the material inverse mass with static nodes
// zeroed.
struct Ray {
    double ox, oy, oz, dx, dy, dz, radius2;
};

// pick.js:53-66 for node n: its depth along the ray if it is grabbable, in
// front of the origin and within the radius of the ray; else -1.
__device__ __forceinline__ double rayDepth(const float4* __restrict__ pos, const float* __restrict__ baseW,
                                           uint32_t n, const Ray& r) {
    if (!(baseW[n] > 0.0f)) return -1.0;
    const float4 P = pos[n];
    const double dx = double(P.x) - r.ox;
    const double dy = double(P.y) - r.oy;
    const double dz = double(P.z) - r.oz;
    const double depth = dx * r.dx + dy * r.dy + dz * r.dz;
    if (!(depth > 0.0)) return -1.0;
    const double offAxis = dx * dx + dy * dy + dz * dz - depth * depth;
    return offAxis > r.radius2 ? -1.0 : depth;
}

// The smallest qualifying depth: positive doubles order as their bit patterns.
__global__ void pickDepthKernel(const float4* __restrict__ pos, const float* __restrict__ baseW, uint32_t n, Ray r,
                                unsigned long long* __restrict__ best) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double depth = rayDepth(pos, baseW, i, r);
    if (depth > 0.0) atomicMin(best, static_cast<unsigned long long>(__double_as_longlong(depth)));
}

// The lowest node at that depth: the loop of pick.js keeps the first one.
__global__ void pickIndexKernel(const float4* __restrict__ pos, const float* __restrict__ baseW, uint32_t n, Ray r,
                                const unsigned long long* __restrict__ best, uint32_t* __restrict__ anchor) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double depth = rayDepth(pos, baseW, i, r);
    if (depth > 0.0 && static_cast<unsigned long long>(__double_as_longlong(depth)) == *best) atomicMin(anchor, i);
}

struct GripCandidate {
    uint32_t node;
    uint32_t pad;
    double distance2;
    double offset[3];
};

// grip.js:113-125: grabbable nodes of [first, end) other than the anchor
// within the radius of it, appended in any order.
__global__ void gripKernel(const float4* __restrict__ pos, const float* __restrict__ baseW, uint32_t first,
                           uint32_t end, uint32_t anchor, double ax, double ay, double az, double radius2,
                           GripCandidate* __restrict__ out, uint32_t* __restrict__ count) {
    const uint32_t n = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= end || n == anchor || !(baseW[n] > 0.0f)) return;
    const float4 P = pos[n];
    const double dx = double(P.x) - ax;
    const double dy = double(P.y) - ay;
    const double dz = double(P.z) - az;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 <= radius2) {
        const uint32_t slot = atomicAdd(count, 1u);
        out[slot] = GripCandidate{n, 0, d2, {dx, dy, dz}};
    }
}

// Device scratch of one grab, freed on every path out.
struct Scratch {
    void* p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace
}  // namespace vsim

using namespace vsim;

extern "C" int vsim_grab(vsim_sim* s, const double origin[3], const double direction[3], int grip,
                         double grip_radius, vsim_grab_result* out) {
    SIM_GUARD(s);
    if (!origin || !direction || !out) return fail(VSIM_ERR_INVALID, "NULL argument");
    if (grip != VSIM_GRIP_SINGLE_NODE && grip != VSIM_GRIP_WITHIN_RADIUS)
        return fail(VSIM_ERR_RANGE, "grip must be VSIM_GRIP_SINGLE_NODE or VSIM_GRIP_WITHIN_RADIUS");
    std::memset(out, 0, sizeof *out);
    out->body = -1;
    if (s->nodeCount == 0) return VSIM_OK;
    // simulator.js:399: a little over the widest node spacing (a lattice's is h).
    double coarsest = 0;
    for (const Lattice& L : s->lat) coarsest = std::max(coarsest, L.h);
    const double aim = coarsest * 1.2;
    const Ray ray{origin[0], origin[1], origin[2], direction[0], direction[1], direction[2], aim * aim};

    Scratch scratch;
    CK(cudaMalloc(&scratch.p, 16), "grab");
    auto* best = static_cast<unsigned long long*>(scratch.p);
    auto* anchorDev = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch.p) + 8);
    CK(cudaMemsetAsync(best, 0xff, 8, s->stream), "grab");
    CK(cudaMemsetAsync(anchorDev, 0xff, 4, s->stream), "grab");
    const uint32_t n = s->nodeCount, blocks = (n + 255) / 256;
    pickDepthKernel<<<blocks, 256, 0, s->stream>>>(s->d.pos, s->d.baseW, n, ray, best);
    pickIndexKernel<<<blocks, 256, 0, s->stream>>>(s->d.pos, s->d.baseW, n, ray, best, anchorDev);
    CK(cudaGetLastError(), "pick");
    uint32_t anchor = 0xffffffffu;
    CK(cudaMemcpyAsync(&anchor, anchorDev, 4, cudaMemcpyDeviceToHost, s->stream), "pick");
    float4 at{};
    CK(cudaStreamSynchronize(s->stream), "pick");
    if (anchor >= n) return VSIM_OK;  // the ray missed
    CK(cudaMemcpyAsync(&at, s->d.pos + anchor, 16, cudaMemcpyDeviceToHost, s->stream), "pick");
    CK(cudaStreamSynchronize(s->stream), "pick");
    const double ax = at.x, ay = at.y, az = at.z;
    const uint32_t body = bodyOfNode(s, anchor);

    std::vector<uint32_t> nodes{anchor};
    std::vector<float> offsets{0.0f, 0.0f, 0.0f};
    uint32_t found = 1;
    if (grip == VSIM_GRIP_WITHIN_RADIUS) {
        const uint32_t first = s->offsets[body], end = first + s->lat[body].nodeCount;
        Scratch list;
        CK(cudaMalloc(&list.p, size_t(end - first) * sizeof(GripCandidate) + 16), "grip");
        auto* count = reinterpret_cast<uint32_t*>(list.p);
        auto* cand = reinterpret_cast<GripCandidate*>(static_cast<char*>(list.p) + 16);
        CK(cudaMemsetAsync(count, 0, 4, s->stream), "grip");
        gripKernel<<<(end - first + 255) / 256, 256, 0, s->stream>>>(s->d.pos, s->d.baseW, first, end, anchor, ax, ay,
                                                                     az, grip_radius * grip_radius, cand, count);
        CK(cudaGetLastError(), "grip");
        uint32_t m = 0;
        CK(cudaMemcpyAsync(&m, count, 4, cudaMemcpyDeviceToHost, s->stream), "grip");
        CK(cudaStreamSynchronize(s->stream), "grip");
        std::vector<GripCandidate> c(m);
        if (m) {
            CK(cudaMemcpyAsync(c.data(), cand, size_t(m) * sizeof(GripCandidate), cudaMemcpyDeviceToHost, s->stream),
               "grip");
            CK(cudaStreamSynchronize(s->stream), "grip");
        }
        // grip.js:126-135: nearest first, ties by index, anchor first.
        std::sort(c.begin(), c.end(), [](const GripCandidate& a, const GripCandidate& b) {
            return a.distance2 != b.distance2 ? a.distance2 < b.distance2 : a.node < b.node;
        });
        found = m + 1;
        const size_t kept = std::min<size_t>(m, VSIM_MAX_DRIVEN - 1);
        for (size_t k = 0; k < kept; k++) {
            nodes.push_back(c[k].node);
            for (int a = 0; a < 3; a++) offsets.push_back(float(c[k].offset[a]));
        }
    }
    const int rc = holdNodes(s, nodes.data(), offsets.data(), uint32_t(nodes.size()));
    if (rc) return rc;
    const double position[3] = {ax, ay, az};
    std::memcpy(s->grabPos, position, sizeof s->grabPos);
    std::memcpy(s->grabPrev, position, sizeof s->grabPrev);
    s->frameDirty = true;
    out->body = int32_t(body);
    out->anchor = anchor;
    std::memcpy(out->position, position, sizeof position);
    out->held = uint32_t(nodes.size());
    out->found = found;
    return VSIM_OK;
}
