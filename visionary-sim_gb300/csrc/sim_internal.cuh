// The simulator object and the helpers that the C entry points of sim.cu
// and the session server of server.cu share. Internal to libvsim.
#pragma once

#include <string>
#include <vector>

#include "kernels.cuh"

namespace vsim {

// Restores the caller's current device when a call returns.
struct DeviceGuard {
    int previous = -1;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&previous) != cudaSuccess) previous = -1;
        if (previous != device) cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        if (previous >= 0 && cudaGetDevice(&now) == cudaSuccess && now != previous) cudaSetDevice(previous);
    }
};

inline int cudaFail(cudaError_t e, const char* what) {
    return fail(VSIM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr, what)                                       \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return cudaFail(_e, what);    \
    } while (0)

template <class T>
cudaError_t allocN(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
}

struct GraphEntry {
    uint64_t key;
    cudaGraphExec_t exec;
};

// The spans of one frame's launches: the nodes predict and finalize visit,
// each colour's cells, the surface records.
struct FramePlan {
    bool chunked = false;  // spans cover only some bodies (built per frame)
    Span nodes{};
    Span colour[8]{};
    Span records{};
};

}  // namespace vsim

struct vsim_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    cudaStream_t capture = nullptr;
    uint32_t sms = 1;

    // topology
    std::vector<vsim::Lattice> lat;
    std::vector<vsim_material> mat;
    std::vector<uint32_t> offsets;
    std::vector<uint8_t> isStatic;
    std::vector<float> invMass;  // material inverse mass (Particles.invMass)
    std::vector<float> baseW;    // invMass with static nodes zeroed
    std::vector<float> restPos;  // xyzw per node, w = baseW
    uint32_t nodeCount = 0, activeCount = 0, cellCount = 0, surfaceCount = 0;
    uint32_t colorStart[9] = {};
    std::vector<uint4> surfHost;
    vsim_tank tank{};
    // Contact grids: one shared by all bodies, or one per body when the
    // bodies are isolated (they never touch each other).
    bool isolated = false;
    std::vector<vsim::Grid> grids;
    std::vector<uint32_t> gridBase;
    uint64_t bucketTotal = 0;

    // settings
    double gravity[3] = {0, -9.81, 0};
    bool paused = false, pendingStep = false;
    bool contact = true, selfContact = false;
    uint32_t iterations = 1;
    bool useGraph = true, pdl = true;
    int gatherMapping = VSIM_GATHER_AUTO;
    uint32_t block = 256, brick = 0;
    vsim::Clock clock;
    bool stepOverridden = false;

    // drive
    std::vector<uint32_t> held;      // global nodes held
    std::vector<uint32_t> heldBody;  // the body of each
    int law = VSIM_DRIVE_HARD;
    double responseTime = vsim::kResponseTime;
    double grabPos[3] = {0, 0, 0}, grabPrev[3] = {0, 0, 0};
    double grabVel[3] = {0, 0, 0};
    bool perBodyGrab = false;        // targets from grabsHost (one row pair per body)
    std::vector<float4> grabsHost;
    std::vector<uint32_t> activeHost;  // 1 where a body takes part in frames
    bool tablesDirty = true;

    // device
    vsim::DeviceState d;
    float4* staging = nullptr;
    uint32_t* pairs = nullptr;
    size_t pairsCapacity = 0;
    unsigned long long* pairCount = nullptr;
    vsim::SplatState sp;
    uint32_t splatCount = 0;
    std::vector<std::vector<float>> splatMeans, splatQuats, splatScales;  // per body, host copies
    vsim::FrameParams fpHost{};
    bool paramsDirty = true, frameDirty = true;
    std::vector<vsim::GraphEntry> graphs;

    // Where each body's items start in the active-node list, in each
    // colour's cell range (relative to the colour's start) and in the
    // surface records; one past the last body closes each list.
    std::vector<uint32_t> nodeBodyStart, recordBodyStart, colourBodyStart[8];
    vsim::FramePlan plan;     // the current frame's spans
    vsim::FramePlan dense;    // every body
    vsim::FramePlan chunked;  // the bodies planBodies listed (fixed grids over the chunk table)
    uint2* chunkDev = nullptr;     // span descriptors, then chunks (Work)
    uint2* chunkPinned = nullptr;  // host staging of the chunk table
    size_t chunkCapacity = 0;      // chunks, not counting the descriptors
    uint32_t* activePinned = nullptr;  // host staging of the activity and drive tables
    float4* grabsPinned = nullptr;
    vsim::TmaPass tma;
    bool quadCells = false;  // small dense colour passes: four lanes a cell (vsim_set_cell_lanes)
};

namespace vsim {

int createSim(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, void* stream, bool isolated,
              vsim_sim* s);
// The TMA brick colour pass (colour_tma.cu): tables built for the
// simulator's bodies (up to kTmaBodies; with more it stays unbuilt), freed,
// and one pass launched.
int buildTmaPass(vsim_sim* s);
void freeTmaPass(TmaPass& t);
cudaError_t launchElasticTma(const LaunchCtx& c, const vsim_sim* s, int colour, const StretchLengths& lens);
// stretch.js:5-7 rest lengths, and whether any body limits its stretch.
StretchLengths stretchLengths();
bool anyStretch(const vsim_sim* s);
void freeSim(vsim_sim* s);
int runFrame(vsim_sim* s, uint32_t steps);
int syncParams(vsim_sim* s);
// Replaces the held set (global nodes, offsets xyz), keeping the hard law's
// prescription in step.
int holdNodes(vsim_sim* s, const uint32_t* nodes, const float* offsets, uint32_t count);
// Node state to the host as xyzw with w = 0 (vsim_read_state's form).
int readNodes(vsim_sim* s, size_t first, size_t count, float* const out[3]);
int releaseNodes(vsim_sim* s);
uint32_t bodyOfNode(const vsim_sim* s, uint32_t node);
Grid bodyGrid(const Lattice& L, const vsim_tank& tank);
// Spans over the listed bodies only (ascending), staged and uploaded on the
// simulator's stream; the next frames run them until useDensePlan.
int planBodies(vsim_sim* s, const std::vector<uint32_t>& bodies);
void useDensePlan(vsim_sim* s);

}  // namespace vsim

#define SIM_GUARD(s)                                                                  \
    if (!(s)) return vsim::fail(VSIM_ERR_INVALID, "simulator handle is NULL");        \
    vsim::DeviceGuard _guard((s)->device);                                            \
    vsim::clearError()
