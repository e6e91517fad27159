// Internal declarations shared by the host code and the CUDA kernels of
// libvsim. Nothing here is part of the C ABI (that is include/vsim.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/vsim.h"

namespace vsim {

// ---- errors ------------------------------------------------------------

// Records `msg` as this thread's last error and returns `code`.
int fail(int code, const std::string& msg);
void clearError();

// Whether [a, a + n) and [b, b + n) share a 32-bit word.
inline bool wordRangesOverlap(const uint32_t* a, const uint32_t* b, uint32_t n) {
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    const uintptr_t len = uintptr_t(n) * sizeof(uint32_t);
    return x < y + len && y < x + len;
}

// ---- constants of the discretisation ------------------------------------

constexpr uint32_t kBucketSlots = 32;          // contacts.wgsl:75, visible entries per bucket
constexpr double kContactRadiusCells = 0.5;    // voxelLattice.js:17
constexpr double kGridLimit = double(1u << 26);  // buckets before the grid falls back to the bodies' box
constexpr float kResponseTime = 0.05f;         // kinematicDrive.js:65
constexpr uint32_t kMaxStepsPerFrame = 24;     // timestep.js:30
constexpr double kTargetCfl = 0.75;            // timestep.js:17
constexpr double kMaxStepDuration = 1.0 / 240; // timestep.js:23

// ---- material arithmetic (material.js, compliance.js) --------------------

void lame(const vsim_material& m, double& mu, double& lambda);
double waveSpeed(const vsim_material& m);
bool validMaxStretch(double v);
vsim_material defaultMaterial();

// ---- one body's lattice (lattice.js:166-239) ----------------------------

struct Lattice {
    uint32_t cellDims[3] = {0, 0, 0};
    uint32_t nodeDims[3] = {0, 0, 0};
    uint32_t nodeCount = 0;
    double origin[3] = {0, 0, 0};
    double h = 0;
    std::vector<float> rest;        // xyz per node, f32 of origin + i h
    std::vector<float> invMass;     // per node, 0 where no cell touches it
    std::vector<uint32_t> cellsByColor[8];  // linear cell indices, lattice order
    std::vector<uint32_t> surface;  // boundary nodes, ascending (lattice.js:128-158)
    std::vector<uint8_t> occupancy;
    uint32_t cellCount = 0;
};

int buildLattice(const vsim_body_desc& d, Lattice& out);
// The colour of cell (i, j, k) (lattice.js:44-46).
inline int cellColor(uint32_t i, uint32_t j, uint32_t k) { return int((i & 1) | ((j & 1) << 1) | ((k & 1) << 2)); }

// Contact grid layout (broadphase.js:46-58), with the fallback for an
// unbounded or oversized tank: the bodies' rest box padded by half its extent
// (at least four buckets) per side, clipped to the tank.
struct Grid {
    double origin[3];
    double bucket;
    uint32_t dims[3];
    uint64_t count() const { return uint64_t(dims[0]) * dims[1] * dims[2]; }
};
Grid contactGrid(const vsim_tank& tank, double widestRadius, const double lo[3], const double hi[3]);

// ---- fixed timestep clock (timestep.js:56-180) --------------------------

struct Clock {
    double stepDuration = kMaxStepDuration;
    uint32_t maxStepsPerFrame = kMaxStepsPerFrame;
    double accumulator = 0, simulatedTime = 0, droppedTime = 0, lastElapsed = 0, lastDroppedTime = 0;
    uint64_t totalSteps = 0;
    uint32_t lastSteps = 0;
    void reset();
    void consume(double elapsed, bool forceStep);
    void idle();
    void singleStep();
    vsim_clock_report snapshot() const;
};
double stableStepDuration(double waveRate);  // caller validates the rate

// ---- device-side records ------------------------------------------------

// Per-body constants the kernels read, rewritten when the step duration or a
// material changes. The elastic fields are the f32 values project.wgsl:64-73
// derives per thread, derived once here in the same order.
struct DevBody {
    uint32_t nodeOffset;
    uint32_t nx;      // node stride along y
    uint32_t nxy;     // node stride along z
    uint32_t pad0;
    float alphaDev;   // alphaDev / dt^2
    float alphaHyd;   // alphaHyd / dt^2
    float gamma;
    float relax;      // relaxation / dt
    float restScale;  // 1 / h
    float h;
    float maxStretch;
    float friction;
    float damp;       // exp(-damping dt), finalize.wgsl:72
    float pad1, pad2, pad3;
    // The contact grid this body bins into (contacts.wgsl:84-91): shared by
    // every body of a scene, or the body's own when bodies must never meet.
    float gridOrigin[3];
    float bucket;
    uint32_t gridDims[3];
    uint32_t gridBase;  // index of the grid's first bucket in the bucket arrays
    // Reciprocals for dividing a bucket's linear index by dims[0] and by
    // dims[0] * dims[1]: floor(2^64 / d) + 1, exact for 32-bit numerators
    // (0 stands for d = 1).
    uint64_t divX, divXY;
};
static_assert(sizeof(DevBody) == 112, "DevBody is one 112-byte record");

// floor(2^64 / d) + 1 for a 32-bit divisor d > 1, 0 for d = 1: with it,
// n / d = high 64 bits of n * m for every 32-bit n (Lemire, Kaser and
// Kurz, "Faster remainder by direct computation", 2019).
inline uint64_t reciprocal64(uint32_t d) { return d > 1 ? ~uint64_t(0) / d + 1 : 0; }

// Scalars every substep kernel reads, refreshed by one small copy per frame.
struct FrameParams {
    float dt;
    float gx, gy, gz;
    float tankMin[3];
    float invDt2;
    float tankMax[3];
    float responseTime;
    float grabTarget[3];
    uint32_t drivenCount;
    float grabVelocity[3];
    uint32_t law;
    uint32_t surfaceCount;
    uint32_t selfContact;
    uint32_t activeCount;
    uint32_t perBodyGrab;  // drive targets come from the per-body table, not grabTarget
};

}  // namespace vsim
