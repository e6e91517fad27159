// Declarations shared between the kernel files and the simulator object.
#pragma once

#include <cuda_runtime.h>

#include "vmath.cuh"
#include "vsim_internal.h"

namespace vsim {

// Device buffers of one simulator, as the kernels see them.
struct DeviceState {
    float4* pos = nullptr;        // xyz position, w = inverse mass the solver uses
    float4* prev = nullptr;       // position at the start of the substep
    float4* vel = nullptr;
    float* baseW = nullptr;       // material inverse mass with static nodes zeroed
    uint32_t* active = nullptr;   // nodes with material (predict and finalize visit these)
    uint32_t* activeBody = nullptr;
    int32_t* nodeRecord = nullptr;  // surface record of each node, -1 for none
    uint32_t* bodyActive = nullptr;  // 1 where a body takes part in this frame
    float4* grabs = nullptr;      // per body: drive target, drive target velocity
    uint4* cells = nullptr;       // colour-major (corner-0 node, body, y stride, z stride)
    DevBody* bodies = nullptr;
    FrameParams* fp = nullptr;
    // contact
    uint4* surf = nullptr;        // (node, body, packed rest coords, radius bits)
    uint32_t* key = nullptr;
    uint32_t* rank = nullptr;
    uint32_t* entries = nullptr;
    uint32_t* count = nullptr;    // per bucket
    uint32_t* start = nullptr;    // per bucket
    uint32_t* cursor = nullptr;
    float4* delta = nullptr;
    uint4* sMeta = nullptr;       // every bucket entry in bucket order (visible prefix first): its record
    float4* sPos = nullptr;       //   ... its node's position
    float4* sMoved = nullptr;     //   ... its motion over the substep, its body's friction
    uint32_t* sRec = nullptr;     //   ... its record index
    uint32_t* sKey = nullptr;     //   ... its bucket
    // drive
    uint32_t* driven = nullptr;
    float4* drivenOffset = nullptr;
    int32_t* drivenOf = nullptr;  // per node: its row in driven[], -1 for none
};

struct LaunchCtx {
    cudaStream_t stream;
    bool pdl;
    uint32_t sms;            // multiprocessors of the device
    bool quadCells = false;  // small dense colour passes split each cell over four lanes
};

// The items one launch covers. Dense (`table` null): [0, count), one thread
// each. Chunked: `table[span]` = (first chunk, chunk count) of this launch,
// and `table[kSpans + first + c]` = (first item, item count <= kChunk) --
// the ranges of the bodies a frame steps, so idle bodies cost no threads.
// Blocks of kChunk threads take the chunks in turn, so a fixed grid covers
// any set of bodies and the launch can be captured once in a graph.
struct Work {
    const uint2* table;
    uint32_t span;
    uint32_t count;
};

// Spans of a frame: the active nodes, the eight colours' cells, the surface
// records.
constexpr uint32_t kSpans = 10;
constexpr uint32_t kNodeSpan = 0, kRecordSpan = 9;
constexpr uint32_t colourSpan(int c) { return 1 + uint32_t(c); }

// Calls f(item) for each item of `w` this thread owns.
template <class F>
__device__ __forceinline__ void forEachItem(const Work& w, F&& f) {
    if (!w.table) {
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < w.count) f(i);
        return;
    }
    const uint2 d = w.table[w.span];
    for (uint32_t c = blockIdx.x; c < d.y; c += gridDim.x) {
        const uint2 chunk = w.table[kSpans + d.x + c];
        if (threadIdx.x < chunk.y) f(chunk.x + threadIdx.x);
    }
}

// As forEachItem, with the kernel's programmatic-launch wait inside. pre(item)
// may read only what no kernel of the frame writes -- the cell and record
// tables, body constants, activity flags, the chunk table, all uploaded by
// copies before the frame's first kernel -- and runs before the wait for the
// thread's first item, so those loads overlap the previous kernel's tail;
// body(item, pre(item)) runs after it.
template <class Pre, class Body>
__device__ __forceinline__ void forEachItemAfterWait(const Work& w, Pre&& pre, Body&& body) {
    using P = decltype(pre(0u));
    if (!w.table) {
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        const bool has = i < w.count;
        P first{};
        if (has) first = pre(i);
        pdlWait();
        pdlLaunchNext();
        if (has) body(i, first);
        return;
    }
    const uint2 d = w.table[w.span];
    uint32_t c = blockIdx.x;
    bool has = false;
    uint32_t item = 0;
    P first{};
    if (c < d.y) {
        const uint2 chunk = w.table[kSpans + d.x + c];
        has = threadIdx.x < chunk.y;
        item = chunk.x + threadIdx.x;
        if (has) first = pre(item);
    }
    pdlWait();
    pdlLaunchNext();
    if (has) body(item, first);
    for (c += gridDim.x; c < d.y; c += gridDim.x) {
        const uint2 chunk = w.table[kSpans + d.x + c];
        if (threadIdx.x < chunk.y) body(chunk.x + threadIdx.x, pre(chunk.x + threadIdx.x));
    }
}

// As forEachItem, but every thread of the block calls f(has, item) the same
// number of times (for block-wide scans); `has` says whether `item` is real.
template <class F>
__device__ __forceinline__ void forEachItemUniform(const Work& w, F&& f) {
    if (!w.table) {
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        f(i < w.count, i);
        return;
    }
    const uint2 d = w.table[w.span];
    for (uint32_t c = blockIdx.x; c < d.y; c += gridDim.x) {
        const uint2 chunk = w.table[kSpans + d.x + c];
        f(threadIdx.x < chunk.y, chunk.x + threadIdx.x);
    }
}

// One launch: its work, grid and block.
struct Span {
    Work work;
    uint32_t grid;
    uint32_t block;
    // Records spans over chunk tables: blocks an SM of the contact gather.
    uint32_t gatherPerSm = 64;
};

// Chunks of at most kChunk items per block.
constexpr uint32_t kChunk = 128;

// Rest lengths of the cube's edges, face and body diagonals (stretch.js:5-7),
// as f32; indexed by the number of axes the two corners differ in, minus one.
struct StretchLengths {
    float len[3];
};

enum class ContactMode { Solve, Pairs };

void kuhnTable(float out[54]);

// Dense spans: `count` items, blocks of `block` threads.
Span denseSpan(uint32_t count, uint32_t block);
// A colour pass's span over `count` cells: blocks shrink for small passes
// so that every SM gets a share.
Span elasticSpan(uint32_t count, uint32_t block, uint32_t sms);

// Prediction of the frame's first substep; with `drive` the driven nodes
// then take the drive law (driveHard/driveCompliant.wgsl), the substep's
// first constraint.
cudaError_t launchPredict(const LaunchCtx& c, const DeviceState& s, const Span& nodes, bool drive);
// drivenOf[driven[i]] := i for the n driven records, or := -1 with `clear`.
cudaError_t launchMarkDriven(cudaStream_t st, const uint32_t* driven, uint32_t n, int32_t* drivenOf, bool clear);
cudaError_t launchElastic(const LaunchCtx& c, const DeviceState& s, const uint4* cells, const Span& span,
                          bool limitOnly, const StretchLengths& lens);

// The streaming colour pass (elasticStreamKernel): blocks of kStreamBlock
// threads, kStreamBlocksPerSm of them per SM (what the ~127 registers of a
// cell allow). A dense pass of at least two cells per resident thread
// streams.
constexpr uint32_t kStreamBlock = 128;
constexpr uint32_t kStreamBlocksPerSm = 4;
inline bool streamsColourPass(uint32_t count, uint32_t sms) {
    return count >= 2 * kStreamBlocksPerSm * sms * kStreamBlock;
}

// The substep's closing pass; with `contact` it first applies the contact
// corrections and empties the grid, with `predictNext` it goes on into the
// next substep's prediction (and, with `drive`, its drive).
cudaError_t launchFinalize(const LaunchCtx& c, const DeviceState& s, const Span& nodes, bool contact,
                           bool predictNext, bool drive);
// `records` covers the surface records of the stepped bodies; at most
// `recordItems` of them are binned. `mapping` is a VSIM_GATHER_* value.
// `marks`, when given, are six events recorded around the five kernels (before
// bin, between each, after the gather).
cudaError_t launchContact(const LaunchCtx& c, const DeviceState& s, const Span& records, uint32_t recordItems,
                          int mapping, ContactMode mode, uint32_t* pairs, uint32_t capacity,
                          unsigned long long* pairCount, cudaEvent_t* marks = nullptr);
// After a Solve-mode contact chain: counts the gather's work on the grid it
// built (out[0] live records, out[1] visible candidates, out[2] occupied
// buckets; added to) and empties the grid without applying corrections.
cudaError_t launchCensus(const LaunchCtx& c, const DeviceState& s, const Span& records, unsigned long long* out);
cudaError_t launchRestoreW(cudaStream_t st, const uint32_t* nodes, uint32_t n, const float* base, float4* pos);
cudaError_t launchZeroW(cudaStream_t st, const uint32_t* nodes, uint32_t n, float4* pos);
cudaError_t launchRefreshW(cudaStream_t st, uint32_t first, uint32_t n, const float* base, float4* pos);
cudaError_t launchMergeXyz(cudaStream_t st, const float4* in, uint32_t n, float4* pos);
cudaError_t launchDropW(cudaStream_t st, const float4* in, uint32_t n, float4* out);

// Every contact entry in bucket order as canonRecord lays them out: its
// record, its node's position, its motion over the substep with its body's
// friction, its record index and its bucket.
struct SortedEntries {
    uint4* sMeta;
    float4* sPos;
    float4* sMoved;
    uint32_t* sRec;
    uint32_t* sKey;
};

// ---- TMA brick colour pass (colour_tma.cu) -----------------------------------

constexpr uint32_t kTmaBodies = 4;   // bodies whose node arrays get tensor maps
constexpr uint32_t kTmaBlock = 128;  // threads: one per cell of an 8 x 4 x 4 brick

// The pass's tables: per colour, the bricks holding its cells (two uint4
// each: body and brick coordinates, then 128 occupancy bits).
struct TmaPass {
    bool ready = false;    // built for the simulator's current arrays
    bool enabled = false;  // large dense passes use it (vsim_set_tma_pass)
    void* maps = nullptr;  // host: the bodies' position and previous-position tensor maps
    uint4* bricks = nullptr;
    uint32_t first[8] = {}, count[8] = {};
    uint32_t* fault = nullptr;  // set by a block whose copies did not arrive
};

// ---- session kernel (session.cu) -------------------------------------------

// One request of an isolated session: its body's ranges and the frames to
// run.
struct SessionJob {
    uint32_t nodeFirst, nodeCount;  // its range of the active-node list
    uint32_t recFirst, recCount;    // its range of the surface records
    uint32_t cellFirst[8];          // per colour: its first cell in the cell list
    uint32_t cellCount[8];
    uint32_t body;
    uint32_t frames;
    int32_t heldBefore;             // global node the session held until now, -1 for none
    int32_t held;                   // global node this request holds, -1 for none
    uint32_t driveFirst;            // its first frame's row pair in the drive table
    uint32_t ticket;                // written to done[body] when the request has run
    uint32_t pad[2];
};

constexpr uint32_t kSessionCluster = 8;   // blocks of a cluster
constexpr uint32_t kSessionBlock = 256;   // threads of a block
constexpr uint32_t kNoJob = 0xffffffffu;
// Largest colour (cells) of a session the serving engine runs in one block
// by default: above it a session's substep -- mostly its contact gather,
// ~10^5 warp instructions once it has settled -- issues faster on more
// SMs. Up to kDefaultClusterCells it runs on a cluster of eight blocks,
// which costs about the SM time of a tick but no tick's wait; larger
// sessions run as ticks, whose launches spread them over every SM.
constexpr uint32_t kDefaultBlockCells = 32;
constexpr uint32_t kDefaultClusterCells = 512;

// Checks a job can fail (SessionLaunch::fault, ::status). A failed job
// skips the rest of its work; the host reports it as an error.
enum SessionFault : uint32_t {
    kFaultNone = 0,
    kFaultRange = 1,    // a range of the job outside the pool's tables
    kFaultRecords = 2,  // the buckets' runs do not add up to the session's records
    kFaultRun = 3,      // a bucket's run outside the session's records
    kFaultScatter = 4,  // a record's place outside its bucket's run
};

// A cluster's work: one wide job run by all its blocks, or up to
// kSessionCluster narrow jobs, one per block (kNoJob: none).
struct SessionGroup {
    uint32_t wide;
    uint32_t job[kSessionCluster];
};

struct SessionLaunch {
    const SessionGroup* groups;
    uint32_t groupCount;
    const SessionJob* jobs;
    const float4* drive;   // per frame of a dragging job: target, target velocity
    uint32_t* cursor;      // per body: segment cursor of its records
    uint32_t* fault;       // per body, device: the check the running job failed, 0 for none
    uint32_t* done;        // per body: ticket of its last request run (host-mapped)
    uint32_t* status;      // per body: its last job's fault, written before the ticket (host-mapped)
    // What the jobs' ranges are checked against.
    uint32_t activeCount, cellCount, surfaceCount, nodeCount, bodyCount, driveRows;
    uint32_t substeps;
    uint32_t iterations;
    uint32_t limited;      // any body has a stretch limit
    uint32_t contact;
    uint32_t warpRecords;  // the gather takes a warp per record while records <= warpRecords x warps
    StretchLengths lens;
};

// `entries` and `sorted` are the session engine's own bucket-order arrays
// (a job lays its runs out inside its session's record range, while a
// tick running at the same time packs its runs from position 0 of the
// simulator's).
cudaError_t launchSessions(cudaStream_t st, const DeviceState& d, uint32_t* entries, const SortedEntries& sorted,
                           const SessionLaunch& L);

// ---- splats ---------------------------------------------------------------

struct SplatBody {
    uint32_t nx, nxy;
    float inv;  // 1 / h
    uint32_t pad;
};

struct SplatState {
    float4* embed = nullptr;    // (u, v, w local coordinates, corner-0 node as bits)
    float4* quat = nullptr;     // xyzw
    float4* scaleBody = nullptr;  // (sx, sy, sz, body as bits)
    SplatBody* bodies = nullptr;
    float4* meanDepth = nullptr;  // deformed mean, depth along the view
    float2* cov = nullptr;        // 3 x float2 per splat: (xx, xy), (xz, yy), (yz, zz)
    uint32_t* keys = nullptr;
    uint32_t* order = nullptr;
    void* sortTemp = nullptr;
    size_t sortTempBytes = 0;
    float4* axesRotation = nullptr;  // per splat: the deformed ellipsoid's unit quaternion xyzw
    float4* axesScale = nullptr;     //   ... and its axis lengths xyz (allocated on first use)
};

// With `axes` the deformation also takes each covariance apart into a
// rotation and axis lengths (s.axesRotation, s.axesScale).
cudaError_t launchSplatDeform(cudaStream_t st, const SplatState& s, const float4* pos, uint32_t n, float vx, float vy,
                              float vz, bool axes = false);

// ---- radix sort -------------------------------------------------------------

size_t radixSortTempBytes(uint32_t n);
// Kernels one radixSortU32 call launches.
uint32_t radixSortLaunches(uint32_t n, uint32_t keyBits);
cudaError_t radixSortU32(const uint32_t* keys, uint32_t* order, uint32_t n, uint32_t keyBits, void* temp,
                         size_t tempBytes, cudaStream_t st);

}  // namespace vsim
