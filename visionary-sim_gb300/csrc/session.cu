// The session kernel: whole requests of isolated sessions, one launch for
// many sessions, each session's frames run start to finish by one block or
// one cluster of blocks.
//
// The per-pass path (step_kernels.cu) runs a frame as ~141 dependent
// launches over every stepped session at once, so a frame of one small
// session costs as much launch latency as a frame of hundreds. Here a
// session's substep -- prediction, the eight colour passes, the contact
// chain (bin, segments, scatter, order, gather) and the closing pass -- runs
// inside one block (narrow) or one cluster of kSessionCluster blocks (wide),
// with a block or cluster barrier where the per-pass path has a launch
// boundary, for all the frames its request asks for. Sessions never share
// nodes, cells, records or buckets (each has its own contact grid), so the
// blocks of different sessions need no ordering between them, and sessions
// in different launches may run at the same time.
//
// The arithmetic is the per-pass path's (step_device.cuh), item for item:
// a session's result does not depend on which path ran it. Cluster barriers
// are barrier.cluster.arrive.release / wait.acquire, which order every
// global-memory access of the cluster's blocks across the barrier; nothing
// here spins.
#include "step_device.cuh"

namespace vsim {

namespace {

// Not the .aligned form: threads reach it straight from strided loops that
// end at different trip counts.
__device__ __forceinline__ void clusterSync() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ uint32_t clusterRank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The device arrays a session's substeps touch.
struct SessionArrays {
    const FrameParams* fp;
    const DevBody* bodies;
    const uint4* cells;
    const uint32_t* active;
    const int32_t* nodeRecord;
    const float* baseW;
    const uint4* surf;
    float4* pos;
    float4* prev;
    float4* vel;
    uint32_t* key;
    uint32_t* rank;
    uint32_t* entries;
    uint32_t* count;
    uint32_t* start;
    float4* delta;
    SortedEntries sorted;
};

// One job's frames, by `threads` threads numbered `tid`; WIDE: the threads
// of a cluster, else of one block.
template <bool WIDE>
__device__ __forceinline__ void runJob(const SessionJob& job, const SessionLaunch& L, const SessionArrays& a,
                                       uint32_t tid, uint32_t threads, uint32_t* starting) {
    auto sync = [] {
        if (WIDE)
            clusterSync();
        else
            __syncthreads();
    };
    const FrameParams* fp = a.fp;
    const uint32_t body = job.body;
    const CellConsts k = cellConsts(a.bodies + body);
    const float friction = a.bodies[body].friction, damp = a.bodies[body].damp;
    const uint32_t selfContact = fp->selfContact;
    const bool hard = fp->law == VSIM_DRIVE_HARD;
    const bool contact = L.contact && job.recCount > 0;
    const bool limits = L.limited && k.maxStretch > 1.0f;
    const uint32_t lane = threadIdx.x & 31;
    auto noEmit = [](uint32_t, uint32_t) {};
    const ContactArrays ca{a.bodies, a.surf, a.key, a.rank, a.start, a.count, a.sorted.sMeta, a.sorted.sPos,
                           a.sorted.sMoved, a.sorted.sRec, a.sorted.sKey, a.delta};
    // Every index below stays inside the pool's tables only if the job's
    // ranges do and the contact runs add up; the checks record a fault and
    // the job skips the rest of its work (its barriers still run: every
    // block of a cluster meets at each of them whatever it found).
    uint32_t* fault = L.fault + body;
    auto failed = [&] { return *static_cast<volatile uint32_t*>(fault) != kFaultNone; };
    // The hold moves to this request's node (the hard law prescribes a held
    // node by zeroing its inverse mass; a released one gets its own back).
    if (tid == 0) {
        bool inside = uint64_t(job.nodeFirst) + job.nodeCount <= L.activeCount &&
                      uint64_t(job.recFirst) + job.recCount <= L.surfaceCount &&
                      (job.held < 0 || uint32_t(job.held) < L.nodeCount) &&
                      (job.heldBefore < 0 || uint32_t(job.heldBefore) < L.nodeCount) &&
                      (job.held < 0 || uint64_t(job.driveFirst) + job.frames <= L.driveRows);
        for (int c = 0; c < 8; c++) inside = inside && uint64_t(job.cellFirst[c]) + job.cellCount[c] <= L.cellCount;
        *fault = inside ? kFaultNone : kFaultRange;
        if (inside) {
            if (hard && job.heldBefore >= 0 && job.heldBefore != job.held)
                a.pos[job.heldBefore].w = a.baseW[job.heldBefore];
            if (hard && job.held >= 0) a.pos[job.held].w = 0.0f;
        }
        L.cursor[body] = 0;
    }
    sync();
    const uint32_t frames = failed() ? 0u : job.frames;  // read by all after the same barrier
    for (uint32_t f = 0; f < frames; f++) {
        // This frame's drive target and its velocity, read by the thread
        // that handles the held node.
        const float4* row = L.drive + 2 * (size_t(job.driveFirst) + f);
        auto drive = [&](uint32_t n, float4 P) {
            if (int32_t(n) == job.held)
                driveNode(fp, xyz(row[0]), xyz(row[1]), mk(0.0f, 0.0f, 0.0f), n, P, a.pos, a.prev, a.vel);
        };
        for (uint32_t i = tid; i < job.nodeCount; i += threads) {
            const uint32_t n = a.active[job.nodeFirst + i];
            const float4 P = predictNode(fp, n, a.pos, a.prev, a.vel);
            drive(n, P);
        }
        sync();
        for (uint32_t step = 0; step < L.substeps; step++) {
            for (uint32_t it = 0; it < L.iterations; it++)
                for (int c = 0; c < 8; c++) {
                    const uint4* cells = a.cells + job.cellFirst[c];
                    for (uint32_t i = tid; i < job.cellCount[c]; i += threads)
                        solveCellAt<false>(cells[i], k, a.pos, a.prev, L.lens);
                    sync();
                }
            if (limits)
                for (int sweep = 0; sweep < 3; sweep++)
                    for (int c = 0; c < 8; c++) {
                        const uint4* cells = a.cells + job.cellFirst[c];
                        for (uint32_t i = tid; i < job.cellCount[c]; i += threads)
                            solveCellAt<true>(cells[i], k, a.pos, a.prev, L.lens);
                        sync();
                    }
            if (contact) {
                const uint32_t first = job.recFirst, records = job.recCount;
                for (uint32_t i = tid; i < records; i += threads)
                    binRecord(first + i, a.surf[first + i], a.bodies, a.pos, a.key, a.rank, a.count);
                sync();
                // Segments: each occupied bucket's first-arriving record
                // reserves the bucket's run inside the session's records,
                // one atomic per warp.
                for (uint32_t base = tid - lane; base < records; base += threads) {
                    const uint32_t i = base + lane;
                    const uint32_t r = first + i;
                    const bool lead = i < records && a.rank[r] == 0;
                    const uint32_t b = lead ? a.key[r] : 0;
                    const uint32_t need = lead ? a.count[b] : 0;
                    uint32_t incl = need;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
                        if (lane >= uint32_t(d)) incl += v;
                    }
                    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                    uint32_t at = 0;
                    if (lane == 31 && total) at = atomicAdd(&L.cursor[body], total);
                    at = __shfl_sync(0xffffffffu, at, 31);
                    if (lead) {
                        const uint32_t run = first + at + incl - need;
                        a.start[b] = run;
                        if (run - first > records || need > first + records - run) *fault = kFaultRun;
                    }
                }
                sync();
                // The runs must add up to the session's records; checked
                // here, seen by every thread after the scatter's barrier.
                // The scatter guards each of its own writes meanwhile.
                if (tid == 0 && *static_cast<volatile uint32_t*>(L.cursor + body) != records) *fault = kFaultRecords;
                bool ok = !failed();
                for (uint32_t i = tid; ok && i < records; i += threads) {
                    const uint32_t r = first + i;
                    const uint32_t b = a.key[r];
                    const uint32_t at = a.start[b] + a.rank[r];
                    if (a.rank[r] >= a.count[b] || at - first >= records) {
                        *fault = kFaultScatter;
                        continue;
                    }
                    a.entries[at] = r;
                }
                sync();
                ok = !failed();
                for (uint32_t i = tid; ok && i < records; i += threads)
                    canonRecord(first + i, ca, a.entries, a.sorted, a.pos, a.prev);
                sync();
                // The gather over the session's entries in bucket order.
                if (ok && records <= L.warpRecords * (threads >> 5)) {
                    for (uint32_t i = tid >> 5; i < records; i += threads >> 5)
                        collideWarp<false>(first + i, ca, selfContact, starting, noEmit);
                } else if (ok) {
                    for (uint32_t i = tid; i < records; i += threads)
                        collideThread<false>(first + i, ca, selfContact, noEmit);
                }
                sync();
            }
            const bool next = step + 1 < L.substeps;
            const bool settle = contact && !failed();
            for (uint32_t i = tid; i < job.nodeCount; i += threads) {
                const uint32_t n = a.active[job.nodeFirst + i];
                if (settle) {
                    const int32_t record = a.nodeRecord[n];
                    if (next)
                        finalizeNode<true, true>(fp, n, friction, damp, record, a.pos, a.prev, a.vel, a.delta, a.key,
                                                 a.count, drive);
                    else
                        finalizeNode<true, false>(fp, n, friction, damp, record, a.pos, a.prev, a.vel, a.delta,
                                                  a.key, a.count, drive);
                } else if (next) {
                    finalizeNode<false, true>(fp, n, friction, damp, -1, a.pos, a.prev, a.vel, a.delta, a.key,
                                              a.count, drive);
                } else {
                    finalizeNode<false, false>(fp, n, friction, damp, -1, a.pos, a.prev, a.vel, a.delta, a.key,
                                               a.count, drive);
                }
            }
            if (tid == 0) L.cursor[body] = 0;
            sync();
        }
    }
    // Every block's writes are ordered before this thread's by the last
    // barrier; the release at system scope publishes them, and the job's
    // fault, with the ticket.
    if (tid == 0) {
        L.status[body] = *static_cast<volatile uint32_t*>(fault);
        uint32_t* word = L.done + body;
        asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(word), "r"(job.ticket) : "memory");
    }
}

__global__ void __launch_bounds__(kSessionBlock, 2) sessionKernel(SessionLaunch L, SessionArrays a) {
    __shared__ uint32_t runAt[kSessionBlock / 32][32];
    __shared__ SessionJob job;  // indexed by colour at run time: kept out of registers
    uint32_t* starting = runAt[threadIdx.x >> 5];
    const uint32_t rank = clusterRank();
    const SessionGroup& g = L.groups[blockIdx.x / kSessionCluster];
    const bool wide = g.wide != 0;
    // A wide group's job is always real, and every block of the cluster
    // takes part so that all of them meet at every barrier.
    const uint32_t j = wide ? g.job[0] : g.job[rank];
    if (j == kNoJob) return;  // uniform over the block
    // The per-body words are indexed before the job's own checks: a body
    // outside the pool ends the job here, the same way in every block.
    if (L.jobs[j].body >= L.bodyCount) return;
    if (threadIdx.x < sizeof(SessionJob) / 4)
        reinterpret_cast<uint32_t*>(&job)[threadIdx.x] = reinterpret_cast<const uint32_t*>(L.jobs + j)[threadIdx.x];
    __syncthreads();
    if (wide)
        runJob<true>(job, L, a, rank * kSessionBlock + threadIdx.x, kSessionCluster * kSessionBlock, starting);
    else
        runJob<false>(job, L, a, threadIdx.x, kSessionBlock, starting);
}

}  // namespace

cudaError_t launchSessions(cudaStream_t st, const DeviceState& d, uint32_t* entries, const SortedEntries& sorted,
                           const SessionLaunch& L) {
    if (L.groupCount == 0) return cudaSuccess;
    const SessionArrays a{d.fp,  d.bodies, d.cells, d.active, d.nodeRecord, d.baseW, d.surf,  d.pos, d.prev,
                          d.vel, d.key,    d.rank,  entries,  d.count,      d.start, d.delta, sorted};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.groupCount * kSessionCluster);
    cfg.blockDim = dim3(kSessionBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kSessionCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, sessionKernel, L, a);
}

}  // namespace vsim
