// The substep kernels of the solver: prediction, the kinematic drive, the
// 8-colour stable Neo-Hookean projection, body contact and the closing pass.
//
// Node state lives in HBM as three float4 arrays in the reference's dense
// node order (pos, prev, vel; state.wgsl:16-19). pos.w carries the node's
// inverse mass as the solver sees it (the reference's separate nodeInvMass
// buffer, particles.js:206-215), so one 16-byte load brings a node's
// position and weight together; every kernel that writes pos keeps w.
#include "step_device.cuh"

namespace vsim {

void kuhnTable(float out[54]) {
    for (int t = 0; t < 6; t++)
        for (int col = 0; col < 3; col++)
            for (int row = 0; row < 3; row++) out[t * 9 + col * 3 + row] = float(kKuhn.v[t][col][row]);
}


// ------------------------------------------------------------- kernels --

// predict.wgsl:19-36 over the active nodes; with DRIVE, a driven node then
// takes the drive law (the reference's next pass in the substep).
template <bool DRIVE>
__global__ void predictKernel(const FrameParams* __restrict__ fp, Work work, const uint32_t* __restrict__ active,
                              const uint32_t* __restrict__ activeBody, const uint32_t* __restrict__ bodyActive,
                              DriveTables drive, float4* __restrict__ pos, float4* __restrict__ prev,
                              float4* __restrict__ vel) {
    struct Pre {
        uint32_t n, live;
        int32_t driven;
    };
    auto pre = [&](uint32_t i) {
        const uint32_t n = active[i];
        return Pre{n, bodyActive[activeBody[i]], DRIVE ? drive.drivenOf[n] : -1};
    };
    forEachItemAfterWait(work, pre, [&](uint32_t i, Pre q) {
        if (!q.live) return;
        const float4 P = predictNode(fp, q.n, pos, prev, vel);
        if (DRIVE && q.driven >= 0) applyDrive(fp, drive.offsets, drive.grabs, q.driven, q.n, P, pos, prev, vel);
    });
}

// Marks (or, with row < 0, clears) the driven nodes' rows in drivenOf.
__global__ void markDrivenKernel(const uint32_t* __restrict__ driven, uint32_t n, int32_t* __restrict__ drivenOf,
                                 int clear) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) drivenOf[driven[i]] = clear ? -1 : int32_t(i);
}

// project.wgsl:35-184: one colour pass, one thread per occupied cell.
// `cells` holds (global node of corner 0, body, node stride along y, along z)
// per cell of this colour, so the corner loads wait on one load only.
template <bool LIMIT_ONLY>
__global__ void __launch_bounds__(512) elasticKernel(const uint4* __restrict__ cells, Work work,
                                                     const DevBody* __restrict__ bodies,
                                                     const uint32_t* __restrict__ bodyActive, float4* __restrict__ pos,
                                                     const float4* __restrict__ prevState, StretchLengths lens) {
    struct Pre {
        uint4 entry;
        uint32_t live;
        CellConsts k;
    };
    auto pre = [&](uint32_t slot) {
        const uint4 entry = cells[slot];
        return Pre{entry, bodyActive[entry.y], cellConsts(bodies + entry.y)};
    };
    forEachItemAfterWait(work, pre, [&](uint32_t, const Pre& q) {
        if (!q.live) return;
        if (LIMIT_ONLY && !(q.k.maxStretch > 1.0f)) return;
        solveCellAt<LIMIT_ONLY>(q.entry, q.k, pos, prevState, lens);
    });
}

// The colour pass with each cell split over the four lanes of a quad
// (solveCellQuad): four times the threads of elasticKernel, each running
// the spine of the cell's chain and a quarter of its per-corner work. Dense
// passes only (the cell list, not a chunk table); every lane loads the
// cell, lane q stores corners q and q + 4.
__global__ void __launch_bounds__(128) elasticQuadKernel(const uint4* __restrict__ cells, uint32_t count,
                                                         const DevBody* __restrict__ bodies,
                                                         const uint32_t* __restrict__ bodyActive,
                                                         float4* __restrict__ pos,
                                                         const float4* __restrict__ prevState, StretchLengths lens) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t slot = t >> 2, q = t & 3;
    const uint32_t quad = 0xfu << (threadIdx.x & 28u);
    const bool has = slot < count;
    uint4 entry = make_uint4(0, 0, 0, 0);
    uint32_t live = 0;
    CellConsts k{};
    if (has) {
        entry = cells[slot];
        live = bodyActive[entry.y];
        k = cellConsts(bodies + entry.y);
    }
    pdlWait();
    pdlLaunchNext();
    if (!has || !live) return;  // the whole quad: its lanes share the cell
    uint32_t ids[8];
    cornerNodes(entry, ids);
    V p[8], prev[8];
    float w[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float4 P = pos[ids[c]];
        p[c] = xyz(P);
        w[c] = P.w;
    }
#pragma unroll
    for (int c = 0; c < 8; c++) prev[c] = xyz(prevState[ids[c]]);
    solveCellQuad(p, prev, w, k, lens, q, quad);
#pragma unroll
    for (int c = 0; c < 8; c++)
        if ((c & 3) == int(q)) pos[ids[c]] = withW(p[c], w[c]);
}

// The colour pass for passes much larger than the GPU: each thread solves
// cells in turn (grid-stride) and copies the next cell's eight positions and
// eight previous positions into its slots of shared memory (cp.async) while
// it solves the current one, so the gathers' latency hides behind the
// arithmetic instead of stalling the warp. Cells of one colour share no
// node, so reading ahead is safe. Same arithmetic as elasticKernel.

__device__ __forceinline__ void copyAsync16(float4* dst, const float4* src) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

__global__ void __launch_bounds__(kStreamBlock) elasticStreamKernel(const uint4* __restrict__ cells, uint32_t count,
                                                                    const DevBody* __restrict__ bodies,
                                                                    const uint32_t* __restrict__ bodyActive,
                                                                    float4* __restrict__ pos,
                                                                    const float4* __restrict__ prevState,
                                                                    StretchLengths lens) {
    __shared__ float4 stage[16][kStreamBlock];  // [corner] pos, [8 + corner] prev
    const uint32_t t = threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t slot = blockIdx.x * blockDim.x + t;
    uint4 entry = slot < count ? cells[slot] : make_uint4(0, 0, 0, 0);  // frame constants: before the wait
    pdlWait();
    pdlLaunchNext();
    if (slot >= count) return;
    // Copies cell `e`'s nodes into the stage; `after` (zero, computed from the
    // values just read out of the stage) orders the copies after those reads.
    auto fetch = [&](uint4 e, uint32_t after) {
        const uint32_t nx = e.z, nxy = e.w, n0 = e.x + after;
        const uint32_t ids[8] = {n0,       n0 + 1,       n0 + nx,       n0 + nx + 1,
                                 n0 + nxy, n0 + nxy + 1, n0 + nxy + nx, n0 + nxy + nx + 1};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            copyAsync16(&stage[c][t], pos + ids[c]);
            copyAsync16(&stage[8 + c][t], prevState + ids[c]);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    fetch(entry, 0);
    while (true) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        V p[8], prev[8];
        float w[8];
        uint32_t bits = 0;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float4 P = stage[c][t];
            const float4 Q = stage[8 + c][t];
            p[c] = xyz(P);
            w[c] = P.w;
            prev[c] = xyz(Q);
            // One word of each 16-byte read is enough: a read's registers
            // are written together.
            bits ^= __float_as_uint(P.w) ^ __float_as_uint(Q.x);
        }
        uint32_t zero;
        asm volatile("and.b32 %0, %1, 0;" : "=r"(zero) : "r"(bits));
        const uint4 cur = entry;
        const uint32_t next = slot + stride;
        if (next < count) {
            entry = cells[next];
            fetch(entry, zero);
        }
        if (bodyActive[cur.y]) {
            solveCell<false>(p, prev, w, cellConsts(bodies + cur.y), lens);
            uint32_t ids[8];
            cornerNodes(cur, ids);
#pragma unroll
            for (int c = 0; c < 8; c++) pos[ids[c]] = withW(p[c], w[c]);
        }
        if (next >= count) break;
        slot = next;
    }
}

// finalize.wgsl:44-74 over the active nodes; the velocity factor
// exp(-damping dt) is the body's, evaluated once on the host.
//
// With CONTACT the pass first does what settle.wgsl:20-36 does for a node
// with a surface record -- apply its averaged contact correction, empty its
// bucket -- so no separate pass runs between contact and the closing pass.
// With PREDICT it continues straight into the next substep's
// predict.wgsl:19-36 from the position and velocity it has just computed,
// which are the values that pass would read back; with DRIVE as well a
// driven node then takes the drive law, that substep's first constraint.
template <bool CONTACT, bool PREDICT, bool DRIVE>
__global__ void finalizeKernel(const FrameParams* __restrict__ fp, Work work, const uint32_t* __restrict__ active,
                               const uint32_t* __restrict__ activeBody, const DevBody* __restrict__ bodies,
                               float4* __restrict__ pos, float4* __restrict__ prevState, float4* __restrict__ vel,
                               const int32_t* __restrict__ nodeRecord, const float4* __restrict__ delta,
                               const uint32_t* __restrict__ key, uint32_t* __restrict__ count,
                               uint32_t* __restrict__ cursor, const uint32_t* __restrict__ bodyActive,
                               DriveTables drive) {
    struct Pre {
        uint32_t n, live;
        int32_t record, driven;
        float friction, damp;
    };
    auto pre = [&](uint32_t i) {
        const uint32_t body = activeBody[i];
        const uint32_t n = active[i];
        return Pre{n, bodyActive[body], CONTACT ? nodeRecord[n] : -1, DRIVE ? drive.drivenOf[n] : -1,
                   bodies[body].friction, bodies[body].damp};
    };
    forEachItemAfterWait(work, pre, [&](uint32_t, const Pre& q) {
        if (!q.live) return;
        finalizeNode<CONTACT, PREDICT>(fp, q.n, q.friction, q.damp, q.record, pos, prevState, vel, delta, key, count,
                                       [&](uint32_t n, float4 P) {
                                           if (DRIVE && q.driven >= 0)
                                               applyDrive(fp, drive.offsets, drive.grabs, q.driven, n, P, pos,
                                                          prevState, vel);
                                       });
    });
    // After the wait (inside the loop above): the gather has read it.
    if (CONTACT && blockIdx.x == 0 && threadIdx.x == 0) *cursor = 0;
}

// ------------------------------------------------------------- contact --
//
// The reference bins every surface record into a fixed 32-slot bucket with
// an atomic, then canonicalises each bucket by an insertion sort
// (bin.wgsl, sort.wgsl). Here the grid is a counting sort: per-bucket
// counts with the arrival rank of each record, one contiguous segment
// allocated per occupied bucket, a scatter, and an ascending sort of each
// segment's first 32 entries -- the same visible set, in the same order, with
// work proportional to the surface rather than to the grid.

__global__ void binKernel(const FrameParams* __restrict__ fp, Work work, const uint4* __restrict__ surf,
                          const DevBody* __restrict__ bodies, const uint32_t* __restrict__ bodyActive,
                          const float4* __restrict__ pos, uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                          uint32_t* __restrict__ count) {
    struct Pre {
        uint4 rec;
        uint32_t live;
    };
    auto pre = [&](uint32_t r) {
        const uint4 rec = surf[r];
        return Pre{rec, bodyActive[rec.y]};
    };
    forEachItemAfterWait(work, pre, [&](uint32_t r, const Pre& q) {
        const uint4 rec = q.rec;
        if (!q.live) {
            key[r] = kIdle;
            rank[r] = kIdle;
            return;
        }
        binRecord(r, rec, bodies, pos, key, rank, count);
    });
}

// Each bucket's first-arriving record reserves the bucket's segment; one
// atomic per block on the shared cursor.
__global__ void allocKernel(const FrameParams* __restrict__ fp, Work work, const uint32_t* __restrict__ key,
                            const uint32_t* __restrict__ rank, const uint32_t* __restrict__ count,
                            uint32_t* __restrict__ start, uint32_t* __restrict__ cursor) {
    pdlWait();
    pdlLaunchNext();
    __shared__ uint32_t warpSum[32];
    __shared__ uint32_t blockBase;
    forEachItemUniform(work, [&](bool has, uint32_t r) {
        const bool first = has && rank[r] == 0;
        const uint32_t b = first ? key[r] : 0;
        const uint32_t need = first ? count[b] : 0;
        // Block-wide exclusive prefix of `need`.
        const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = need;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= uint32_t(d)) incl += v;
        }
        if (lane == 31) warpSum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t nw = blockDim.x >> 5;
            uint32_t v = lane < nw ? warpSum[lane] : 0;
            uint32_t scan = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, scan, d);
                if (lane >= uint32_t(d)) scan += u;
            }
            if (lane < nw) warpSum[lane] = scan - v;
            if (lane == nw - 1) blockBase = scan > 0 ? atomicAdd(cursor, scan) : 0;
        }
        __syncthreads();
        if (first) start[b] = blockBase + warpSum[warp] + (incl - need);
        __syncthreads();  // warpSum and blockBase are rewritten by the next chunk
    });
}

__global__ void scatterKernel(const FrameParams* __restrict__ fp, Work work, const uint32_t* __restrict__ key,
                              const uint32_t* __restrict__ rank, const uint32_t* __restrict__ start,
                              uint32_t* __restrict__ entries) {
    pdlWait();
    pdlLaunchNext();
    forEachItem(work, [&](uint32_t r) {
        if (key[r] == kIdle) return;
        entries[start[key[r]] + rank[r]] = r;
    });
}

// sort.wgsl:14-53: the bucket's visible entries -- its kBucketSlots lowest
// record indices -- in ascending order at the front of its segment, the
// rest after them; every entry's record, position, motion over the substep
// (position - its substep start, as collide.wgsl:100-101 subtracts them)
// with its body's friction, record index and bucket copied out in that
// order, so the gather reads each neighbour bucket's visible entries as one
// contiguous run and both a record's own data and a candidate's one load
// deep.
//
// A bucket of at most kBucketSlots entries is all visible: each of its
// records finds its own place (how many of the bucket's records have a lower
// index) and copies itself there, all records at once. A larger bucket is
// ordered by its first-arriving record alone, an insertion sort that keeps
// the lowest kBucketSlots in front (rare: 32 surface nodes in one bucket of
// edge h).
__global__ void canonKernel(const FrameParams* __restrict__ fp, Work work, const uint32_t* __restrict__ key,
                            const uint32_t* __restrict__ rank, const uint32_t* __restrict__ start,
                            const uint32_t* __restrict__ count, uint32_t* __restrict__ entries,
                            const uint4* __restrict__ surf, const float4* __restrict__ pos,
                            const float4* __restrict__ prevState, const DevBody* __restrict__ bodies,
                            uint4* __restrict__ sMeta, float4* __restrict__ sPos, float4* __restrict__ sMoved,
                            uint32_t* __restrict__ sRec, uint32_t* __restrict__ sKey) {
    pdlWait();
    pdlLaunchNext();
    const ContactArrays arrays{bodies, surf, key, rank, start, count, nullptr, nullptr, nullptr, nullptr, nullptr,
                               nullptr};
    const SortedEntries out{sMeta, sPos, sMoved, sRec, sKey};
    forEachItem(work, [&](uint32_t r) {
        if (key[r] == kIdle) return;
        canonRecord(r, arrays, entries, out, pos, prevState);
    });
}

// collide.wgsl:16-125, reading each neighbour bucket's visible entries as
// the contiguous run canonKernel laid out. With EMIT, every counted hit
// (r, other) is also appended to `pairs` (capacity-checked), for the
// pair-set checks.
//
// Records are taken in bucket order (the counting sort's output as canonKernel
// copied it, `*cursor` long), so neighbouring records read the same runs.
// Two mappings
// of records to threads, chosen per launch from the number of records:
//
// - few records (below `warpModeBelow`): one warp per record. The record's
//   candidates -- the visible entries of its 27 neighbour buckets,
//   concatenated in the reference's order (buckets dz, dy, dx; entries in
//   bucket order) -- are dealt to the lanes 32 at a time: lane q < 27 sizes
//   neighbour bucket q, a warp scan turns the sizes into offsets, and each
//   lane finds its candidate's run as the last one starting at or before it
//   (a ballot of the runs starting in the round, the run carried over from
//   the round before). The record's chain of
//   dependent candidate loads is spread over 32 lanes, which is what a
//   launch too small to fill the GPU needs;
// - many records: one thread per record, scanning the runs itself, which
//   costs fewer instructions per record once the GPU is full anyway.
//
// Either way each record's hits are added to its sum one at a time in
// candidate order, so both give the sequential result.

template <bool EMIT>
__global__ void __launch_bounds__(kCollideBlock, 5) collideKernel(
    const FrameParams* __restrict__ fp, uint32_t items, uint32_t warpModeBelow, const uint32_t* __restrict__ cursor,
    const DevBody* __restrict__ bodies, const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
    const uint4* __restrict__ sMeta, const float4* __restrict__ sPos, const float4* __restrict__ sMoved,
    const uint32_t* __restrict__ sRec, const uint32_t* __restrict__ sKey, float4* __restrict__ delta,
    uint32_t* __restrict__ pairs, uint32_t capacity, unsigned long long* __restrict__ pairCount) {
    pdlWait();
    pdlLaunchNext();
    const uint32_t total = min(items, *cursor);
    const uint32_t selfContact = fp->selfContact;
    const uint32_t thread = blockIdx.x * blockDim.x + threadIdx.x;
    const ContactArrays arrays{bodies, nullptr, nullptr, nullptr, start, count, sMeta, sPos, sMoved, sRec, sKey, delta};
    auto emit = [&](uint32_t r, uint32_t at) {
        const unsigned long long slot = atomicAdd(pairCount, 1ull);
        if (slot < capacity) {
            pairs[2 * slot] = r;
            pairs[2 * slot + 1] = sRec[at];
        }
    };
    if (total >= warpModeBelow) {
        for (uint32_t i = thread; i < total; i += gridDim.x * blockDim.x)
            collideThread<EMIT>(i, arrays, selfContact, emit);
        return;
    }
    // Per warp: the neighbour bucket (lane) whose run starts at each
    // candidate position of the current round.
    __shared__ uint32_t runAt[kCollideBlock / 32][32];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = thread >> 5; i < total; i += warps)
        collideWarp<EMIT>(i, arrays, selfContact, runAt[threadIdx.x >> 5], emit);
}

// settle.wgsl:20-36 (gain 1, bodyContact.js:48), then empties the buckets
// this substep used and the segment cursor, restoring the empty grid.
__global__ void settleKernel(const FrameParams* __restrict__ fp, Work work, const uint4* __restrict__ surf,
                             const uint32_t* __restrict__ key, const float4* __restrict__ delta,
                             float4* __restrict__ pos, uint32_t* __restrict__ count, uint32_t* __restrict__ cursor,
                             int apply) {
    pdlWait();
    pdlLaunchNext();
    if (blockIdx.x == 0 && threadIdx.x == 0) *cursor = 0;
    forEachItem(work, [&](uint32_t r) {
        if (apply) {
            const float4 d = delta[r];
            if (d.w > 0.0f) {
                const uint32_t node = surf[r].x;
                const float4 P = pos[node];
                const V step = xyz(d) * (1.0f / d.w);
                pos[node] = withW(xyz(P) + step, P.w);
            }
        }
        if (key[r] != kIdle) count[key[r]] = 0;
    });
}

// The gather's work on the current grid, for measurement: per live record,
// its 27 neighbour buckets' visible entries (min(count, kBucketSlots) each,
// what collideKernel reads), summed into out[1]; live records into out[0],
// occupied buckets (their first-arriving records) into out[2]. Runs between
// the gather and the pass that empties the grid.
__global__ void censusKernel(Work work, const uint4* __restrict__ surf, const DevBody* __restrict__ bodies,
                             const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                             const uint32_t* __restrict__ count, unsigned long long* __restrict__ out) {
    forEachItem(work, [&](uint32_t r) {
        const uint32_t b = key[r];
        if (b == kIdle) return;
        const DevBody* g = bodies + surf[r].y;
        const uint32_t linear = b - g->gridBase;
        const uint32_t z = divBy(linear, g->divXY);
        const uint32_t rest = linear - z * (g->gridDims[0] * g->gridDims[1]);
        const uint32_t y = divBy(rest, g->divX);
        const int c[3] = {int(rest - y * g->gridDims[0]), int(y), int(z)};
        unsigned long long seen = 0;
        for (int q = 0; q < 27; q++) {
            const int x = c[0] + q % 3 - 1, yy = c[1] + (q / 3) % 3 - 1, zz = c[2] + q / 9 - 1;
            if (x < 0 || yy < 0 || zz < 0 || x >= int(g->gridDims[0]) || yy >= int(g->gridDims[1]) ||
                zz >= int(g->gridDims[2]))
                continue;
            const uint32_t n = count[g->gridBase + uint32_t(x) + g->gridDims[0] * (uint32_t(yy) + g->gridDims[1] * uint32_t(zz))];
            seen += n < kBucketSlots ? n : kBucketSlots;
        }
        atomicAdd(&out[0], 1ull);
        atomicAdd(&out[1], seen);
        if (rank[r] == 0) atomicAdd(&out[2], 1ull);
    });
}

// ------------------------------------------------------- node utilities --

// pos.w := base[n] for a list of nodes (restoring a released hold).
__global__ void restoreWKernel(const uint32_t* __restrict__ nodes, uint32_t n, const float* __restrict__ base,
                               float4* __restrict__ pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[nodes[i]].w = base[nodes[i]];
}

// pos.w := 0 for a list of nodes (a hard hold prescribes them).
__global__ void zeroWKernel(const uint32_t* __restrict__ nodes, uint32_t n, float4* __restrict__ pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[nodes[i]].w = 0.0f;
}

// pos.w := base[n] for a node range (after a density change).
__global__ void refreshWKernel(uint32_t first, uint32_t n, const float* __restrict__ base, float4* __restrict__ pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[first + i].w = base[first + i];
}

// pos.xyz := in.xyz keeping w (writing a state from the host).
__global__ void mergeXyzKernel(const float4* __restrict__ in, uint32_t n, float4* __restrict__ pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 a = in[i];
        pos[i] = make_float4(a.x, a.y, a.z, pos[i].w);
    }
}

// out := (in.xyz, 0): a state read out (positions cross the ABI with w 0).
__global__ void dropWKernel(const float4* __restrict__ in, uint32_t n, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 a = in[i];
        out[i] = make_float4(a.x, a.y, a.z, 0.0f);
    }
}

// ------------------------------------------------------------ launchers --

namespace {
template <class... KArgs, class... Args>
cudaError_t launch(const LaunchCtx& ctx, void (*kernel)(KArgs...), uint32_t grid, uint32_t block, Args... args) {
    if (grid == 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = ctx.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

inline uint32_t blocks(uint32_t n, uint32_t b) { return (n + b - 1) / b; }
}  // namespace

Span denseSpan(uint32_t count, uint32_t block) { return Span{Work{nullptr, 0, count}, blocks(count, block), block}; }

// A colour pass of a small scene has too few cells to put a block of the
// configured size on every SM; smaller blocks spread it over all of them
// (at the headline body's 15,800 cells a pass, blocks of 32 measured faster
// in the frame than blocks of 64: 4.97 against 5.15 us a pass).
Span elasticSpan(uint32_t count, uint32_t block, uint32_t sms) {
    while (block > 32 && blocks(count, block) < 2 * sms) block /= 2;
    return denseSpan(count, block);
}

namespace {
DriveTables driveTables(const DeviceState& s) {
    return DriveTables{s.drivenOf, s.drivenOffset, s.grabs};
}
}  // namespace

cudaError_t launchPredict(const LaunchCtx& c, const DeviceState& s, const Span& n, bool drive) {
    auto go = [&](auto kernel) {
        return launch(c, kernel, n.grid, n.block, s.fp, n.work, s.active, s.activeBody,
                      (const uint32_t*)s.bodyActive, driveTables(s), s.pos, s.prev, s.vel);
    };
    return drive ? go(predictKernel<true>) : go(predictKernel<false>);
}

cudaError_t launchMarkDriven(cudaStream_t st, const uint32_t* driven, uint32_t n, int32_t* drivenOf, bool clear) {
    if (n == 0) return cudaSuccess;
    markDrivenKernel<<<blocks(n, 256), 256, 0, st>>>(driven, n, drivenOf, clear ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launchElastic(const LaunchCtx& c, const DeviceState& s, const uint4* cells, const Span& sp,
                          bool limitOnly, const StretchLengths& lens) {
    if (c.quadCells && !limitOnly && !sp.work.table && !streamsColourPass(sp.work.count, c.sms))
        return launch(c, elasticQuadKernel, blocks(4 * sp.work.count, 128), 128, cells, sp.work.count, s.bodies,
                      (const uint32_t*)s.bodyActive, s.pos, (const float4*)s.prev, lens);
    if (!limitOnly && !sp.work.table && streamsColourPass(sp.work.count, c.sms))
        return launch(c, elasticStreamKernel, std::min(blocks(sp.work.count, kStreamBlock), kStreamBlocksPerSm * c.sms),
                      kStreamBlock,
                      cells, sp.work.count, s.bodies, (const uint32_t*)s.bodyActive, s.pos, (const float4*)s.prev,
                      lens);
    if (limitOnly)
        return launch(c, elasticKernel<true>, sp.grid, sp.block, cells, sp.work, s.bodies,
                      (const uint32_t*)s.bodyActive, s.pos, (const float4*)s.prev, lens);
    return launch(c, elasticKernel<false>, sp.grid, sp.block, cells, sp.work, s.bodies,
                  (const uint32_t*)s.bodyActive, s.pos, (const float4*)s.prev, lens);
}

cudaError_t launchFinalize(const LaunchCtx& c, const DeviceState& s, const Span& n, bool contact, bool predictNext,
                           bool drive) {
    auto go = [&](auto kernel) {
        return launch(c, kernel, n.grid, n.block, s.fp, n.work, s.active, s.activeBody, s.bodies, s.pos, s.prev,
                      s.vel, (const int32_t*)s.nodeRecord, (const float4*)s.delta, (const uint32_t*)s.key, s.count,
                      s.cursor, (const uint32_t*)s.bodyActive, driveTables(s));
    };
    if (predictNext && drive)
        return contact ? go(finalizeKernel<true, true, true>) : go(finalizeKernel<false, true, true>);
    if (contact) return predictNext ? go(finalizeKernel<true, true, false>) : go(finalizeKernel<true, false, false>);
    return predictNext ? go(finalizeKernel<false, true, false>) : go(finalizeKernel<false, false, false>);
}

// Solve mode leaves the corrections in `delta` for the closing pass, which
// applies them and empties the grid; Pairs mode lists the hits and empties
// the grid itself.
cudaError_t launchContact(const LaunchCtx& c, const DeviceState& s, const Span& r, uint32_t recordItems,
                          int mapping, ContactMode mode, uint32_t* pairs, uint32_t capacity,
                          unsigned long long* pairCount, cudaEvent_t* marks) {
    const uint32_t g = r.grid, b = r.block;
    const Work w = r.work;
    cudaError_t e;
    auto mark = [&](int i) { return marks ? cudaEventRecord(marks[i], c.stream) : cudaSuccess; };
    if ((e = mark(0))) return e;
    if ((e = launch(c, binKernel, g, b, s.fp, w, s.surf, (const DevBody*)s.bodies, (const uint32_t*)s.bodyActive,
                    (const float4*)s.pos, s.key, s.rank, s.count)))
        return e;
    if ((e = mark(1))) return e;
    if ((e = launch(c, allocKernel, g, b, s.fp, w, (const uint32_t*)s.key, (const uint32_t*)s.rank,
                    (const uint32_t*)s.count, s.start, s.cursor)))
        return e;
    if ((e = mark(2))) return e;
    if ((e = launch(c, scatterKernel, g, b, s.fp, w, (const uint32_t*)s.key, (const uint32_t*)s.rank,
                    (const uint32_t*)s.start, s.entries)))
        return e;
    if ((e = mark(3))) return e;
    if ((e = launch(c, canonKernel, g, b, s.fp, w, (const uint32_t*)s.key, (const uint32_t*)s.rank,
                    (const uint32_t*)s.start, (const uint32_t*)s.count, s.entries, (const uint4*)s.surf,
                    (const float4*)s.pos, (const float4*)s.prev, (const DevBody*)s.bodies, s.sMeta, s.sPos,
                    s.sMoved, s.sRec, s.sKey)))
        return e;
    if ((e = mark(4))) return e;
    // The gather runs over the bucket-ordered entries (at most recordItems),
    // a warp each while fewer than 2048 per SM, else a thread each. Over one
    // body (a dense span) one resident wave of blocks (five an SM at its
    // launch bounds) loops over the records: on the headline body 32.8
    // against 34.8 us for a block per eight records. Over many isolated
    // bodies (a chunked span: settled sessions whose records' candidate
    // counts vary widely) the span says: up to a block per eight records
    // (64 an SM) keeps the SMs balanced on large frames -- the looping wave
    // cut the serving pool's saturation by 7 % -- and 16 an SM suits small
    // ones (a one-session tick 0.62 against 0.68 ms).
    const uint32_t cg = std::min(blocks(recordItems, 8), (r.work.table ? r.gatherPerSm : 5u) * c.sms);
    const uint32_t warpModeBelow = mapping == VSIM_GATHER_WARP     ? 0xffffffffu
                                   : mapping == VSIM_GATHER_THREAD ? 0u
                                                                   : 2048 * c.sms;
    auto collide = [&](auto kernel, uint32_t* out, uint32_t cap, unsigned long long* n) {
        return launch(c, kernel, cg, kCollideBlock, s.fp, recordItems, warpModeBelow, (const uint32_t*)s.cursor,
                      (const DevBody*)s.bodies, (const uint32_t*)s.start, (const uint32_t*)s.count,
                      (const uint4*)s.sMeta, (const float4*)s.sPos, (const float4*)s.sMoved,
                      (const uint32_t*)s.sRec, (const uint32_t*)s.sKey, s.delta, out, cap, n);
    };
    if (mode == ContactMode::Pairs) {
        if ((e = collide(collideKernel<true>, pairs, capacity, pairCount))) return e;
        if ((e = mark(5))) return e;
        return launch(c, settleKernel, g, b, s.fp, w, s.surf, (const uint32_t*)s.key, (const float4*)s.delta, s.pos,
                      s.count, s.cursor, 0);
    }
    if ((e = collide(collideKernel<false>, (uint32_t*)nullptr, 0u, (unsigned long long*)nullptr))) return e;
    return mark(5);
}

cudaError_t launchCensus(const LaunchCtx& c, const DeviceState& s, const Span& r, unsigned long long* out) {
    cudaError_t e_;
    if ((e_ = launch(c, censusKernel, r.grid, r.block, r.work, (const uint4*)s.surf, (const DevBody*)s.bodies,
                     (const uint32_t*)s.key, (const uint32_t*)s.rank, (const uint32_t*)s.count, out)))
        return e_;
    // empty the grid without applying the corrections
    return launch(c, settleKernel, r.grid, r.block, s.fp, r.work, s.surf, (const uint32_t*)s.key,
                  (const float4*)s.delta, s.pos, s.count, s.cursor, 0);
}

cudaError_t launchRestoreW(cudaStream_t st, const uint32_t* nodes, uint32_t n, const float* base, float4* pos) {
    if (n == 0) return cudaSuccess;
    restoreWKernel<<<blocks(n, 256), 256, 0, st>>>(nodes, n, base, pos);
    return cudaGetLastError();
}

cudaError_t launchZeroW(cudaStream_t st, const uint32_t* nodes, uint32_t n, float4* pos) {
    if (n == 0) return cudaSuccess;
    zeroWKernel<<<blocks(n, 256), 256, 0, st>>>(nodes, n, pos);
    return cudaGetLastError();
}

cudaError_t launchRefreshW(cudaStream_t st, uint32_t first, uint32_t n, const float* base, float4* pos) {
    if (n == 0) return cudaSuccess;
    refreshWKernel<<<blocks(n, 256), 256, 0, st>>>(first, n, base, pos);
    return cudaGetLastError();
}

cudaError_t launchDropW(cudaStream_t st, const float4* in, uint32_t n, float4* out) {
    if (n == 0) return cudaSuccess;
    dropWKernel<<<blocks(n, 256), 256, 0, st>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t launchMergeXyz(cudaStream_t st, const float4* in, uint32_t n, float4* pos) {
    if (n == 0) return cudaSuccess;
    mergeXyzKernel<<<blocks(n, 256), 256, 0, st>>>(in, n, pos);
    return cudaGetLastError();
}

}  // namespace vsim
