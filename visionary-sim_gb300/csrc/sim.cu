// The simulator object behind the C ABI: it owns every device buffer of a
// scene, encodes a frame's substeps as kernel launches (captured once per
// topology into a CUDA graph and replayed), and carries the host-side state
// of the reference's Simulator (simulator.js:35-518): clock, grab, drive law,
// materials.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>

#include "sim_internal.cuh"

using namespace vsim;

namespace vsim {

__global__ void setParamsKernel(FrameParams* dst, FrameParams src) { *dst = src; }

StretchLengths stretchLengths() {
    StretchLengths s;
    // stretch.js:5-7: Math.hypot of the corner offset, one to three unit axes.
    s.len[0] = float(std::hypot(std::hypot(1.0, 0.0), 0.0));
    s.len[1] = float(std::hypot(std::hypot(1.0, 1.0), 0.0));
    s.len[2] = float(std::hypot(std::hypot(1.0, 1.0), 1.0));
    return s;
}

bool anyStretch(const vsim_sim* s) {
    for (const auto& m : s->mat)
        if (m.max_stretch > 1) return true;
    return false;
}

double waveRateOf(const vsim_sim* s, int* worst) {
    // simulator.js:162-186: the body with the largest wave speed / cflLength
    // (the cell edge, voxelLattice.js:63); the first of equals wins.
    double best = 0;
    int at = -1;
    for (size_t b = 0; b < s->lat.size(); b++) {
        const double rate = waveSpeed(s->mat[b]) / s->lat[b].h;
        if (at < 0 || rate > best) {
            best = rate;
            at = int(b);
        }
    }
    if (worst) *worst = at;
    return at < 0 ? 0 : best;
}

// Per-body constants, in the order and precision project.wgsl:64-73 and
// finalize.wgsl:71-72 derive them.
void bodyParams(const vsim_sim* s, std::vector<DevBody>& out) {
    const float dt = float(s->clock.stepDuration);
    const float invDt2 = 1.0f / (dt * dt);
    out.resize(s->lat.size());
    for (size_t b = 0; b < s->lat.size(); b++) {
        const Lattice& L = s->lat[b];
        const vsim_material& m = s->mat[b];
        double mu, lambda;
        lame(m, mu, lambda);
        const double volume = (1.0 / 6.0) * std::pow(L.h, 3.0);  // kuhn.js:48-50
        const float alphaDev = float(1 / (mu * volume));         // compliance.js:30-37
        const float alphaHyd = float(1 / (lambda * volume));
        DevBody& d = out[b];
        std::memset(&d, 0, sizeof d);
        d.nodeOffset = s->offsets[b];
        d.nx = L.nodeDims[0];
        d.nxy = L.nodeDims[0] * L.nodeDims[1];
        d.alphaDev = alphaDev * invDt2;
        d.alphaHyd = alphaHyd * invDt2;
        d.gamma = float(1 + mu / lambda);
        d.relax = float(m.relaxation) / dt;
        d.h = float(L.h);
        d.restScale = 1.0f / d.h;
        d.maxStretch = float(m.max_stretch);
        d.friction = float(m.friction);
        const float damping = float(m.damping);
        const float arg = -damping * dt;
        d.damp = float(std::exp(double(arg)));
        const size_t g = s->isolated ? b : 0;
        for (int a = 0; a < 3; a++) {
            d.gridOrigin[a] = float(s->grids[g].origin[a]);
            d.gridDims[a] = s->grids[g].dims[a];
        }
        d.bucket = float(s->grids[g].bucket);
        d.gridBase = s->gridBase[g];
        d.divX = reciprocal64(d.gridDims[0]);
        d.divXY = reciprocal64(d.gridDims[0] * d.gridDims[1]);
    }
}

void frameParams(vsim_sim* s) {
    FrameParams& f = s->fpHost;
    std::memset(&f, 0, sizeof f);
    f.dt = float(s->clock.stepDuration);
    f.gx = float(s->gravity[0]);
    f.gy = float(s->gravity[1]);
    f.gz = float(s->gravity[2]);
    for (int a = 0; a < 3; a++) {
        f.tankMin[a] = float(s->tank.min[a]);
        f.tankMax[a] = float(s->tank.max[a]);
        f.grabTarget[a] = float(s->grabPos[a]);
        f.grabVelocity[a] = float(s->grabVel[a]);
    }
    f.invDt2 = 1.0f / (f.dt * f.dt);
    f.responseTime = float(s->responseTime);
    f.drivenCount = uint32_t(s->held.size());
    f.law = uint32_t(s->law);
    f.surfaceCount = s->surfaceCount;
    f.perBodyGrab = s->perBodyGrab ? 1u : 0u;
    f.selfContact = s->selfContact ? 1u : 0u;
    f.activeCount = s->activeCount;
}

// Uploads what changed since the last frame, in stream order.
int syncParams(vsim_sim* s) {
    if (s->tablesDirty) {
        // Through pinned staging; the staging may still feed a copy queued
        // by an earlier frame, so let the stream drain before rewriting it
        // (these tables change between frames, not during a run of them).
        CK(cudaStreamSynchronize(s->stream), "upload body activity");
        std::copy(s->activeHost.begin(), s->activeHost.end(), s->activePinned);
        std::copy(s->grabsHost.begin(), s->grabsHost.end(), s->grabsPinned);
        CK(cudaMemcpyAsync(s->d.bodyActive, s->activePinned, s->activeHost.size() * 4, cudaMemcpyHostToDevice,
                           s->stream),
           "upload body activity");
        CK(cudaMemcpyAsync(s->d.grabs, s->grabsPinned, s->grabsHost.size() * 16, cudaMemcpyHostToDevice, s->stream),
           "upload drive targets");
        s->tablesDirty = false;
    }
    if (s->paramsDirty) {
        std::vector<DevBody> bodies;
        bodyParams(s, bodies);
        CK(cudaMemcpyAsync(s->d.bodies, bodies.data(), bodies.size() * sizeof(DevBody), cudaMemcpyHostToDevice,
                           s->stream),
           "upload body constants");
        s->paramsDirty = false;
        s->frameDirty = true;
    }
    if (s->frameDirty) {
        frameParams(s);
        setParamsKernel<<<1, 1, 0, s->stream>>>(s->d.fp, s->fpHost);
        CK(cudaGetLastError(), "upload frame parameters");
        s->frameDirty = false;
    }
    return VSIM_OK;
}

// The cell list, colour-major over bodies (elasticCells.js:143-163). Inside a
// colour and body the cells run in lattice order, or brick by brick when
// `brick` is 4 or 8 (bricks of that many cells per axis).
void buildCells(vsim_sim* s, std::vector<uint4>& out) {
    out.clear();
    out.reserve(s->cellCount);
    for (int c = 0; c < 8; c++) {
        s->colorStart[c] = uint32_t(out.size());
        s->colourBodyStart[c].assign(s->lat.size() + 1, 0);
        for (size_t b = 0; b < s->lat.size(); b++) {
            s->colourBodyStart[c][b] = uint32_t(out.size()) - s->colorStart[c];
            const Lattice& L = s->lat[b];
            std::vector<uint32_t> order(L.cellsByColor[c]);
            if (s->brick > 1) {
                const uint32_t B = s->brick;
                auto brickKey = [&](uint32_t cell) {
                    const uint32_t i = cell % L.cellDims[0], j = (cell / L.cellDims[0]) % L.cellDims[1],
                                   k = cell / (L.cellDims[0] * L.cellDims[1]);
                    const uint32_t bx = (L.cellDims[0] + B - 1) / B, by = (L.cellDims[1] + B - 1) / B;
                    return uint64_t((i / B) + bx * ((j / B) + by * (k / B))) << 32 | cell;
                };
                std::sort(order.begin(), order.end(),
                          [&](uint32_t a, uint32_t bb) { return brickKey(a) < brickKey(bb); });
            }
            for (uint32_t cell : order) {
                const uint32_t i = cell % L.cellDims[0], j = (cell / L.cellDims[0]) % L.cellDims[1],
                               k = cell / (L.cellDims[0] * L.cellDims[1]);
                out.push_back(make_uint4(s->offsets[b] + i + L.nodeDims[0] * (j + L.nodeDims[1] * k), uint32_t(b),
                                         L.nodeDims[0], L.nodeDims[0] * L.nodeDims[1]));
            }
        }
        s->colourBodyStart[c][s->lat.size()] = uint32_t(out.size()) - s->colorStart[c];
    }
    s->colorStart[8] = uint32_t(out.size());
}

// Spans over every body.
void buildDensePlan(vsim_sim* s) {
    FramePlan& p = s->dense;
    p.chunked = false;
    p.nodes = denseSpan(s->activeCount, 256);
    for (int c = 0; c < 8; c++) p.colour[c] = elasticSpan(s->colorStart[c + 1] - s->colorStart[c], s->block, s->sms);
    p.records = denseSpan(s->surfaceCount, 256);
}

void useDensePlan(vsim_sim* s) { s->plan = s->dense; }

// Chunks of at most kChunk items over the listed bodies' ranges, one table
// for the whole frame: kSpans descriptors, then the chunks. The spans' grids
// and the table's address never change, so one captured graph serves every
// set of bodies; only the table is uploaded per frame.
int planBodies(vsim_sim* s, const std::vector<uint32_t>& bodies) {
    uint2* table = s->chunkPinned;
    uint2* chunks = table + kSpans;
    size_t at = 0;
    auto emit = [&](uint32_t span, const std::vector<uint32_t>& start) {
        const size_t first = at;
        for (uint32_t b : bodies)
            for (uint32_t i = start[b]; i < start[b + 1]; i += kChunk) {
                if (at == s->chunkCapacity) return false;
                chunks[at++] = make_uint2(i, std::min(kChunk, start[b + 1] - i));
            }
        table[span] = make_uint2(uint32_t(first), uint32_t(at - first));
        return true;
    };
    // The staging may still feed the previous frame's upload.
    CK(cudaStreamSynchronize(s->stream), "upload work chunks");
    bool ok = emit(kNodeSpan, s->nodeBodyStart);
    for (int c = 0; c < 8 && ok; c++) ok = emit(colourSpan(c), s->colourBodyStart[c]);
    ok = ok && emit(kRecordSpan, s->recordBodyStart);
    if (!ok) return fail(VSIM_ERR_CAPACITY, "chunk table too small (a body listed twice?)");
    CK(cudaMemcpyAsync(s->chunkDev, table, (kSpans + at) * sizeof(uint2), cudaMemcpyHostToDevice, s->stream),
       "upload work chunks");
    // The gather's grid for this frame's records: small frames take fewer,
    // looping blocks (a second captured graph serves them).
    uint64_t records = 0;
    for (uint32_t b : bodies) records += s->recordBodyStart[b + 1] - s->recordBodyStart[b];
    s->chunked.records.gatherPerSm = records <= (1u << 18) ? 16 : 64;
    s->plan = s->chunked;
    return VSIM_OK;
}

// Brackets kernel groups with events on the launching stream.
struct Profiler {
    cudaStream_t stream;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    struct Span {
        int kind;
        cudaEvent_t a, b;
        uint32_t launches;
    };
    std::vector<Span> spans;
    cudaEvent_t next() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(int kind, uint32_t launches) {
        Span sp{kind, next(), nullptr, launches};
        cudaEventRecord(sp.a, stream);
        spans.push_back(sp);
    }
    void end() {
        spans.back().b = next();
        cudaEventRecord(spans.back().b, stream);
    }
    ~Profiler() {
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

constexpr uint32_t kContactKernels = 5;  // bin, segment, scatter, order, collide

// One colour pass: the TMA brick form for a large dense pass when it is on,
// else launchElastic's choice.
cudaError_t launchColourPass(const LaunchCtx& c, const vsim_sim* s, int col, bool limitOnly,
                             const StretchLengths& lens) {
    const Span& sp = s->plan.colour[col];
    if (!limitOnly && s->tma.enabled && s->tma.ready && !sp.work.table && streamsColourPass(sp.work.count, c.sms))
        return launchElasticTma(c, s, col, lens);
    return launchElastic(c, s->d, s->d.cells + s->colorStart[col], sp, limitOnly, lens);
}

// stepper.js:101-108 with simulator.js:83's constraint order.
cudaError_t encodeFrame(vsim_sim* s, cudaStream_t st, uint32_t steps, ContactMode mode = ContactMode::Solve,
                        Profiler* prof = nullptr) {
    const LaunchCtx c{st, s->pdl, s->sms, s->quadCells};
    const StretchLengths lens = stretchLengths();
    const bool limited = anyStretch(s);
    const bool driving = !s->held.empty();
    const bool contact = s->contact && s->surfaceCount > 0;
    cudaError_t e;
    auto begin = [&](int kind, uint32_t launches) {
        if (prof) prof->begin(kind, launches);
    };
    auto end = [&]() {
        if (prof) prof->end();
    };
    // The first substep's prediction runs on its own; every later one rides
    // on the closing pass of the substep before it.
    const FramePlan& plan = s->plan;
    // The drive (the substep's first constraint) rides on the pass that
    // predicts the substep.
    if (steps > 0) {
        begin(VSIM_KIND_PREDICT, 1);
        if ((e = launchPredict(c, s->d, plan.nodes, driving))) return e;
        end();
    }
    for (uint32_t step = 0; step < steps; step++) {
        for (uint32_t it = 0; it < s->iterations; it++)
            for (int col = 0; col < 8; col++) {
                if (!plan.colour[col].grid) continue;
                begin(VSIM_KIND_ELASTIC, 1);
                if ((e = launchColourPass(c, s, col, false, lens))) return e;
                end();
            }
        if (limited)
            for (int sweep = 0; sweep < 3; sweep++)
                for (int col = 0; col < 8; col++) {
                    if (!plan.colour[col].grid) continue;
                    begin(VSIM_KIND_LIMIT, 1);
                    if ((e = launchColourPass(c, s, col, true, lens))) return e;
                    end();
                }
        if (contact && plan.records.grid) {
            begin(VSIM_KIND_CONTACT, kContactKernels);
            if ((e = launchContact(c, s->d, plan.records, s->surfaceCount, s->gatherMapping, mode, nullptr, 0, nullptr))) return e;
            end();
        }
        begin(VSIM_KIND_FINALIZE, 1);
        if ((e = launchFinalize(c, s->d, plan.nodes, contact && mode == ContactMode::Solve, step + 1 < steps,
                                driving)))
            return e;
        end();
    }
    return cudaSuccess;
}

uint64_t graphKey(const vsim_sim* s, uint32_t steps) {
    uint64_t k = steps;
    k = k * 31 + (s->held.empty() ? 0 : 1);
    k = k * 31 + ((s->contact && s->surfaceCount > 0) ? 1 : 0);
    k = k * 31 + s->iterations;
    k = k * 31 + (anyStretch(s) ? 1 : 0);
    k = k * 1031 + s->block;
    k = k * 31 + (s->pdl ? 1 : 0);
    k = k * 31 + (s->plan.chunked ? 1 : 0);
    k = k * 31 + uint64_t(s->gatherMapping);
    k = k * 31 + (s->tma.enabled ? 1 : 0);
    k = k * 31 + (s->quadCells ? 1 : 0);
    k = k * 131 + s->plan.records.gatherPerSm;
    return k;
}

void dropGraphs(vsim_sim* s) {
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
}

int runFrame(vsim_sim* s, uint32_t steps) {
    int rc = syncParams(s);
    if (rc) return rc;
    if (!s->useGraph) {
        CK(encodeFrame(s, s->stream, steps), "launch substep");
        return VSIM_OK;
    }
    const uint64_t key = graphKey(s, steps);
    cudaGraphExec_t exec = nullptr;
    for (auto& g : s->graphs)
        if (g.key == key) exec = g.exec;
    if (!exec) {
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal), "begin capture");
        const cudaError_t enc = encodeFrame(s, s->capture, steps);
        const cudaError_t end = cudaStreamEndCapture(s->capture, &graph);
        if (enc != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cudaFail(enc, "capture substep");
        }
        CK(end, "end capture");
        const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(inst, "instantiate frame graph");
        if (s->graphs.size() >= 8) {
            cudaGraphExecDestroy(s->graphs.front().exec);
            s->graphs.erase(s->graphs.begin());
        }
        s->graphs.push_back({key, exec});
    }
    CK(cudaGraphLaunch(exec, s->stream), "launch frame graph");
    return VSIM_OK;
}

// Nodes [first, first + count) of pos, prev and vel (those of `out` not
// NULL) to the host as xyzw with w = 0, the ABI's form: w is cleared on the
// device into the staging buffer, one array at a time (stream order keeps
// the next clear behind the previous copy), so the host gets each array in
// one copy and touches nothing after it.
int readNodes(vsim_sim* s, size_t first, size_t count, float* const out[3]) {
    const float4* from[3] = {s->d.pos + first, s->d.prev + first, s->d.vel + first};
    if (count > 0 && !s->staging) CK(allocN(&s->staging, s->nodeCount), "allocate staging");
    for (int a = 0; a < 3; a++) {
        if (!out[a] || count == 0) continue;
        CK(launchDropW(s->stream, from[a], uint32_t(count), s->staging), "read state");
        CK(cudaMemcpyAsync(out[a], s->staging, count * 16, cudaMemcpyDeviceToHost, s->stream), "read state");
    }
    CK(cudaStreamSynchronize(s->stream), "read state");
    return VSIM_OK;
}

void freeSim(vsim_sim* s) {
    dropGraphs(s);
    DeviceState& d = s->d;
    void* ptrs[] = {d.pos, d.prev, d.vel, d.baseW, d.active, d.activeBody, d.cells, d.bodies, d.fp,
                    d.surf, d.key, d.rank, d.entries, d.count, d.start, d.cursor, d.delta, d.driven,
                    d.drivenOffset, d.drivenOf, d.nodeRecord, d.sMeta, d.sPos, d.sMoved, d.sRec, d.sKey, d.bodyActive, d.grabs,
                    s->chunkDev, s->staging, s->pairs, s->pairCount, s->sp.embed, s->sp.quat,
                    s->sp.scaleBody, s->sp.bodies, s->sp.meanDepth, s->sp.cov, s->sp.keys, s->sp.order,
                    s->sp.sortTemp};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    freeTmaPass(s->tma);
    void* pinned[] = {s->chunkPinned, s->activePinned, s->grabsPinned};
    for (void* p : pinned)
        if (p) cudaFreeHost(p);
    if (s->capture) cudaStreamDestroy(s->capture);
    if (s->ownStream && s->stream) cudaStreamDestroy(s->stream);
}

int restoreHeld(vsim_sim* s) {
    if (s->law == VSIM_DRIVE_HARD && !s->held.empty())
        CK(launchRestoreW(s->stream, s->d.driven, uint32_t(s->held.size()), s->d.baseW, s->d.pos), "restore hold");
    return VSIM_OK;
}

int zeroHeld(vsim_sim* s) {
    if (s->law == VSIM_DRIVE_HARD && !s->held.empty())
        CK(launchZeroW(s->stream, s->d.driven, uint32_t(s->held.size()), s->d.pos), "prescribe hold");
    return VSIM_OK;
}

// An isolated body's contact grid: its rest box padded by a quarter of its
// extent (at least four buckets) per side, clipped to the tank. A node that
// leaves it is binned at the rim, which costs gather time, never a contact.
Grid bodyGrid(const Lattice& L, const vsim_tank& tank) {
    vsim_tank box;
    for (int a = 0; a < 3; a++) {
        const double pad = std::max(0.25 * L.cellDims[a] * L.h, 8 * L.h * kContactRadiusCells);
        box.min[a] = std::max(tank.min[a], L.origin[a] - pad);
        box.max[a] = std::min(tank.max[a], L.origin[a] + L.cellDims[a] * L.h + pad);
    }
    const double zero[3] = {0, 0, 0};
    return contactGrid(box, L.h * kContactRadiusCells, zero, zero);
}

int createSim(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, void* stream, bool isolated,
              vsim_sim* s) {
    s->isolated = isolated;
    if (n > 0 && !bodies) return fail(VSIM_ERR_INVALID, "bodies is NULL");
    CK(cudaGetDevice(&s->device), "query device");
    int major = 0;
    CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, s->device), "query device");
    if (major < 10) return fail(VSIM_ERR_INVALID, "libvsim is built for sm_103a (GB300) only");
    int sms = 1;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device), "query device");
    s->sms = uint32_t(sms);
    if (tank) {
        s->tank = *tank;
    } else {
        for (int a = 0; a < 3; a++) {
            s->tank.min[a] = -INFINITY;
            s->tank.max[a] = INFINITY;
        }
    }
    s->lat.resize(n);
    s->mat.resize(n);
    uint64_t total = 0;
    for (uint32_t b = 0; b < n; b++) {
        int rc = buildLattice(bodies[b], s->lat[b]);
        if (rc) return rc;
        s->mat[b] = bodies[b].material;
        s->offsets.push_back(uint32_t(total));
        total += s->lat[b].nodeCount;
        if (total >= (1ull << 31)) return fail(VSIM_ERR_RANGE, "scene has too many nodes");
    }
    s->nodeCount = uint32_t(total);
    s->isStatic.assign(total, 0);
    s->invMass.assign(total, 0.0f);
    for (uint32_t b = 0; b < n; b++) {
        const Lattice& L = s->lat[b];
        std::copy(L.invMass.begin(), L.invMass.end(), s->invMass.begin() + s->offsets[b]);
        for (uint32_t i = 0; i < bodies[b].static_count; i++) {
            const uint32_t node = bodies[b].static_nodes[i];
            if (node >= L.nodeCount) return fail(VSIM_ERR_RANGE, "static node outside its body");
            s->isStatic[s->offsets[b] + node] = 1;
        }
        s->cellCount += L.cellCount;
    }
    s->baseW.resize(total);
    for (uint64_t i = 0; i < total; i++) s->baseW[i] = s->isStatic[i] ? 0.0f : s->invMass[i];

    // Active nodes: every node with material. Predict and finalize skip those
    // whose solver inverse mass is zero, as the reference does; the closing
    // pass still settles and un-bins the static ones on the surface.
    std::vector<uint32_t> active, activeBody;
    s->nodeBodyStart.assign(size_t(n) + 1, 0);
    for (uint32_t b = 0; b < n; b++) {
        s->nodeBodyStart[b] = uint32_t(active.size());
        for (uint32_t m = 0; m < s->lat[b].nodeCount; m++) {
            const uint32_t node = s->offsets[b] + m;
            if (s->invMass[node] > 0) {
                active.push_back(node);
                activeBody.push_back(b);
            }
        }
    }
    s->nodeBodyStart[n] = uint32_t(active.size());
    s->activeCount = uint32_t(active.size());

    // Surface records (bodyContact.js:325-340), radius h/2.
    double widest = 0;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    s->recordBodyStart.assign(size_t(n) + 1, 0);
    for (uint32_t b = 0; b < n; b++) {
        const Lattice& L = s->lat[b];
        const float radius = float(L.h * kContactRadiusCells);
        s->recordBodyStart[b] = uint32_t(s->surfHost.size());
        for (uint32_t node : L.surface) {
            const uint32_t i = node % L.nodeDims[0], j = (node / L.nodeDims[0]) % L.nodeDims[1],
                           k = node / (L.nodeDims[0] * L.nodeDims[1]);
            uint32_t bits;
            std::memcpy(&bits, &radius, 4);
            const uint32_t coord = (i & 1023u) | ((j & 1023u) << 10) | ((k & 1023u) << 20);
            s->surfHost.push_back(make_uint4(s->offsets[b] + node, b, coord, bits));
            widest = std::max(widest, double(radius));
        }
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], L.origin[a]);
            hi[a] = std::max(hi[a], L.origin[a] + L.cellDims[a] * L.h);
        }
    }
    s->surfaceCount = uint32_t(s->surfHost.size());
    s->recordBodyStart[n] = s->surfaceCount;
    if (!s->isolated) {
        s->grids.push_back(contactGrid(s->tank, widest, lo, hi));
    } else {
        for (uint32_t b = 0; b < n; b++) s->grids.push_back(bodyGrid(s->lat[b], s->tank));
    }
    for (const Grid& g : s->grids) {
        s->gridBase.push_back(uint32_t(s->bucketTotal));
        s->bucketTotal += g.count();
    }
    if (double(s->bucketTotal) > 16.0 * kGridLimit) return fail(VSIM_ERR_RANGE, "contact grids too large");
    s->activeHost.assign(n ? n : 1, 1u);
    s->grabsHost.assign(2 * size_t(n ? n : 1), make_float4(0, 0, 0, 0));
    s->tablesDirty = true;

    // Clock (simulator.js:88).
    s->clock.stepDuration = stableStepDuration(waveRateOf(s, nullptr));
    s->clock.reset();

    // Streams.
    if (stream) {
        s->stream = static_cast<cudaStream_t>(stream);
    } else {
        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "create stream");
        s->ownStream = true;
    }
    CK(cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking), "create capture stream");

    // Device buffers.
    DeviceState& d = s->d;
    const size_t N = s->nodeCount;
    CK(allocN(&d.pos, N), "allocate positions");
    CK(allocN(&d.prev, N), "allocate previous positions");
    CK(allocN(&d.vel, N), "allocate velocities");
    CK(allocN(&d.baseW, N), "allocate masses");
    CK(allocN(&d.active, s->activeCount), "allocate active list");
    CK(allocN(&d.activeBody, s->activeCount), "allocate active list");
    CK(allocN(&d.cells, s->cellCount), "allocate cells");
    CK(allocN(&d.bodies, n), "allocate body constants");
    CK(allocN(&d.fp, 1), "allocate frame parameters");
    CK(allocN(&d.surf, s->surfaceCount), "allocate surface");
    CK(allocN(&d.key, s->surfaceCount), "allocate contact keys");
    CK(allocN(&d.rank, s->surfaceCount), "allocate contact ranks");
    CK(allocN(&d.entries, s->surfaceCount), "allocate contact entries");
    CK(allocN(&d.delta, s->surfaceCount), "allocate contact deltas");
    CK(allocN(&d.sMeta, s->surfaceCount), "allocate contact runs");
    CK(allocN(&d.sPos, s->surfaceCount), "allocate contact runs");
    CK(allocN(&d.sRec, s->surfaceCount), "allocate contact runs");
    CK(allocN(&d.sKey, s->surfaceCount), "allocate contact runs");
    CK(allocN(&d.sMoved, s->surfaceCount), "allocate contact runs");
    CK(allocN(&d.nodeRecord, N), "allocate node records");
    CK(allocN(&d.count, s->bucketTotal), "allocate contact grid");
    CK(allocN(&d.start, s->bucketTotal), "allocate contact grid");
    CK(allocN(&d.bodyActive, s->activeHost.size()), "allocate body activity");
    CK(allocN(&d.grabs, s->grabsHost.size()), "allocate drive targets");
    CK(allocN(&d.cursor, 1), "allocate contact cursor");
    CK(allocN(&d.driven, VSIM_MAX_DRIVEN), "allocate drive");
    CK(allocN(&d.drivenOffset, VSIM_MAX_DRIVEN), "allocate drive");
    CK(allocN(&d.drivenOf, N), "allocate drive");
    CK(allocN(&s->pairCount, 4), "allocate pair counter");  // [0] pairs, [1..3] the contact census
    CK(cudaMallocHost(&s->activePinned, s->activeHost.size() * 4), "allocate staging");
    CK(cudaMallocHost(&s->grabsPinned, s->grabsHost.size() * 16), "allocate staging");

    // Initial state (particles.js:67-102).
    s->restPos.assign(4 * N, 0.0f);
    for (uint32_t b = 0; b < n; b++) {
        const Lattice& L = s->lat[b];
        for (uint32_t m = 0; m < L.nodeCount; m++) {
            const size_t node = s->offsets[b] + m;
            s->restPos[4 * node] = L.rest[3 * m];
            s->restPos[4 * node + 1] = L.rest[3 * m + 1];
            s->restPos[4 * node + 2] = L.rest[3 * m + 2];
            s->restPos[4 * node + 3] = s->baseW[node];
        }
    }
    std::vector<uint4> cells;
    buildCells(s, cells);
    buildDensePlan(s);
    useDensePlan(s);
    if (isolated) {
        // Room for a chunk table over every body at once, and the spans
        // over it: blocks of kChunk threads, as many as fill the device
        // (the elastic pass holds 4 such blocks per SM at its registers).
        size_t chunks = 0;
        auto span = [&](uint32_t index, const std::vector<uint32_t>& start, uint32_t perSm) {
            size_t most = 0;
            for (uint32_t b = 0; b < n; b++) most += (start[b + 1] - start[b] + kChunk - 1) / kChunk;
            chunks += most;
            const uint32_t grid = uint32_t(std::min<size_t>(most, size_t(perSm) * s->sms));
            return Span{Work{nullptr, index, 0}, grid, kChunk};
        };
        FramePlan& p = s->chunked;
        p.chunked = true;
        p.nodes = span(kNodeSpan, s->nodeBodyStart, 16);
        for (int c = 0; c < 8; c++) p.colour[c] = span(colourSpan(c), s->colourBodyStart[c], 4);
        p.records = span(kRecordSpan, s->recordBodyStart, 16);
        s->chunkCapacity = chunks;
        CK(allocN(&s->chunkDev, kSpans + chunks), "allocate work chunks");
        CK(cudaMallocHost(&s->chunkPinned, (kSpans + chunks) * sizeof(uint2)), "allocate staging");
        p.nodes.work.table = s->chunkDev;
        for (int c = 0; c < 8; c++) p.colour[c].work.table = s->chunkDev;
        p.records.work.table = s->chunkDev;
    }
    std::vector<int32_t> nodeRecord(N, -1);
    for (uint32_t r = 0; r < s->surfaceCount; r++) nodeRecord[s->surfHost[r].x] = int32_t(r);
    CK(cudaMemcpyAsync(d.nodeRecord, nodeRecord.data(), N * 4, cudaMemcpyHostToDevice, s->stream), "upload records");
    CK(cudaMemcpyAsync(d.pos, s->restPos.data(), N * 16, cudaMemcpyHostToDevice, s->stream), "upload state");
    CK(cudaMemcpyAsync(d.prev, s->restPos.data(), N * 16, cudaMemcpyHostToDevice, s->stream), "upload state");
    CK(cudaMemsetAsync(d.vel, 0, N * 16, s->stream), "upload state");
    CK(cudaMemsetAsync(d.drivenOf, 0xff, N * 4, s->stream), "clear drive rows");  // -1: not driven
    CK(cudaMemcpyAsync(d.baseW, s->baseW.data(), N * 4, cudaMemcpyHostToDevice, s->stream), "upload masses");
    CK(cudaMemcpyAsync(d.active, active.data(), active.size() * 4, cudaMemcpyHostToDevice, s->stream), "upload");
    CK(cudaMemcpyAsync(d.activeBody, activeBody.data(), activeBody.size() * 4, cudaMemcpyHostToDevice, s->stream),
       "upload");
    CK(cudaMemcpyAsync(d.cells, cells.data(), cells.size() * 16, cudaMemcpyHostToDevice, s->stream), "upload cells");
    CK(cudaMemcpyAsync(d.surf, s->surfHost.data(), s->surfHost.size() * 16, cudaMemcpyHostToDevice, s->stream),
       "upload surface");
    CK(cudaMemsetAsync(d.count, 0, s->bucketTotal * 4, s->stream), "clear grid");
    CK(cudaMemsetAsync(d.cursor, 0, 4, s->stream), "clear grid");
    s->paramsDirty = true;
    int rc = syncParams(s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream), "initialise");
    s->splatMeans.resize(n);
    s->splatQuats.resize(n);
    s->splatScales.resize(n);
    return VSIM_OK;
}

}  // namespace vsim

extern "C" {

int vsim_create_ex(const vsim_body_desc* bodies, uint32_t body_count, const vsim_tank* tank, void* stream,
                   uint32_t flags, vsim_sim** out) {
    clearError();
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (flags & ~uint32_t(VSIM_CREATE_ISOLATED)) return fail(VSIM_ERR_INVALID, "unknown creation flags");
    vsim_sim* s = new (std::nothrow) vsim_sim();
    if (!s) return fail(VSIM_ERR_NOMEM, "out of host memory");
    int rc;
    try {
        rc = createSim(bodies, body_count, tank, stream, (flags & VSIM_CREATE_ISOLATED) != 0, s);
    } catch (const std::bad_alloc&) {
        rc = fail(VSIM_ERR_NOMEM, "out of host memory");
    }
    if (rc != VSIM_OK) {
        freeSim(s);
        delete s;
        return rc;
    }
    *out = s;
    return VSIM_OK;
}

int vsim_create(const vsim_body_desc* bodies, uint32_t body_count, const vsim_tank* tank, void* stream,
                vsim_sim** out) {
    return vsim_create_ex(bodies, body_count, tank, stream, 0, out);
}

int vsim_set_bodies_active(vsim_sim* s, const uint8_t* active, uint32_t count) {
    SIM_GUARD(s);
    if (count != s->lat.size()) return fail(VSIM_ERR_CAPACITY, "count does not match the body count");
    for (uint32_t b = 0; b < count; b++) s->activeHost[b] = active ? (active[b] ? 1u : 0u) : 1u;
    s->tablesDirty = true;
    return VSIM_OK;
}

int vsim_destroy(vsim_sim* sim) {
    if (!sim) return VSIM_OK;
    {
        DeviceGuard guard(sim->device);
        cudaStreamSynchronize(sim->stream);
        freeSim(sim);
    }
    delete sim;
    return VSIM_OK;
}

int vsim_synchronize(vsim_sim* s) {
    SIM_GUARD(s);
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    if (s->tma.fault) {
        uint32_t fault = 0;
        CK(cudaMemcpy(&fault, s->tma.fault, 4, cudaMemcpyDeviceToHost), "synchronize");
        if (fault) return fail(VSIM_ERR_CUDA, "TMA colour pass: a block's copies did not arrive");
    }
    return VSIM_OK;
}

int vsim_set_cell_lanes(vsim_sim* s, uint32_t lanes) {
    SIM_GUARD(s);
    if (lanes != 1 && lanes != 4) return fail(VSIM_ERR_RANGE, "lanes must be 1 or 4");
    s->quadCells = lanes == 4;
    return VSIM_OK;
}

int vsim_set_tma_pass(vsim_sim* s, int enabled) {
    SIM_GUARD(s);
    if (enabled && !s->tma.ready) {
        if (int rc = buildTmaPass(s)) return rc;
        if (!s->tma.ready) return fail(VSIM_ERR_RANGE, "the TMA colour pass takes 1 to 4 bodies");
    }
    s->tma.enabled = enabled != 0;
    return VSIM_OK;
}

// simulator.js:292-318.
int vsim_dispatch(vsim_sim* s, uint32_t steps) {
    SIM_GUARD(s);
    if (steps < 1 || s->nodeCount == 0) return VSIM_OK;
    if (!s->held.empty()) {
        const double frameDt = steps * s->clock.stepDuration;
        for (int a = 0; a < 3; a++) s->grabVel[a] = (s->grabPos[a] - s->grabPrev[a]) / frameDt;
        std::memcpy(s->grabPrev, s->grabPos, sizeof s->grabPos);
        s->frameDirty = true;
    }
    return runFrame(s, steps);
}

// simulator.js:239-278.
int vsim_step(vsim_sim* s, double dt) {
    SIM_GUARD(s);
    if (s->nodeCount == 0) {
        s->pendingStep = false;
        s->clock.idle();
        return VSIM_OK;
    }
    const double elapsed = std::isfinite(dt) && dt >= 0 ? dt : 0;
    const bool pending = s->pendingStep;
    s->pendingStep = false;
    if (s->paused) {
        if (!pending) {
            s->clock.idle();
            return VSIM_OK;
        }
        s->clock.singleStep();
    } else {
        s->clock.consume(elapsed, pending);
    }
    return vsim_dispatch(s, s->clock.lastSteps);
}

int vsim_request_step(vsim_sim* s) {
    SIM_GUARD(s);
    s->pendingStep = true;
    return VSIM_OK;
}

// simulator.js:495-500, particles.js:245-249.
int vsim_reset(vsim_sim* s) {
    SIM_GUARD(s);
    int rc = vsim_release(s);
    if (rc) return rc;
    const size_t N = s->nodeCount;
    CK(cudaMemcpyAsync(s->d.pos, s->restPos.data(), N * 16, cudaMemcpyHostToDevice, s->stream), "reset");
    CK(cudaMemcpyAsync(s->d.prev, s->restPos.data(), N * 16, cudaMemcpyHostToDevice, s->stream), "reset");
    CK(cudaMemsetAsync(s->d.vel, 0, N * 16, s->stream), "reset");
    s->clock.reset();
    s->pendingStep = false;
    return VSIM_OK;
}

int vsim_read_positions(vsim_sim* s, float* xyzw, size_t node_count) {
    return vsim_read_state(s, xyzw, nullptr, nullptr, node_count);
}

int vsim_read_state(vsim_sim* s, float* pos, float* prev, float* vel, size_t node_count) {
    SIM_GUARD(s);
    if (node_count != s->nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match the simulator");
    float* const out[3] = {pos, prev, vel};
    return readNodes(s, 0, node_count, out);
}

int vsim_write_state(vsim_sim* s, const float* pos, const float* prev, const float* vel, size_t node_count) {
    SIM_GUARD(s);
    if (node_count != s->nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match the simulator");
    if (pos) {
        if (!s->staging) CK(allocN(&s->staging, s->nodeCount), "allocate staging");
        CK(cudaMemcpyAsync(s->staging, pos, node_count * 16, cudaMemcpyHostToDevice, s->stream), "write state");
        CK(launchMergeXyz(s->stream, s->staging, s->nodeCount, s->d.pos), "write state");
    }
    if (prev) CK(cudaMemcpyAsync(s->d.prev, prev, node_count * 16, cudaMemcpyHostToDevice, s->stream), "write state");
    if (vel) CK(cudaMemcpyAsync(s->d.vel, vel, node_count * 16, cudaMemcpyHostToDevice, s->stream), "write state");
    CK(cudaStreamSynchronize(s->stream), "write state");
    return VSIM_OK;
}

uint32_t vsim_node_count(const vsim_sim* s) { return s ? s->nodeCount : 0; }

uint32_t vsim_body_node_offset(const vsim_sim* s, uint32_t body) {
    return s && body < s->offsets.size() ? s->offsets[body] : 0;
}

int vsim_read_inv_mass(vsim_sim* s, float* inv_mass, size_t node_count) {
    SIM_GUARD(s);
    if (node_count != s->nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match the simulator");
    std::copy(s->invMass.begin(), s->invMass.end(), inv_mass);
    return VSIM_OK;
}

}  // extern "C"

namespace vsim {

uint32_t bodyOfNode(const vsim_sim* s, uint32_t node) {
    // pick.js:77-83, by bisection over the ascending body offsets.
    const auto it = std::upper_bound(s->offsets.begin(), s->offsets.end(), node);
    return uint32_t(it - s->offsets.begin()) - 1;
}

int holdNodes(vsim_sim* s, const uint32_t* nodes, const float* offsets, uint32_t count) {
    if (count == 0) return releaseNodes(s);
    const uint32_t kept = std::min<uint32_t>(count, VSIM_MAX_DRIVEN);
    int rc = restoreHeld(s);
    if (rc) return rc;
    CK(launchMarkDriven(s->stream, s->d.driven, uint32_t(s->held.size()), s->d.drivenOf, true), "release hold");
    std::vector<float4> off(kept);
    s->heldBody.resize(kept);
    for (uint32_t i = 0; i < kept; i++) {
        const uint32_t body = bodyOfNode(s, nodes[i]);
        float bits;
        std::memcpy(&bits, &body, 4);
        s->heldBody[i] = body;
        off[i] = make_float4(offsets[3 * i], offsets[3 * i + 1], offsets[3 * i + 2], bits);
    }
    CK(cudaMemcpyAsync(s->d.driven, nodes, kept * 4, cudaMemcpyHostToDevice, s->stream), "upload hold");
    CK(cudaMemcpyAsync(s->d.drivenOffset, off.data(), kept * 16, cudaMemcpyHostToDevice, s->stream), "upload hold");
    // Copies from pageable memory return once the data is staged, so `off`
    // may go out of scope; everything after them is in stream order.
    s->held.assign(nodes, nodes + kept);
    CK(launchMarkDriven(s->stream, s->d.driven, kept, s->d.drivenOf, false), "upload hold");
    rc = zeroHeld(s);
    if (rc) return rc;
    s->frameDirty = true;
    return kept < count ? fail(VSIM_OK, "hold truncated to VSIM_MAX_DRIVEN nodes") : VSIM_OK;
}

int releaseNodes(vsim_sim* s) {
    int rc = restoreHeld(s);
    if (rc) return rc;
    CK(launchMarkDriven(s->stream, s->d.driven, uint32_t(s->held.size()), s->d.drivenOf, true), "release hold");
    s->held.clear();
    s->heldBody.clear();
    s->frameDirty = true;
    return VSIM_OK;
}

}  // namespace vsim

extern "C" {

// kinematicDrive.js:155-191.
int vsim_hold(vsim_sim* s, const uint32_t* nodes, const float* offsets, uint32_t count) {
    SIM_GUARD(s);
    if (count > 0 && (!nodes || !offsets)) return fail(VSIM_ERR_INVALID, "nodes or offsets is NULL");
    for (uint32_t i = 0; i < count; i++) {
        if (nodes[i] >= s->nodeCount) return fail(VSIM_ERR_RANGE, "held node outside the scene");
        if (s->isStatic[nodes[i]]) return fail(VSIM_ERR_INVALID, "[drive] cannot hold a static prescribed node");
    }
    return holdNodes(s, nodes, offsets, count);
}

int vsim_move_grab(vsim_sim* s, const double position[3]) {
    SIM_GUARD(s);
    std::memcpy(s->grabPos, position, sizeof s->grabPos);
    s->frameDirty = true;
    return VSIM_OK;
}

int vsim_place_grab(vsim_sim* s, const double position[3]) {
    SIM_GUARD(s);
    std::memcpy(s->grabPos, position, sizeof s->grabPos);
    std::memcpy(s->grabPrev, position, sizeof s->grabPrev);
    s->frameDirty = true;
    return VSIM_OK;
}

int vsim_release(vsim_sim* s) {
    SIM_GUARD(s);
    return releaseNodes(s);
}

int vsim_set_drive_law(vsim_sim* s, int law) {
    SIM_GUARD(s);
    if (law != VSIM_DRIVE_HARD && law != VSIM_DRIVE_COMPLIANT) return fail(VSIM_ERR_INVALID, "[drive] unknown law");
    if (law == s->law) return VSIM_OK;
    int rc = restoreHeld(s);
    if (rc) return rc;
    s->law = law;
    rc = zeroHeld(s);
    if (rc) return rc;
    s->frameDirty = true;
    return VSIM_OK;
}

int vsim_set_drive_response_time(vsim_sim* s, double seconds) {
    SIM_GUARD(s);
    if (!std::isfinite(seconds) || seconds <= 0)
        return fail(VSIM_ERR_RANGE, "drive responseTime must be a finite positive number of seconds");
    s->responseTime = seconds;
    s->frameDirty = true;
    return VSIM_OK;
}

// simulator.js:332-353.
int vsim_set_material(vsim_sim* s, uint32_t body, const vsim_material* m, uint32_t fields) {
    SIM_GUARD(s);
    if (!m) return fail(VSIM_ERR_INVALID, "changes is NULL");
    if (body >= s->mat.size()) return fail(VSIM_ERR_RANGE, "body index out of range");
    if ((fields & VSIM_MAT_MAX_STRETCH) && !validMaxStretch(m->max_stretch))
        return fail(VSIM_ERR_RANGE, "maxStretch must be zero (disabled) or a finite ratio greater than one");
    vsim_material& mat = s->mat[body];
    if (fields & VSIM_MAT_YOUNGS) mat.youngs_modulus = m->youngs_modulus;
    if (fields & VSIM_MAT_POISSON) mat.poisson_ratio = m->poisson_ratio;
    if (fields & VSIM_MAT_FRICTION) mat.friction = m->friction;
    if (fields & VSIM_MAT_DAMPING) mat.damping = m->damping;
    if (fields & VSIM_MAT_RELAXATION) mat.relaxation = m->relaxation;
    if (fields & VSIM_MAT_MAX_STRETCH) mat.max_stretch = m->max_stretch;
    if ((fields & VSIM_MAT_DENSITY) && m->density > 0 && m->density != mat.density) {
        // voxelLattice.js:188-195: node masses rescale in place.
        const double ratio = mat.density / m->density;
        const uint32_t first = s->offsets[body], count = s->lat[body].nodeCount;
        for (uint32_t i = 0; i < count; i++) {
            float& inv = s->invMass[first + i];
            inv = float(double(inv) * ratio);
            s->baseW[first + i] = s->isStatic[first + i] ? 0.0f : inv;
            s->restPos[4 * size_t(first + i) + 3] = s->baseW[first + i];
        }
        mat.density = m->density;
        CK(cudaMemcpyAsync(s->d.baseW + first, s->baseW.data() + first, count * 4, cudaMemcpyHostToDevice, s->stream),
           "upload masses");
        CK(launchRefreshW(s->stream, first, count, s->d.baseW, s->d.pos), "upload masses");
        int rc = zeroHeld(s);
        if (rc) return rc;
        CK(cudaStreamSynchronize(s->stream), "upload masses");
    }
    if (!s->stepOverridden) s->clock.stepDuration = stableStepDuration(waveRateOf(s, nullptr));
    s->paramsDirty = true;
    return VSIM_OK;
}

int vsim_set_contact(vsim_sim* s, int enabled) {
    SIM_GUARD(s);
    s->contact = enabled != 0;
    return VSIM_OK;
}

int vsim_set_self_contact(vsim_sim* s, int enabled) {
    SIM_GUARD(s);
    for (const Lattice& L : s->lat)
        for (int a = 0; a < 3; a++)
            if (enabled && L.nodeDims[a] > 1024) return fail(VSIM_ERR_RANGE, "self contact needs bodies of at most 1023 cells per axis");
    s->selfContact = enabled != 0;
    s->frameDirty = true;
    return VSIM_OK;
}

int vsim_set_gravity(vsim_sim* s, const double g[3]) {
    SIM_GUARD(s);
    std::memcpy(s->gravity, g, sizeof s->gravity);
    s->frameDirty = true;
    return VSIM_OK;
}

int vsim_set_paused(vsim_sim* s, int paused) {
    SIM_GUARD(s);
    s->paused = paused != 0;
    return VSIM_OK;
}

int vsim_set_step_duration(vsim_sim* s, double seconds) {
    SIM_GUARD(s);
    if (!std::isfinite(seconds) || seconds <= 0)
        return fail(VSIM_ERR_RANGE, "stepDuration must be a finite positive number");
    s->clock.stepDuration = seconds;
    s->stepOverridden = true;
    s->paramsDirty = true;
    return VSIM_OK;
}

int vsim_set_iterations(vsim_sim* s, uint32_t iterations) {
    SIM_GUARD(s);
    if (iterations < 1 || iterations > 64) return fail(VSIM_ERR_RANGE, "iterations must be in [1, 64]");
    s->iterations = iterations;
    return VSIM_OK;
}

int vsim_set_graph(vsim_sim* s, int enabled) {
    SIM_GUARD(s);
    s->useGraph = enabled != 0;
    return VSIM_OK;
}

int vsim_set_launch_shape(vsim_sim* s, uint32_t block, uint32_t brick) {
    SIM_GUARD(s);
    if (block != 128 && block != 256 && block != 512) return fail(VSIM_ERR_RANGE, "block must be 128, 256 or 512");
    if (brick != 0 && brick != 4 && brick != 8) return fail(VSIM_ERR_RANGE, "brick must be 0, 4 or 8");
    s->block = block;
    if (brick != s->brick) {
        s->brick = brick;
        std::vector<uint4> cells;
        buildCells(s, cells);
        CK(cudaMemcpyAsync(s->d.cells, cells.data(), cells.size() * 16, cudaMemcpyHostToDevice, s->stream),
           "upload cells");
        CK(cudaStreamSynchronize(s->stream), "upload cells");
    }
    buildDensePlan(s);
    if (!s->plan.chunked) useDensePlan(s);
    return VSIM_OK;
}

int vsim_tune(vsim_sim* s, uint32_t frames, uint32_t* block, uint32_t* brick) {
    SIM_GUARD(s);
    if (frames < 1) frames = 1;
    const size_t N = s->nodeCount;
    std::vector<float> saved(12 * N);
    CK(cudaMemcpyAsync(saved.data(), s->d.pos, N * 16, cudaMemcpyDeviceToHost, s->stream), "tune");
    CK(cudaMemcpyAsync(saved.data() + 4 * N, s->d.prev, N * 16, cudaMemcpyDeviceToHost, s->stream), "tune");
    CK(cudaMemcpyAsync(saved.data() + 8 * N, s->d.vel, N * 16, cudaMemcpyDeviceToHost, s->stream), "tune");
    CK(cudaStreamSynchronize(s->stream), "tune");
    const uint32_t steps = std::max<uint32_t>(1, uint32_t(std::lround(1.0 / 60.0 / s->clock.stepDuration)));
    // Events are released, and the state and launch shape put back, on every
    // way out; a failed sweep leaves the shape the caller had.
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    const uint32_t callerBlock = s->block, callerBrick = s->brick;
    auto restore = [&](uint32_t bl, uint32_t br) {
        int rc = vsim_set_launch_shape(s, bl, br);
        cudaError_t e = cudaMemcpyAsync(s->d.pos, saved.data(), N * 16, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d.prev, saved.data() + 4 * N, N * 16, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d.vel, saved.data() + 8 * N, N * 16, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess && rc == VSIM_OK) rc = cudaFail(e, "tune: restore state");
        return rc;
    };
    // A failure inside the sweep: its error stays the reported one.
    auto abandon = [&](int rc) {
        const std::string why = vsim_last_error();
        restore(callerBlock, callerBrick);
        return fail(rc, why);
    };
    cudaError_t e;
    if ((e = cudaEventCreate(&ev.a)) || (e = cudaEventCreate(&ev.b))) return cudaFail(e, "tune");
    float best = INFINITY;
    uint32_t bestBlock = callerBlock, bestBrick = callerBrick;
    const uint32_t bricks[3] = {0, 4, 8}, blocksz[3] = {128, 256, 512};
    for (uint32_t br : bricks)
        for (uint32_t bl : blocksz) {
            int rc = vsim_set_launch_shape(s, bl, br);
            if (rc) return abandon(rc);
            rc = runFrame(s, steps);  // warm-up and graph capture
            if (rc) return abandon(rc);
            if ((e = cudaEventRecord(ev.a, s->stream))) return abandon(cudaFail(e, "tune"));
            for (uint32_t f = 0; f < frames; f++) {
                rc = runFrame(s, steps);
                if (rc) return abandon(rc);
            }
            if ((e = cudaEventRecord(ev.b, s->stream)) || (e = cudaEventSynchronize(ev.b)))
                return abandon(cudaFail(e, "tune"));
            float ms = 0;
            if ((e = cudaEventElapsedTime(&ms, ev.a, ev.b))) return abandon(cudaFail(e, "tune"));
            if (ms < best) {
                best = ms;
                bestBlock = bl;
                bestBrick = br;
            }
        }
    const int rc = restore(bestBlock, bestBrick);
    if (rc) return rc;
    if (block) *block = bestBlock;
    if (brick) *brick = bestBrick;
    return VSIM_OK;
}

int vsim_get_stats(vsim_sim* s, vsim_stats* o) {
    SIM_GUARD(s);
    if (!o) return fail(VSIM_ERR_INVALID, "out is NULL");
    std::memset(o, 0, sizeof *o);
    o->body_count = uint32_t(s->lat.size());
    o->nodes = s->nodeCount;
    uint32_t material = 0;
    for (float m : s->invMass) material += m > 0 ? 1 : 0;
    o->active_nodes = material;
    o->cells = s->cellCount;
    o->contact_nodes = s->surfaceCount;
    o->contact = s->contact;
    o->self_contact = s->selfContact;
    o->iterations = s->iterations;
    const vsim_clock_report r = s->clock.snapshot();
    o->steps = r.total_steps;
    o->last_steps = r.steps;
    o->max_steps_per_frame = r.max_steps_per_frame;
    o->step_duration = r.step_duration;
    o->simulated_time = r.simulated_time;
    o->backlog_time = r.backlog_time;
    o->frame_dropped_time = r.frame_dropped_time;
    o->dropped_time = r.dropped_time;
    o->overloaded = r.overloaded;
    int worst = -1;
    o->cfl = waveRateOf(s, &worst) * s->clock.stepDuration;
    o->limited_by = worst;
    o->driven = uint32_t(s->held.size());
    o->drive_capacity = VSIM_MAX_DRIVEN;
    return VSIM_OK;
}

int vsim_cfl_number(vsim_sim* s, double* out) {
    SIM_GUARD(s);
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    *out = waveRateOf(s, nullptr) * s->clock.stepDuration;
    return VSIM_OK;
}

int vsim_contact_pairs(vsim_sim* s, uint32_t* pairs, size_t capacity, size_t* count) {
    SIM_GUARD(s);
    if (!count) return fail(VSIM_ERR_INVALID, "count is NULL");
    *count = 0;
    if (s->surfaceCount == 0) return VSIM_OK;
    if (capacity > s->pairsCapacity) {
        if (s->pairs) cudaFree(s->pairs);
        s->pairs = nullptr;
        s->pairsCapacity = 0;
        CK(allocN(&s->pairs, 2 * capacity), "allocate pairs");
        s->pairsCapacity = capacity;
    }
    int rc = syncParams(s);
    if (rc) return rc;
    CK(cudaMemsetAsync(s->pairCount, 0, sizeof(unsigned long long), s->stream), "count pairs");
    const LaunchCtx c{s->stream, false, s->sms};
    CK(launchContact(c, s->d, s->dense.records, s->surfaceCount, s->gatherMapping, ContactMode::Pairs, s->pairs,
                     uint32_t(capacity), s->pairCount),
       "list pairs");
    unsigned long long total = 0;
    CK(cudaMemcpyAsync(&total, s->pairCount, sizeof total, cudaMemcpyDeviceToHost, s->stream), "count pairs");
    CK(cudaStreamSynchronize(s->stream), "count pairs");
    const size_t copied = std::min<size_t>(total, capacity);
    if (copied && pairs)
        CK(cudaMemcpy(pairs, s->pairs, copied * 8, cudaMemcpyDeviceToHost), "copy pairs");
    *count = size_t(total);
    return total > capacity ? fail(VSIM_ERR_CAPACITY, "pair buffer too small") : VSIM_OK;
}

int vsim_contact_census(vsim_sim* s, vsim_census* out) {
    SIM_GUARD(s);
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    std::memset(out, 0, sizeof *out);
    if (s->surfaceCount == 0 || !s->contact) return VSIM_OK;
    int rc = syncParams(s);
    if (rc) return rc;
    struct Marks {
        cudaEvent_t e[6] = {};
        ~Marks() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } m;
    for (cudaEvent_t& x : m.e) CK(cudaEventCreate(&x), "census events");
    unsigned long long* counts = s->pairCount + 1;
    CK(cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), s->stream), "census");
    const LaunchCtx c{s->stream, false, s->sms};
    CK(launchContact(c, s->d, s->dense.records, s->surfaceCount, s->gatherMapping, ContactMode::Solve, nullptr, 0,
                     nullptr, m.e),
       "census contact");
    CK(launchCensus(c, s->d, s->dense.records, counts), "census");
    unsigned long long host[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(host, counts, sizeof host, cudaMemcpyDeviceToHost, s->stream), "census");
    CK(cudaStreamSynchronize(s->stream), "census");
    out->records = host[0];
    out->candidates = host[1];
    out->occupied_buckets = host[2];
    for (int k = 0; k < 5; k++) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, m.e[k], m.e[k + 1]), "census timing");
        out->ms[k] = ms;
    }
    return VSIM_OK;
}

int vsim_contact_surface(vsim_sim* s, uint32_t* nodes, uint32_t* bodies, size_t capacity, size_t* count) {
    SIM_GUARD(s);
    if (count) *count = s->surfaceCount;
    const size_t n = std::min<size_t>(capacity, s->surfaceCount);
    for (size_t i = 0; i < n; i++) {
        if (nodes) nodes[i] = s->surfHost[i].x;
        if (bodies) bodies[i] = s->surfHost[i].y;
    }
    return capacity < s->surfaceCount ? fail(VSIM_ERR_CAPACITY, "surface buffer too small") : VSIM_OK;
}

int vsim_kuhn_rest_inverse(float out[54]) {
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    kuhnTable(out);
    return VSIM_OK;
}

int vsim_set_pdl(vsim_sim* s, int enabled) {
    SIM_GUARD(s);
    s->pdl = enabled != 0;
    return VSIM_OK;
}

int vsim_set_gather_mapping(vsim_sim* s, int mapping) {
    SIM_GUARD(s);
    if (mapping != VSIM_GATHER_AUTO && mapping != VSIM_GATHER_WARP && mapping != VSIM_GATHER_THREAD)
        return fail(VSIM_ERR_RANGE, "gather mapping must be VSIM_GATHER_AUTO, _WARP or _THREAD");
    s->gatherMapping = mapping;
    return VSIM_OK;
}

int vsim_color_counts(const vsim_sim* s, uint32_t out[8]) {
    if (!s || !out) return fail(VSIM_ERR_INVALID, "NULL argument");
    for (int c = 0; c < 8; c++) out[c] = s->colorStart[c + 1] - s->colorStart[c];
    return VSIM_OK;
}

uint32_t vsim_frame_launches(const vsim_sim* s, uint32_t steps) {
    if (!s) return 0;
    uint32_t colours = 0;
    for (int c = 0; c < 8; c++) colours += s->colorStart[c + 1] > s->colorStart[c] ? 1 : 0;
    uint32_t per = 1 + colours * s->iterations;
    if (anyStretch(s)) per += 3 * colours;
    if (s->contact && s->surfaceCount > 0) per += kContactKernels;
    return steps ? 1 + per * steps : 0;
}

uint32_t vsim_splat_launches(const vsim_sim* s) {
    if (!s || s->splatCount == 0) return 0;
    return 1 + radixSortLaunches(s->splatCount, 32);  // deformation, then the depth sort
}

int vsim_time_colour_passes(vsim_sim* s, uint32_t sweeps, float* ms) {
    SIM_GUARD(s);
    if (!ms) return fail(VSIM_ERR_INVALID, "ms is NULL");
    *ms = 0;
    if (sweeps < 1) return VSIM_OK;
    int rc = syncParams(s);
    if (rc) return rc;
    const size_t bytes = size_t(s->nodeCount) * 16;
    float4* saved = nullptr;
    CK(cudaMalloc(&saved, bytes), "save positions");
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool savedOk = false;
    auto body = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = cudaMemcpyAsync(saved, s->d.pos, bytes, cudaMemcpyDeviceToDevice, s->stream))) return e;
        savedOk = true;
        const LaunchCtx c{s->capture, s->pdl, s->sms, s->quadCells};
        const StretchLengths lens = stretchLengths();
        if ((e = cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal))) return e;
        cudaError_t enc = cudaSuccess;
        for (uint32_t sweep = 0; sweep < sweeps && enc == cudaSuccess; sweep++)
            for (int col = 0; col < 8 && enc == cudaSuccess; col++)
                if (s->plan.colour[col].grid) enc = launchColourPass(c, s, col, false, lens);
        const cudaError_t end = cudaStreamEndCapture(s->capture, &graph);
        if (enc) return enc;
        if (end) return end;
        if ((e = cudaGraphInstantiate(&exec, graph, 0))) return e;
        if ((e = cudaEventCreate(&e0)) || (e = cudaEventCreate(&e1))) return e;
        if ((e = cudaGraphLaunch(exec, s->stream))) return e;  // warm-up
        if ((e = cudaEventRecord(e0, s->stream))) return e;
        if ((e = cudaGraphLaunch(exec, s->stream))) return e;
        if ((e = cudaEventRecord(e1, s->stream))) return e;
        if ((e = cudaEventSynchronize(e1))) return e;
        return cudaEventElapsedTime(ms, e0, e1);
    };
    cudaError_t e = body();
    if (savedOk) {  // put back what the passes moved
        const cudaError_t back = cudaMemcpyAsync(s->d.pos, saved, bytes, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess) e = back;
    }
    cudaStreamSynchronize(s->stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(saved);
    CK(e, "time colour passes");
    return VSIM_OK;
}

int vsim_profile_frame(vsim_sim* s, uint32_t steps, int with_splats, const float view_dir[3], vsim_profile* out) {
    SIM_GUARD(s);
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    std::memset(out, 0, sizeof *out);
    if (steps < 1) return VSIM_OK;
    if (!s->held.empty()) {
        const double frameDt = steps * s->clock.stepDuration;
        for (int a = 0; a < 3; a++) s->grabVel[a] = (s->grabPos[a] - s->grabPrev[a]) / frameDt;
        std::memcpy(s->grabPrev, s->grabPos, sizeof s->grabPos);
        s->frameDirty = true;
    }
    int rc = syncParams(s);
    if (rc) return rc;
    Profiler prof;
    prof.stream = s->stream;
    const bool pdl = s->pdl;
    s->pdl = false;
    const cudaError_t enc = encodeFrame(s, s->stream, steps, ContactMode::Solve, &prof);
    s->pdl = pdl;
    CK(enc, "profile frame");
    if (with_splats && s->splatCount) {
        const float v[3] = {view_dir ? view_dir[0] : 0.0f, view_dir ? view_dir[1] : 0.0f,
                            view_dir ? view_dir[2] : -1.0f};
        prof.begin(VSIM_KIND_SPLAT, 1);
        CK(launchSplatDeform(s->stream, s->sp, s->d.pos, s->splatCount, v[0], v[1], v[2]), "profile splats");
        prof.end();
        prof.begin(VSIM_KIND_SORT, radixSortLaunches(s->splatCount, 32));
        CK(radixSortU32(s->sp.keys, s->sp.order, s->splatCount, 32, s->sp.sortTemp, s->sp.sortTempBytes, s->stream),
           "profile sort");
        prof.end();
    }
    CK(cudaStreamSynchronize(s->stream), "profile frame");
    for (const auto& sp : prof.spans) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, sp.a, sp.b), "profile timing");
        out->ms[sp.kind] += ms;
        out->launches[sp.kind] += sp.launches;
    }
    return VSIM_OK;
}

// ---- splats -------------------------------------------------------------

namespace {

int rebuildSplats(vsim_sim* s) {
    SplatState& sp = s->sp;
    void* old[] = {sp.embed,  sp.quat,  sp.scaleBody, sp.bodies,       sp.meanDepth, sp.cov,
                   sp.keys,   sp.order, sp.sortTemp,  sp.axesRotation, sp.axesScale};
    CK(cudaStreamSynchronize(s->stream), "rebind splats");
    for (void* p : old)
        if (p) cudaFree(p);
    sp = SplatState{};
    size_t total = 0;
    for (auto& m : s->splatMeans) total += m.size() / 3;
    if (total >= (1ull << 31)) return fail(VSIM_ERR_RANGE, "too many splats");
    s->splatCount = uint32_t(total);
    const size_t n = total;
    std::vector<float4> embed(n), quat(n), scaleBody(n);
    std::vector<SplatBody> bodies(s->lat.size());
    size_t at = 0;
    for (size_t b = 0; b < s->lat.size(); b++) {
        const Lattice& L = s->lat[b];
        // sample.wgsl:40-51 in f32: the uniforms deformOrigin and deformH.
        const float origin[3] = {float(L.origin[0]), float(L.origin[1]), float(L.origin[2])};
        const float inv = 1.0f / float(L.h);
        bodies[b] = SplatBody{L.nodeDims[0], L.nodeDims[0] * L.nodeDims[1], inv, 0};
        const std::vector<float>& m = s->splatMeans[b];
        const size_t count = m.size() / 3;
        for (size_t i = 0; i < count; i++, at++) {
            float local[3];
            uint32_t base[3];
            for (int a = 0; a < 3; a++) {
                const float grid = (m[3 * i + a] - origin[a]) * inv;
                const float cell = std::min(std::max(std::floor(grid), 0.0f), float(L.cellDims[a]) - 1.0f);
                local[a] = grid - cell;
                base[a] = uint32_t(cell);
            }
            const uint32_t node = s->offsets[b] + base[0] + L.nodeDims[0] * (base[1] + L.nodeDims[1] * base[2]);
            float nodeBits, bodyBits;
            std::memcpy(&nodeBits, &node, 4);
            const uint32_t body = uint32_t(b);
            std::memcpy(&bodyBits, &body, 4);
            embed[at] = make_float4(local[0], local[1], local[2], nodeBits);
            const std::vector<float>& q = s->splatQuats[b];
            const std::vector<float>& sc = s->splatScales[b];
            quat[at] = make_float4(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
            scaleBody[at] = make_float4(sc[3 * i], sc[3 * i + 1], sc[3 * i + 2], bodyBits);
        }
    }
    if (n == 0) return VSIM_OK;
    CK(allocN(&sp.embed, n), "allocate splats");
    CK(allocN(&sp.quat, n), "allocate splats");
    CK(allocN(&sp.scaleBody, n), "allocate splats");
    CK(allocN(&sp.bodies, bodies.size()), "allocate splats");
    CK(allocN(&sp.meanDepth, n), "allocate splats");
    CK(allocN(&sp.cov, 3 * n), "allocate splats");
    CK(allocN(&sp.keys, n), "allocate splats");
    CK(allocN(&sp.order, n), "allocate splats");
    sp.sortTempBytes = radixSortTempBytes(uint32_t(n));
    CK(cudaMalloc(&sp.sortTemp, sp.sortTempBytes), "allocate sort scratch");
    CK(cudaMemcpyAsync(sp.embed, embed.data(), n * 16, cudaMemcpyHostToDevice, s->stream), "upload splats");
    CK(cudaMemcpyAsync(sp.quat, quat.data(), n * 16, cudaMemcpyHostToDevice, s->stream), "upload splats");
    CK(cudaMemcpyAsync(sp.scaleBody, scaleBody.data(), n * 16, cudaMemcpyHostToDevice, s->stream), "upload splats");
    CK(cudaMemcpyAsync(sp.bodies, bodies.data(), bodies.size() * sizeof(SplatBody), cudaMemcpyHostToDevice,
                       s->stream),
       "upload splats");
    CK(cudaStreamSynchronize(s->stream), "upload splats");
    return VSIM_OK;
}

}  // namespace

int vsim_splats_bind(vsim_sim* s, uint32_t body, const float* means, const float* quats, const float* scales,
                     uint32_t count) {
    SIM_GUARD(s);
    if (body >= s->lat.size()) return fail(VSIM_ERR_RANGE, "body index out of range");
    if (count && (!means || !quats || !scales)) return fail(VSIM_ERR_INVALID, "splat arrays are NULL");
    s->splatMeans[body].assign(means, means + 3 * size_t(count));
    s->splatQuats[body].assign(quats, quats + 4 * size_t(count));
    s->splatScales[body].assign(scales, scales + 3 * size_t(count));
    return rebuildSplats(s);
}

uint32_t vsim_splats_count(const vsim_sim* s) { return s ? s->splatCount : 0; }

int vsim_splats_deform(vsim_sim* s, const float view_dir[3]) {
    SIM_GUARD(s);
    if (!view_dir) return fail(VSIM_ERR_INVALID, "view_dir is NULL");
    if (s->splatCount == 0) return VSIM_OK;
    CK(launchSplatDeform(s->stream, s->sp, s->d.pos, s->splatCount, view_dir[0], view_dir[1], view_dir[2]),
       "deform splats");
    return VSIM_OK;
}

int vsim_splats_deform_axes(vsim_sim* s, const float view_dir[3]) {
    SIM_GUARD(s);
    if (!view_dir) return fail(VSIM_ERR_INVALID, "view_dir is NULL");
    if (s->splatCount == 0) return VSIM_OK;
    if (!s->sp.axesRotation) {
        CK(allocN(&s->sp.axesRotation, s->splatCount), "allocate splat axes");
        CK(allocN(&s->sp.axesScale, s->splatCount), "allocate splat axes");
    }
    CK(launchSplatDeform(s->stream, s->sp, s->d.pos, s->splatCount, view_dir[0], view_dir[1], view_dir[2], true),
       "deform splats");
    return VSIM_OK;
}

int vsim_splats_read_axes(vsim_sim* s, float* rotation, float* scale, size_t count) {
    SIM_GUARD(s);
    if (count != s->splatCount) return fail(VSIM_ERR_CAPACITY, "count does not match the bound splats");
    if (count == 0) return VSIM_OK;
    if (!s->sp.axesRotation) return fail(VSIM_ERR_INVALID, "no axes yet: call vsim_splats_deform_axes first");
    std::vector<float4> rot(count), sc(count);
    CK(cudaMemcpyAsync(rot.data(), s->sp.axesRotation, count * 16, cudaMemcpyDeviceToHost, s->stream), "read axes");
    CK(cudaMemcpyAsync(sc.data(), s->sp.axesScale, count * 16, cudaMemcpyDeviceToHost, s->stream), "read axes");
    CK(cudaStreamSynchronize(s->stream), "read axes");
    for (size_t i = 0; i < count; i++) {
        if (rotation) {
            rotation[4 * i] = rot[i].x;
            rotation[4 * i + 1] = rot[i].y;
            rotation[4 * i + 2] = rot[i].z;
            rotation[4 * i + 3] = rot[i].w;
        }
        if (scale) {
            scale[3 * i] = sc[i].x;
            scale[3 * i + 1] = sc[i].y;
            scale[3 * i + 2] = sc[i].z;
        }
    }
    return VSIM_OK;
}

int vsim_splats_sort(vsim_sim* s) {
    SIM_GUARD(s);
    if (s->splatCount == 0) return VSIM_OK;
    CK(radixSortU32(s->sp.keys, s->sp.order, s->splatCount, 32, s->sp.sortTemp, s->sp.sortTempBytes, s->stream),
       "sort splats");
    return VSIM_OK;
}

int vsim_splats_read(vsim_sim* s, float* means, float* cov6, uint32_t* order, size_t count) {
    SIM_GUARD(s);
    if (count != s->splatCount) return fail(VSIM_ERR_CAPACITY, "count does not match the bound splats");
    if (count == 0) return VSIM_OK;
    if (means || cov6) {
        std::vector<float4> md(count);
        std::vector<float2> cv(3 * count);
        CK(cudaMemcpyAsync(md.data(), s->sp.meanDepth, count * 16, cudaMemcpyDeviceToHost, s->stream), "read splats");
        CK(cudaMemcpyAsync(cv.data(), s->sp.cov, count * 24, cudaMemcpyDeviceToHost, s->stream), "read splats");
        CK(cudaStreamSynchronize(s->stream), "read splats");
        for (size_t i = 0; i < count; i++) {
            if (means) {
                means[3 * i] = md[i].x;
                means[3 * i + 1] = md[i].y;
                means[3 * i + 2] = md[i].z;
            }
            if (cov6) {
                cov6[6 * i] = cv[3 * i].x;
                cov6[6 * i + 1] = cv[3 * i].y;
                cov6[6 * i + 2] = cv[3 * i + 1].x;
                cov6[6 * i + 3] = cv[3 * i + 1].y;
                cov6[6 * i + 4] = cv[3 * i + 2].x;
                cov6[6 * i + 5] = cv[3 * i + 2].y;
            }
        }
    }
    if (order) {
        CK(cudaMemcpyAsync(order, s->sp.order, count * 4, cudaMemcpyDeviceToHost, s->stream), "read order");
        CK(cudaStreamSynchronize(s->stream), "read order");
    }
    return VSIM_OK;
}

int vsim_radix_sort_u32(const uint32_t* d_keys, uint32_t* d_order, uint32_t n, uint32_t key_bits, void* d_temp,
                        size_t* temp_bytes, void* stream) {
    clearError();
    if (!temp_bytes) return fail(VSIM_ERR_INVALID, "temp_bytes is NULL");
    if (key_bits < 1 || key_bits > 32) return fail(VSIM_ERR_RANGE, "key_bits must be in [1, 32]");
    const size_t need = radixSortTempBytes(n);
    if (!d_temp) {
        *temp_bytes = need;
        return VSIM_OK;
    }
    if (*temp_bytes < need) return fail(VSIM_ERR_CAPACITY, "scratch smaller than the size query returned");
    if (n == 0) return VSIM_OK;
    if (!d_keys || !d_order) return fail(VSIM_ERR_INVALID, "keys or order is NULL");
    if (wordRangesOverlap(d_keys, d_order, n)) return fail(VSIM_ERR_INVALID, "keys and order overlap");
    CK(radixSortU32(d_keys, d_order, n, key_bits, d_temp, *temp_bytes, static_cast<cudaStream_t>(stream)),
       "radix sort");
    return VSIM_OK;
}

}  // extern "C"
