// Serving: a pool of sessions resident on the device, stepped in shared
// frames. No counterpart in the reference (its Simulator serves one page).
//
// The resident sessions live in one simulator created with isolated bodies
// (each session is a body with its own contact grid), so a frame's kernels
// run over every session at once. A tick picks the sessions with a pending
// request, marks them active (the rest sit the frame out untouched), sets
// their drag targets, runs one frame and retires the requests it finished.
// Requests that arrive while a frame runs are queued and join at the next
// tick: batching is per frame, continuously, not per request.
//
// Sessions keep their ids; which of them are resident can change between
// ticks (vsim_server_set_resident): the server holds every session's
// description, checkpoints the state of those that leave to host memory,
// and rebuilds the device pool for the new set with every session's state
// restored.
//
// A session's arithmetic never reads another session's data: bodies own
// disjoint node ranges, their contact grids are disjoint, and inactive bodies
// are skipped by every kernel. So a request's result is the same whether it
// ran alone or among others.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <thread>

#include "sim_internal.cuh"

using namespace vsim;

namespace {

struct Request {
    uint64_t id = 0;
    uint32_t session = 0;
    uint32_t frames = 0;
    uint32_t done = 0;
    bool drag = false;
    vsim_drag path{};
    double t = 0;  // curve parameter of the drag target
    double submitted = 0;
    uint64_t firstTick = 0;
};

// Cubic Bezier position and derivative.
void bezier(const float c[4][3], double t, double p[3], double dp[3]) {
    const double u = 1 - t;
    for (int a = 0; a < 3; a++) {
        p[a] = u * u * u * c[0][a] + 3 * u * u * t * c[1][a] + 3 * u * t * t * c[2][a] + t * t * t * c[3][a];
        dp[a] = 3 * u * u * (c[1][a] - c[0][a]) + 6 * u * t * (c[2][a] - c[1][a]) + 3 * t * t * (c[3][a] - c[2][a]);
    }
}

}  // namespace

struct vsim_server;

namespace {

// A session as offered: its body, copied, and what admission charges.
struct Session {
    vsim_body_desc desc{};
    std::vector<uint8_t> occupancy;
    std::vector<uint32_t> statics;
    double bytes = 0;
    uint32_t cells = 0;
    uint32_t nodes = 0;
    // The state it left the device with (empty: never run, or resident).
    std::vector<float> pos, prev, vel;
};

int applyHolds(vsim_server* s);

}  // namespace

struct vsim_server {
    vsim_sim* sim = nullptr;
    vsim_tank world{};
    vsim_server_config config{};
    void* stream = nullptr;
    std::vector<Session> sessions;
    std::vector<uint32_t> resident;  // session of each body of `sim`
    std::vector<int32_t> slot;       // body of each session in `sim`, -1 when not resident
    uint32_t rejected = 0;
    double residentBytes = 0;
    std::vector<std::deque<Request>> queue;  // per session
    std::vector<int64_t> held;               // per session: session-local node its drag holds, -1 for none
    std::vector<double> prevTarget;          // 3 per session
    std::vector<vsim_completion> completed;
    uint64_t ticks = 0, nextId = 1, sessionFrames = 0, cellUpdates = 0;
    uint32_t pending = 0;
    double tickSeconds = 0, prepareSeconds = 0, frameSeconds = 0;
    uint64_t tickCellBudget = 0;  // cells one tick may step; 0: every session with a pending request
    std::chrono::steady_clock::time_point origin = std::chrono::steady_clock::now();
    cudaEvent_t frameStart = nullptr, frameDone = nullptr;
};

namespace {

// Holds exactly the nodes the resident sessions' drags name.
int applyHolds(vsim_server* s) {
    std::vector<uint32_t> nodes;
    for (uint32_t b = 0; b < s->resident.size(); b++) {
        const int64_t local = s->held[s->resident[b]];
        if (local >= 0) nodes.push_back(s->sim->offsets[b] + uint32_t(local));
    }
    const std::vector<float> zero(3 * nodes.size(), 0.0f);
    return nodes.empty() ? releaseNodes(s->sim) : holdNodes(s->sim, nodes.data(), zero.data(), uint32_t(nodes.size()));
}

int residentBody(const vsim_server* s, uint32_t session, uint32_t& body) {
    if (session >= s->sessions.size() || s->slot[session] < 0) return fail(VSIM_ERR_RANGE, "session is not resident");
    body = uint32_t(s->slot[session]);
    return VSIM_OK;
}

// A session's state may be read, replaced or reset only between its
// requests; a drag it still holds from its last request is let go first.
int idleSession(vsim_server* s, uint32_t session) {
    uint32_t body;
    if (int rc = residentBody(s, session, body)) return rc;
    if (!s->queue[session].empty()) return fail(VSIM_ERR_INVALID, "session has requests pending");
    if (s->held[session] >= 0) {
        s->held[session] = -1;
        return applyHolds(s);
    }
    return VSIM_OK;
}

double seconds(const vsim_server* s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->origin).count();
}

// Device bytes one isolated session holds (what admission charges).
double sessionBytes(const Lattice& L, const Grid& g) {
    const double nodes = L.nodeCount, surface = double(L.surface.size());
    return nodes * (3 * 16 + 4 * 4)            // pos, prev, vel; mass, active list, body, record
           + double(L.cellCount) * 16          // cell records
           + surface * (16 + 4 + 4 + 4 + 16 + 16 + 16 + 16 + 4 + 4)  // record, key, rank, entry, correction, runs
           + double(g.count()) * 8             // bucket counts and starts
           + sizeof(DevBody) + 2 * 16 + 4;     // constants, drag target, activity
}

void dropSim(vsim_sim*& sim) {
    if (!sim) return;
    DeviceGuard guard(sim->device);
    cudaStreamSynchronize(sim->stream);
    freeSim(sim);
    delete sim;
    sim = nullptr;
}

int destroyServer(vsim_server* s) {
    if (s->sim) {
        DeviceGuard guard(s->sim->device);
        cudaStreamSynchronize(s->sim->stream);
        if (s->frameStart) cudaEventDestroy(s->frameStart);
        if (s->frameDone) cudaEventDestroy(s->frameDone);
    }
    dropSim(s->sim);
    delete s;
    return VSIM_OK;
}

// A simulator over `members` (session ids, in body order), set up as the
// server runs it: the server's substep, self contact, a drag target per
// body, every body sitting out until a request names it.
int buildPool(vsim_server* s, const std::vector<uint32_t>& members, vsim_sim** out) {
    *out = nullptr;
    std::vector<vsim_body_desc> descs;
    descs.reserve(members.size());
    for (uint32_t q : members) descs.push_back(s->sessions[q].desc);
    auto* sim = new (std::nothrow) vsim_sim();
    if (!sim) return fail(VSIM_ERR_NOMEM, "out of host memory");
    int rc;
    try {
        rc = createSim(descs.data(), uint32_t(descs.size()), &s->world, s->stream, true, sim);
    } catch (const std::bad_alloc&) {
        rc = fail(VSIM_ERR_NOMEM, "out of host memory");
    }
    if (rc) {
        dropSim(sim);
        return rc;
    }
    sim->clock.stepDuration = s->config.step_duration;
    sim->stepOverridden = true;
    sim->selfContact = s->config.self_contact != 0;
    sim->perBodyGrab = true;
    std::fill(sim->activeHost.begin(), sim->activeHost.end(), 0u);
    sim->tablesDirty = sim->paramsDirty = sim->frameDirty = true;
    *out = sim;
    return VSIM_OK;
}

}  // namespace

extern "C" {

int vsim_server_create(const vsim_body_desc* sessions, uint32_t count, const vsim_tank* tank,
                       const vsim_server_config* config, void* stream, vsim_server** out) {
    clearError();
    if (!out || !config) return fail(VSIM_ERR_INVALID, "out or config is NULL");
    *out = nullptr;
    if (count > 0 && !sessions) return fail(VSIM_ERR_INVALID, "sessions is NULL");
    if (!std::isfinite(config->step_duration) || config->step_duration <= 0)
        return fail(VSIM_ERR_RANGE, "step_duration must be a finite positive number");
    if (config->substeps < 1) return fail(VSIM_ERR_RANGE, "substeps must be at least 1");
    vsim_server* s = new (std::nothrow) vsim_server();
    if (!s) return fail(VSIM_ERR_NOMEM, "out of host memory");
    s->config = *config;
    s->stream = stream;
    for (int a = 0; a < 3; a++) {
        s->world.min[a] = tank ? tank->min[a] : -INFINITY;
        s->world.max[a] = tank ? tank->max[a] : INFINITY;
    }
    // Every session's body, copied; admission: in order while their device
    // state fits the budget.
    std::vector<uint32_t> admitted;
    try {
        s->sessions.resize(count);
        bool full = false;
        for (uint32_t i = 0; i < count; i++) {
            Lattice L;
            int rc = buildLattice(sessions[i], L);
            if (rc) {
                destroyServer(s);
                return rc;
            }
            Session& q = s->sessions[i];
            const vsim_body_desc& d = sessions[i];
            const size_t cells = size_t(d.cell_dims[0]) * d.cell_dims[1] * d.cell_dims[2];
            q.occupancy.assign(d.occupancy, d.occupancy + cells);
            if (d.static_count) q.statics.assign(d.static_nodes, d.static_nodes + d.static_count);
            q.desc = d;
            q.desc.occupancy = q.occupancy.data();
            q.desc.static_nodes = q.statics.empty() ? nullptr : q.statics.data();
            q.bytes = sessionBytes(L, bodyGrid(L, s->world));
            q.cells = L.cellCount;
            q.nodes = L.nodeCount;
            if (full || (config->hbm_budget_bytes > 0 && s->residentBytes + q.bytes > config->hbm_budget_bytes)) {
                full = true;
                continue;
            }
            s->residentBytes += q.bytes;
            admitted.push_back(i);
        }
        s->slot.assign(count, -1);
        s->queue.resize(count);
        s->held.assign(count, -1);
        s->prevTarget.assign(3 * size_t(count), 0.0);
    } catch (const std::bad_alloc&) {
        destroyServer(s);
        return fail(VSIM_ERR_NOMEM, "out of host memory");
    }
    s->rejected = count - uint32_t(admitted.size());
    if (int rc = buildPool(s, admitted, &s->sim)) {
        destroyServer(s);
        return rc;
    }
    s->resident = admitted;
    for (uint32_t b = 0; b < admitted.size(); b++) s->slot[admitted[b]] = int32_t(b);
    DeviceGuard guard(s->sim->device);
    if (cudaEventCreate(&s->frameStart) != cudaSuccess || cudaEventCreate(&s->frameDone) != cudaSuccess) {
        destroyServer(s);
        return fail(VSIM_ERR_CUDA, "create event");
    }
    *out = s;
    return VSIM_OK;
}

int vsim_server_destroy(vsim_server* server) {
    if (!server) return VSIM_OK;
    return destroyServer(server);
}

uint32_t vsim_server_admitted(const vsim_server* s) { return s ? uint32_t(s->resident.size()) : 0; }

int vsim_server_resident(const vsim_server* s, uint32_t* sessions, uint32_t capacity, uint32_t* count) {
    clearError();
    if (!s || !count) return fail(VSIM_ERR_INVALID, "NULL argument");
    *count = uint32_t(s->resident.size());
    if (!sessions) return VSIM_OK;
    if (capacity < s->resident.size()) return fail(VSIM_ERR_CAPACITY, "capacity below the resident count");
    std::copy(s->resident.begin(), s->resident.end(), sessions);
    return VSIM_OK;
}

int vsim_server_set_resident(vsim_server* s, const uint32_t* sessions, uint32_t count) {
    clearError();
    if (!s || (count > 0 && !sessions)) return fail(VSIM_ERR_INVALID, "NULL argument");
    const uint32_t total = uint32_t(s->sessions.size());
    std::vector<uint8_t> chosen(total, 0);
    double bytes = 0;
    for (uint32_t k = 0; k < count; k++) {
        const uint32_t q = sessions[k];
        if (q >= total) return fail(VSIM_ERR_RANGE, "no such session");
        if (chosen[q]) return fail(VSIM_ERR_INVALID, "a session is listed twice");
        chosen[q] = 1;
        bytes += s->sessions[q].bytes;
    }
    if (s->config.hbm_budget_bytes > 0 && bytes > s->config.hbm_budget_bytes)
        return fail(VSIM_ERR_NOMEM, "the sessions' device state exceeds the HBM budget");
    for (uint32_t q : s->resident)
        if (!chosen[q] && !s->queue[q].empty())
            return fail(VSIM_ERR_INVALID, "a session leaving the device has requests pending");
    vsim_sim* old = s->sim;
    DeviceGuard guard(old->device);
    // Checkpoint every resident session (those staying come back as they
    // were), with every drag let go: the next tick holds what requests name.
    {
        const size_t n = old->nodeCount;
        std::vector<float> pos(4 * n), prev(4 * n), vel(4 * n);
        float* const out[3] = {pos.data(), prev.data(), vel.data()};
        if (n) {
            if (int rc = readNodes(old, 0, n, out)) return rc;
        }
        for (uint32_t b = 0; b < s->resident.size(); b++) {
            Session& q = s->sessions[s->resident[b]];
            const size_t first = 4 * size_t(old->offsets[b]), len = 4 * size_t(q.nodes);
            q.pos.assign(pos.begin() + first, pos.begin() + first + len);
            q.prev.assign(prev.begin() + first, prev.begin() + first + len);
            q.vel.assign(vel.begin() + first, vel.begin() + first + len);
        }
    }
    std::vector<uint32_t> members(sessions, sessions + count);
    vsim_sim* next = nullptr;
    if (int rc = buildPool(s, members, &next)) return rc;  // the old pool is untouched on failure
    // States back: each member's checkpoint, or its rest state if it has none.
    {
        const size_t n = next->nodeCount;
        std::vector<float> pos(next->restPos), prev(next->restPos), vel(4 * n, 0.0f);
        for (uint32_t b = 0; b < count; b++) {
            Session& q = s->sessions[members[b]];
            if (q.pos.empty()) continue;
            const size_t first = 4 * size_t(next->offsets[b]);
            std::copy(q.pos.begin(), q.pos.end(), pos.begin() + first);
            std::copy(q.prev.begin(), q.prev.end(), prev.begin() + first);
            std::copy(q.vel.begin(), q.vel.end(), vel.begin() + first);
        }
        int rc = VSIM_OK;
        if (n) {
            rc = vsim_write_state(next, pos.data(), prev.data(), vel.data(), n);
        }
        if (rc) {
            dropSim(next);
            return rc;
        }
    }
    for (uint32_t b = 0; b < count; b++) {
        Session& q = s->sessions[members[b]];
        std::vector<float>().swap(q.pos);  // resident again: the device holds it
        std::vector<float>().swap(q.prev);
        std::vector<float>().swap(q.vel);
    }
    for (uint32_t q : s->resident) s->held[q] = -1;
    std::fill(s->slot.begin(), s->slot.end(), -1);
    for (uint32_t b = 0; b < count; b++) s->slot[members[b]] = int32_t(b);
    s->resident = members;
    s->residentBytes = bytes;
    s->sim = next;
    dropSim(old);
    return VSIM_OK;
}

double vsim_server_clock(const vsim_server* s) { return s ? seconds(s) : 0.0; }

}  // extern "C"

namespace {

// Queues a request stamped as submitted at `submitted` (server clock).
int submitAt(vsim_server* s, uint32_t session, uint32_t frames, const vsim_drag* drag, double submitted,
             uint64_t* request) {
    uint32_t body;
    if (int rc = residentBody(s, session, body)) return rc;
    if (frames < 1) return fail(VSIM_ERR_RANGE, "frames must be at least 1");
    Request r;
    r.id = s->nextId++;
    r.session = session;
    r.frames = frames;
    r.submitted = submitted;
    if (drag) {
        const vsim_sim* sim = s->sim;
        if (drag->node >= sim->lat[body].nodeCount) return fail(VSIM_ERR_RANGE, "drag node outside the session");
        const uint32_t global = sim->offsets[body] + drag->node;
        if (sim->invMass[global] <= 0 || sim->isStatic[global])
            return fail(VSIM_ERR_INVALID, "[drive] drag node is empty or static");
        if (!std::isfinite(drag->speed) || drag->speed < 0) return fail(VSIM_ERR_RANGE, "drag speed must be finite");
        r.drag = true;
        r.path = *drag;
    }
    s->queue[session].push_back(r);
    s->pending++;
    if (request) *request = r.id;
    return VSIM_OK;
}

}  // namespace

extern "C" {

int vsim_server_submit(vsim_server* s, uint32_t session, uint32_t frames, const vsim_drag* drag, uint64_t* request) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    return submitAt(s, session, frames, drag, seconds(s), request);
}

int vsim_server_tick(vsim_server* s, uint32_t* stepped) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    if (stepped) *stepped = 0;
    vsim_sim* sim = s->sim;
    DeviceGuard guard(sim->device);
    const double frameDt = s->config.substeps * s->config.step_duration;
    const double entered = seconds(s);
    const uint32_t bodies = uint32_t(s->resident.size());

    // The sessions this frame runs: every one with a pending request, or,
    // under a tick budget, those whose requests already run (oldest first)
    // and then waiting ones in arrival order while their cells fit.
    std::vector<uint8_t> runs(bodies, 0);
    {
        std::vector<uint32_t> started, waiting;
        for (uint32_t b = 0; b < bodies; b++) {
            const auto& q = s->queue[s->resident[b]];
            if (q.empty()) continue;
            (q.front().done > 0 ? started : waiting).push_back(b);
        }
        if (s->tickCellBudget == 0) {
            for (uint32_t b : started) runs[b] = 1;
            for (uint32_t b : waiting) runs[b] = 1;
        } else {
            auto front = [&](uint32_t b) -> const Request& { return s->queue[s->resident[b]].front(); };
            std::sort(started.begin(), started.end(), [&](uint32_t x, uint32_t y) {
                return front(x).firstTick != front(y).firstTick ? front(x).firstTick < front(y).firstTick
                                                                : front(x).id < front(y).id;
            });
            std::sort(waiting.begin(), waiting.end(), [&](uint32_t x, uint32_t y) { return front(x).id < front(y).id; });
            uint64_t cells = 0;
            bool any = false;
            for (const std::vector<uint32_t>* list : {&started, &waiting})
                for (uint32_t b : *list) {
                    const uint64_t c = s->sessions[s->resident[b]].cells;
                    if (any && cells + c > s->tickCellBudget) continue;
                    runs[b] = 1;
                    cells += c;
                    any = true;
                }
        }
    }
    // The nodes their drags hold (a session left out keeps what it holds).
    bool holdChanged = false;
    uint32_t active = 0;
    for (uint32_t b = 0; b < bodies; b++) {
        const uint32_t i = s->resident[b];
        const bool busy = runs[b] != 0;
        const int64_t want = !busy                          ? s->held[i]
                             : s->queue[i].front().drag ? int64_t(s->queue[i].front().path.node)
                                                        : int64_t(-1);
        if (want != s->held[i]) {
            holdChanged = true;
            s->held[i] = want;
        }
        if (busy && want >= 0 && s->queue[i].front().done == 0) {
            // A request's drag starts on its curve (the grab's placement),
            // whatever the session held before.
            double p[3], dp[3];
            bezier(s->queue[i].front().path.control, 0.0, p, dp);
            for (int a = 0; a < 3; a++) s->prevTarget[3 * i + a] = p[a];
        }
        const uint32_t flag = busy ? 1u : 0u;
        if (sim->activeHost[b] != flag) {
            sim->activeHost[b] = flag;
            sim->tablesDirty = true;
        }
        active += flag;
    }
    if (active == 0) return VSIM_OK;
    if (holdChanged) {
        const int rc = applyHolds(s);
        if (rc) return rc;
    }
    // Drag targets advance one frame along their curves at their speed;
    // velocity is this frame's motion over its duration (simulator.js:309-315).
    for (uint32_t b = 0; b < bodies; b++) {
        const uint32_t i = s->resident[b];
        if (!runs[b] || s->held[i] < 0) continue;
        Request& r = s->queue[i].front();
        double p[3], dp[3];
        bezier(r.path.control, r.t, p, dp);
        const double rate = std::sqrt(dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
        r.t = std::min(1.0, r.t + r.path.speed * frameDt / std::max(rate, 1e-9));
        bezier(r.path.control, r.t, p, dp);
        float4 target = make_float4(float(p[0]), float(p[1]), float(p[2]), 0.0f);
        float4 velocity = make_float4(float((p[0] - s->prevTarget[3 * i]) / frameDt),
                                      float((p[1] - s->prevTarget[3 * i + 1]) / frameDt),
                                      float((p[2] - s->prevTarget[3 * i + 2]) / frameDt), 0.0f);
        for (int a = 0; a < 3; a++) s->prevTarget[3 * i + a] = p[a];
        sim->grabsHost[2 * b] = target;
        sim->grabsHost[2 * b + 1] = velocity;
        sim->tablesDirty = true;
    }
    // Launch over the active sessions' ranges only.
    std::vector<uint32_t> activeBodies;
    activeBodies.reserve(active);
    for (uint32_t b = 0; b < bodies; b++)
        if (sim->activeHost[b]) activeBodies.push_back(b);
    int rc = planBodies(sim, activeBodies);
    if (rc) return rc;
    rc = syncParams(sim);
    if (rc) return rc;
    s->prepareSeconds += seconds(s) - entered;
    CK(cudaEventRecord(s->frameStart, sim->stream), "serve frame");
    rc = runFrame(sim, s->config.substeps);
    if (rc) return rc;
    CK(cudaEventRecord(s->frameDone, sim->stream), "serve frame");
    CK(cudaEventSynchronize(s->frameDone), "serve frame");
    float frameMs = 0;
    if (cudaEventElapsedTime(&frameMs, s->frameStart, s->frameDone) == cudaSuccess) s->frameSeconds += 1e-3 * frameMs;
    const double now = seconds(s);
    for (uint32_t b = 0; b < bodies; b++) {
        if (!sim->activeHost[b]) continue;
        const uint32_t i = s->resident[b];
        Request& r = s->queue[i].front();
        if (r.done == 0) r.firstTick = s->ticks;
        r.done++;
        s->sessionFrames++;
        s->cellUpdates += uint64_t(s->sessions[i].cells) * s->config.substeps;
        if (r.done == r.frames) {
            s->completed.push_back(vsim_completion{r.id, r.session, r.frames, r.submitted, now, r.firstTick, s->ticks});
            s->queue[i].pop_front();
            s->pending--;
        }
    }
    s->ticks++;
    s->tickSeconds += seconds(s) - entered;
    if (stepped) *stepped = active;
    return VSIM_OK;
}

int vsim_server_run(vsim_server* s, const vsim_scheduled_request* requests, uint32_t n, const vsim_drag* drags,
                    double closed_loop_seconds, vsim_completion* out, uint32_t capacity, vsim_run_report* report) {
    clearError();
    if (!s || (n > 0 && !requests)) return fail(VSIM_ERR_INVALID, "server or requests is NULL");
    if (!(closed_loop_seconds >= 0) || !std::isfinite(closed_loop_seconds))
        return fail(VSIM_ERR_RANGE, "closed_loop_seconds must be finite and not negative");
    const bool closed = closed_loop_seconds > 0;
    if (closed && n == 0) return fail(VSIM_ERR_INVALID, "a closed-loop run needs requests to draw from");
    if (s->pending) return fail(VSIM_ERR_INVALID, "requests are already pending");
    for (uint32_t i = 0; i < n; i++)
        if (requests[i].drag && !drags) return fail(VSIM_ERR_INVALID, "a request drags but drags is NULL");
    std::vector<vsim_completion> done;
    const uint64_t frames0 = s->sessionFrames, ticks0 = s->ticks;
    uint64_t requestsDone = 0;
    uint32_t next = 0;
    auto spec = [&](uint32_t session, const vsim_scheduled_request& q, double at) {
        return submitAt(s, session, q.frames, q.drag ? &drags[session] : nullptr, at, nullptr);
    };
    const double t0 = seconds(s);
    int rc = VSIM_OK;
    bool windowClosed = false;
    uint64_t windowRequests = 0, windowFrames = 0, windowTicks = 0;
    double windowSeconds = 0;
    if (closed) {
        for (uint32_t session : s->resident) {
            if ((rc = spec(session, requests[next], seconds(s)))) return rc;
            next = (next + 1) % n;
        }
    }
    while (true) {
        const double now = seconds(s);
        if (!closed)
            while (next < n && t0 + requests[next].arrival <= now) {
                if ((rc = spec(requests[next].session, requests[next], t0 + requests[next].arrival))) return rc;
                next++;
            }
        if (s->pending) {
            if ((rc = vsim_server_tick(s, nullptr))) return rc;
            const bool refill = closed && seconds(s) - t0 < closed_loop_seconds;
            if (closed && !refill && !windowClosed) {  // the closed loop's measured span ends here
                windowClosed = true;
                windowRequests = requestsDone + s->completed.size();
                windowFrames = s->sessionFrames - frames0;
                windowTicks = s->ticks - ticks0;
                windowSeconds = seconds(s) - t0;
            }
            for (const vsim_completion& c : s->completed) {
                requestsDone++;
                if (out && done.size() < capacity) done.push_back(c);
                if (refill) {
                    if ((rc = spec(c.session, requests[next], seconds(s)))) return rc;
                    next = (next + 1) % n;
                }
            }
            s->completed.clear();
            continue;
        }
        if (closed || next >= n) break;
        // Idle until the next arrival: sleep while it is far, then spin.
        const double wait = t0 + requests[next].arrival - seconds(s);
        if (wait > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(wait - 1e-4));
    }
    if (out) std::copy(done.begin(), done.end(), out);
    if (report) {
        report->requests = closed ? windowRequests : requestsDone;
        report->returned = uint32_t(done.size());
        report->frames = closed ? windowFrames : s->sessionFrames - frames0;
        report->ticks = closed ? windowTicks : s->ticks - ticks0;
        report->seconds = closed ? windowSeconds : seconds(s) - t0;
    }
    return VSIM_OK;
}

int vsim_server_set_tick_budget(vsim_server* s, uint64_t cells) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    s->tickCellBudget = cells;
    return VSIM_OK;
}

int vsim_server_poll(vsim_server* s, vsim_completion* out, uint32_t capacity, uint32_t* count) {
    clearError();
    if (!s || !count) return fail(VSIM_ERR_INVALID, "NULL argument");
    const uint32_t n = std::min<uint32_t>(capacity, uint32_t(s->completed.size()));
    if (n && out) std::copy(s->completed.begin(), s->completed.begin() + n, out);
    s->completed.erase(s->completed.begin(), s->completed.begin() + n);
    *count = n;
    return VSIM_OK;
}

int vsim_server_get_stats(const vsim_server* s, vsim_server_stats* out) {
    if (!s || !out) return fail(VSIM_ERR_INVALID, "NULL argument");
    out->sessions = uint32_t(s->resident.size());
    out->rejected = s->rejected;
    out->resident_bytes = s->residentBytes;
    out->ticks = s->ticks;
    out->session_frames = s->sessionFrames;
    out->cell_updates = s->cellUpdates;
    out->pending = s->pending;
    out->tick_seconds = s->tickSeconds;
    out->prepare_seconds = s->prepareSeconds;
    out->frame_seconds = s->frameSeconds;
    return VSIM_OK;
}

uint32_t vsim_server_node_count(const vsim_server* s, uint32_t session) {
    return s && session < s->sessions.size() ? s->sessions[session].nodes : 0;
}

int vsim_server_read_state(vsim_server* s, uint32_t session, float* pos, float* prev, float* vel,
                           size_t node_count) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    vsim_sim* sim = s->sim;
    DeviceGuard guard(sim->device);
    uint32_t body;
    if (int rc = residentBody(s, session, body)) return rc;
    if (node_count != sim->lat[body].nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match");
    float* const out[3] = {pos, prev, vel};
    return readNodes(sim, sim->offsets[body], node_count, out);
}

int vsim_server_write_state(vsim_server* s, uint32_t session, const float* pos, const float* prev, const float* vel,
                            size_t node_count) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    vsim_sim* sim = s->sim;
    DeviceGuard guard(sim->device);
    int rc = idleSession(s, session);
    if (rc) return rc;
    const uint32_t body = uint32_t(s->slot[session]);
    if (node_count != sim->lat[body].nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match");
    const size_t first = sim->offsets[body];
    if (pos) {
        if (!sim->staging) CK(allocN(&sim->staging, sim->nodeCount), "allocate staging");
        CK(cudaMemcpyAsync(sim->staging, pos, node_count * 16, cudaMemcpyHostToDevice, sim->stream), "write session");
        CK(launchMergeXyz(sim->stream, sim->staging, uint32_t(node_count), sim->d.pos + first), "write session");
    }
    if (prev)
        CK(cudaMemcpyAsync(sim->d.prev + first, prev, node_count * 16, cudaMemcpyHostToDevice, sim->stream),
           "write session");
    if (vel)
        CK(cudaMemcpyAsync(sim->d.vel + first, vel, node_count * 16, cudaMemcpyHostToDevice, sim->stream),
           "write session");
    CK(cudaStreamSynchronize(sim->stream), "write session");
    return VSIM_OK;
}

int vsim_server_reset_session(vsim_server* s, uint32_t session) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    vsim_sim* sim = s->sim;
    DeviceGuard guard(sim->device);
    int rc = idleSession(s, session);
    if (rc) return rc;
    const uint32_t body = uint32_t(s->slot[session]);
    const size_t first = sim->offsets[body], n = sim->lat[body].nodeCount;
    const float* rest = sim->restPos.data() + 4 * first;
    CK(cudaMemcpyAsync(sim->d.pos + first, rest, n * 16, cudaMemcpyHostToDevice, sim->stream), "reset session");
    CK(cudaMemcpyAsync(sim->d.prev + first, rest, n * 16, cudaMemcpyHostToDevice, sim->stream), "reset session");
    CK(cudaMemsetAsync(sim->d.vel + first, 0, n * 16, sim->stream), "reset session");
    CK(cudaStreamSynchronize(sim->stream), "reset session");
    return VSIM_OK;
}

int vsim_server_read_positions(vsim_server* s, uint32_t session, float* xyzw, size_t node_count) {
    clearError();
    if (!s || !xyzw) return fail(VSIM_ERR_INVALID, "NULL argument");
    vsim_sim* sim = s->sim;
    DeviceGuard guard(sim->device);
    uint32_t body;
    if (int rc = residentBody(s, session, body)) return rc;
    if (node_count != sim->lat[body].nodeCount) return fail(VSIM_ERR_CAPACITY, "node_count does not match");
    float* const out[3] = {xyzw, nullptr, nullptr};
    return readNodes(sim, sim->offsets[body], node_count, out);
}

}  // extern "C"
