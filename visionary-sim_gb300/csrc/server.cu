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
//
// The request loop (vsim_server_run) has a second engine, the default: for
// sessions small enough, session kernels (session.cu). There a request is
// a job -- its session's frames, all of them, run by one block or one
// cluster -- and the loop launches every ready request as soon as one of a
// few launch slots is free, without waiting for requests already running;
// each job reports its end through a ticket in host-mapped memory, so a
// short request is retired when it ends, not when its launch does. The
// larger sessions run as ticks of shared frames at the same time. The
// explicit tick (vsim_server_tick) stays the frame-at-a-time engine above;
// every engine gives every session the same result.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <string>
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

// One launch of session kernels in flight: its stream, its end, and the
// tables its kernel reads -- groups, jobs, drive rows -- staged in pinned
// memory and copied to the device in stream order before the launch (both
// rewritten only once it has ended).
struct LaunchSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, end = nullptr;
    bool busy = false;
    double launched = 0;
    std::vector<uint32_t> sessions;  // the sessions it runs
    unsigned char* staging = nullptr;
    unsigned char* tables = nullptr;
    size_t tableCap = 0;
};

constexpr int kLaunchSlots = 8;

// The session-kernel engine of one device pool.
struct SessionEngine {
    LaunchSlot slot[kLaunchSlots];
    uint32_t* done = nullptr;      // per body: ticket of the last job run (host-mapped)
    uint32_t* doneDev = nullptr;
    uint32_t* status = nullptr;    // per body: fault of the last job run (host-mapped)
    uint32_t* statusDev = nullptr;
    uint32_t* cursor = nullptr;    // per body, device
    uint32_t* fault = nullptr;     // per body, device
    // The jobs' own bucket-order arrays, one slot per surface record: a job
    // lays out its runs inside its session's record range, which a tick
    // running alongside (its runs packed from position 0) must not touch.
    uint32_t* entries = nullptr;
    SortedEntries sorted{};
    uint32_t ticket = 0;
};

}  // namespace

struct vsim_server {
    vsim_sim* sim = nullptr;
    vsim_tank world{};
    vsim_server_config config{};
    void* stream = nullptr;
    bool ownStream = false;  // made by the server (none given): destroyed with it
    int streamDevice = 0;
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
    int engine = VSIM_SERVE_SESSIONS;  // how vsim_server_run runs requests
    // Session engine: a session whose largest colour has at most blockCells
    // cells runs in one block, else at most clusterCells in one cluster,
    // else in ticks of shared frames.
    uint32_t blockCells = kDefaultBlockCells, clusterCells = kDefaultClusterCells;
    SessionEngine* sessionEngine = nullptr;  // built on first use for the current pool
    std::vector<uint8_t> kernelHolds;  // per session, during a run: its drag holds are the session kernel's
    // The tick in flight (startTick .. finishTick).
    bool tickInFlight = false;
    double tickEntered = 0;
};

namespace {

// Holds exactly the nodes the resident sessions' drags name.
int applyHolds(vsim_server* s) {
    std::vector<uint32_t> nodes;
    for (uint32_t b = 0; b < s->resident.size(); b++) {
        if (!s->kernelHolds.empty() && s->kernelHolds[s->resident[b]]) continue;
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

void freePinned(void*& p) {
    if (p) cudaFreeHost(p);
    p = nullptr;
}

// Waits for every launch in flight and frees the engine.
void dropEngine(vsim_server* s) {
    SessionEngine* e = s->sessionEngine;
    if (!e) return;
    for (LaunchSlot& l : e->slot) {
        if (l.stream) {
            cudaStreamSynchronize(l.stream);
            cudaStreamDestroy(l.stream);
        }
        if (l.start) cudaEventDestroy(l.start);
        if (l.end) cudaEventDestroy(l.end);
        freePinned(reinterpret_cast<void*&>(l.staging));
        if (l.tables) cudaFree(l.tables);
    }
    freePinned(reinterpret_cast<void*&>(e->done));
    freePinned(reinterpret_cast<void*&>(e->status));
    if (e->cursor) cudaFree(e->cursor);
    if (e->fault) cudaFree(e->fault);
    void* owned[] = {e->entries, e->sorted.sMeta, e->sorted.sPos, e->sorted.sMoved, e->sorted.sRec, e->sorted.sKey};
    for (void* p : owned)
        if (p) cudaFree(p);
    delete e;
    s->sessionEngine = nullptr;
}

int destroyServer(vsim_server* s) {
    if (s->sim) {
        DeviceGuard guard(s->sim->device);
        dropEngine(s);
    }
    if (s->sim) {
        DeviceGuard guard(s->sim->device);
        cudaStreamSynchronize(s->sim->stream);
        if (s->frameStart) cudaEventDestroy(s->frameStart);
        if (s->frameDone) cudaEventDestroy(s->frameDone);
    }
    dropSim(s->sim);
    if (s->ownStream) {
        DeviceGuard guard(s->streamDevice);
        cudaStreamDestroy(static_cast<cudaStream_t>(s->stream));
    }
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
    if (!stream) {
        // The ticks' stream at the device's greatest priority. The session
        // engine's launch slots are made at its least, which is also the
        // priority of a stream made without one: blocks of a tick waiting
        // to start then go before those of a session launch.
        int least = 0, greatest = 0;
        cudaStream_t own = nullptr;
        if (cudaGetDevice(&s->streamDevice) != cudaSuccess ||
            cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
            cudaStreamCreateWithPriority(&own, cudaStreamNonBlocking, greatest) != cudaSuccess) {
            delete s;
            return fail(VSIM_ERR_CUDA, "create the server's stream");
        }
        s->stream = own;
        s->ownStream = true;
    }
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
    dropEngine(s);  // its tables are sized for the old pool
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

}  // extern "C"

namespace {

// The first half of a tick: picks the sessions the frame runs (those with a
// pending request, `eligible` ones only when given), sets their holds and
// drag targets and launches the frame on the pool's stream without waiting.
// *stepped: how many sessions it runs (0: nothing launched).
int startTick(vsim_server* s, const std::vector<uint8_t>* eligible, uint32_t* stepped) {
    *stepped = 0;
    vsim_sim* sim = s->sim;
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
            if (q.empty() || (eligible && !(*eligible)[s->resident[b]])) continue;
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
    s->tickInFlight = true;
    s->tickEntered = entered;
    *stepped = active;
    return VSIM_OK;
}

// The second half: waits for the frame and retires what it finished.
int finishTick(vsim_server* s) {
    vsim_sim* sim = s->sim;
    s->tickInFlight = false;
    CK(cudaEventSynchronize(s->frameDone), "serve frame");
    float frameMs = 0;
    if (cudaEventElapsedTime(&frameMs, s->frameStart, s->frameDone) == cudaSuccess) s->frameSeconds += 1e-3 * frameMs;
    const double now = seconds(s);
    for (uint32_t b = 0; b < s->resident.size(); b++) {
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
    s->tickSeconds += seconds(s) - s->tickEntered;
    return VSIM_OK;
}

}  // namespace

extern "C" {

int vsim_server_tick(vsim_server* s, uint32_t* stepped) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    if (stepped) *stepped = 0;
    DeviceGuard guard(s->sim->device);
    uint32_t active = 0;
    if (int rc = startTick(s, nullptr, &active)) return rc;
    if (active == 0) return VSIM_OK;
    if (int rc = finishTick(s)) return rc;
    if (stepped) *stepped = active;
    return VSIM_OK;
}

}  // extern "C"

namespace {

// What both engines' request loops share: the schedule, the closed loop's
// refills and measured window, the completions handed back.
struct RunState {
    const vsim_scheduled_request* requests;
    uint32_t n;
    const vsim_drag* drags;
    bool closed;
    double closedSeconds;
    vsim_completion* out;
    uint32_t capacity;
    std::vector<vsim_completion> done;
    uint64_t frames0 = 0, ticks0 = 0, requestsDone = 0;
    uint32_t next = 0;
    double t0 = 0;
    bool windowClosed = false;
    uint64_t windowRequests = 0, windowFrames = 0, windowTicks = 0;
    double windowSeconds = 0;

    int submit(vsim_server* s, uint32_t session, const vsim_scheduled_request& q, double at) {
        return submitAt(s, session, q.frames, q.drag ? &drags[session] : nullptr, at, nullptr);
    }
    // Open loop: queue every request whose arrival time has come.
    int admitDue(vsim_server* s) {
        if (closed) return VSIM_OK;
        const double now = seconds(s);
        while (next < n && t0 + requests[next].arrival <= now) {
            if (int rc = submit(s, requests[next].session, requests[next], t0 + requests[next].arrival)) return rc;
            next++;
        }
        return VSIM_OK;
    }
    // Takes the server's new completions; in a closed loop each is replaced
    // by the list's next request, to the session that request names, until
    // the span ends.
    int collect(vsim_server* s) {
        if (s->completed.empty()) return VSIM_OK;
        const bool refill = closed && seconds(s) - t0 < closedSeconds;
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
                if (int rc = submit(s, requests[next].session, requests[next], seconds(s))) return rc;
                next = (next + 1) % n;
            }
        }
        s->completed.clear();
        return VSIM_OK;
    }
    // Sleeps until shortly before the next arrival.
    void idle(const vsim_server* s) const {
        const double wait = t0 + requests[next].arrival - seconds(s);
        if (wait > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(wait - 1e-4));
    }
};

int runFrames(vsim_server* s, RunState& st) {
    while (true) {
        if (int rc = st.admitDue(s)) return rc;
        if (s->pending) {
            if (int rc = vsim_server_tick(s, nullptr)) return rc;
            if (int rc = st.collect(s)) return rc;
            continue;
        }
        if (st.closed || st.next >= st.n) return VSIM_OK;
        st.idle(s);
    }
}

// Room for `need` bytes of tables in the slot's staging and device buffers.
int growTables(LaunchSlot& l, size_t need) {
    if (need <= l.tableCap) return VSIM_OK;
    const size_t want = std::max<size_t>(need, 2 * l.tableCap);
    if (l.staging) cudaFreeHost(l.staging);
    if (l.tables) cudaFree(l.tables);
    l.staging = l.tables = nullptr;
    l.tableCap = 0;
    CK(cudaMallocHost(reinterpret_cast<void**>(&l.staging), want), "allocate job tables");
    CK(cudaMalloc(reinterpret_cast<void**>(&l.tables), want), "allocate job tables");
    l.tableCap = want;
    return VSIM_OK;
}

inline size_t align16(size_t n) { return (n + 15) & ~size_t(15); }

template <class T>
T* devicePointer(T* host) {
    void* d = nullptr;
    return cudaHostGetDevicePointer(&d, host, 0) == cudaSuccess ? static_cast<T*>(d) : nullptr;
}

int buildEngine(vsim_server* s) {
    if (s->sessionEngine) return VSIM_OK;
    auto* e = new (std::nothrow) SessionEngine();
    if (!e) return fail(VSIM_ERR_NOMEM, "out of host memory");
    s->sessionEngine = e;
    const size_t bodies = std::max<size_t>(1, s->resident.size());
    CK(cudaHostAlloc(reinterpret_cast<void**>(&e->done), bodies * 4, cudaHostAllocMapped), "allocate tickets");
    std::memset(e->done, 0, bodies * 4);
    CK(cudaHostAlloc(reinterpret_cast<void**>(&e->status), bodies * 4, cudaHostAllocMapped), "allocate tickets");
    std::memset(e->status, 0, bodies * 4);
    e->doneDev = devicePointer(e->done);
    e->statusDev = devicePointer(e->status);
    if (!e->doneDev || !e->statusDev) return fail(VSIM_ERR_CUDA, "map tickets");
    CK(cudaMalloc(reinterpret_cast<void**>(&e->cursor), bodies * 4), "allocate segment cursors");
    CK(cudaMalloc(reinterpret_cast<void**>(&e->fault), bodies * 4), "allocate job checks");
    const size_t records = s->sim->surfaceCount;
    CK(allocN(&e->entries, records), "allocate the jobs' bucket order");
    CK(allocN(&e->sorted.sMeta, records), "allocate the jobs' bucket order");
    CK(allocN(&e->sorted.sPos, records), "allocate the jobs' bucket order");
    CK(allocN(&e->sorted.sMoved, records), "allocate the jobs' bucket order");
    CK(allocN(&e->sorted.sRec, records), "allocate the jobs' bucket order");
    CK(allocN(&e->sorted.sKey, records), "allocate the jobs' bucket order");
    // Session launches yield to the ticks' frames: each of those is a chain
    // of short dependent launches whose blocks should get SMs first.
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "query stream priorities");
    // Every slot sized up front for a launch of every resident session (and
    // four drag frames each): growing one later frees device memory, which
    // waits for every kernel in flight.
    const size_t jobs = std::max<size_t>(1, s->resident.size());
    const size_t tableBytes = align16(jobs * sizeof(SessionGroup)) + align16(jobs * sizeof(SessionJob)) +
                              2 * 4 * jobs * sizeof(float4);
    for (LaunchSlot& l : e->slot) {
        CK(cudaStreamCreateWithPriority(&l.stream, cudaStreamNonBlocking, least), "create launch stream");
        CK(cudaEventCreate(&l.start), "create launch event");
        CK(cudaEventCreate(&l.end), "create launch event");
        if (int rc = growTables(l, tableBytes)) return rc;
    }
    return VSIM_OK;
}

// Marks session i's running request done, at `now`.
void retire(vsim_server* s, uint32_t i, double now) {
    Request& r = s->queue[i].front();
    r.done = r.frames;
    s->sessionFrames += r.frames;
    s->cellUpdates += uint64_t(s->sessions[i].cells) * s->config.substeps * r.frames;
    s->completed.push_back(vsim_completion{r.id, r.session, r.frames, r.submitted, now, r.firstTick, r.firstTick});
    s->queue[i].pop_front();
    s->pending--;
}

// One launch over every session that has a request and none running, if a
// launch slot is free. A request's drag targets for all its frames are
// computed here, as the frame-at-a-time engine computes them frame by frame.
int launchReady(vsim_server* s, const std::vector<uint8_t>& inKernel, std::vector<int8_t>& running,
                std::vector<uint32_t>& ticketOf, bool& launched) {
    launched = false;
    SessionEngine* e = s->sessionEngine;
    LaunchSlot* l = nullptr;
    for (LaunchSlot& c : e->slot)
        if (!c.busy) {
            l = &c;
            break;
        }
    if (!l) return VSIM_OK;
    const double entered = seconds(s);
    vsim_sim* sim = s->sim;
    std::vector<uint32_t> ready;
    size_t driveRows = 0;
    for (uint32_t i : s->resident)
        if (inKernel[i] && running[i] < 0 && !s->queue[i].empty()) {
            ready.push_back(i);
            if (s->queue[i].front().drag) driveRows += s->queue[i].front().frames;
        }
    if (ready.empty()) return VSIM_OK;
    const size_t groupBytes = align16(ready.size() * sizeof(SessionGroup));
    const size_t jobBytes = align16(ready.size() * sizeof(SessionJob));
    if (int rc = growTables(*l, groupBytes + jobBytes + 2 * std::max<size_t>(driveRows, 1) * sizeof(float4)))
        return rc;
    auto* groupTable = reinterpret_cast<SessionGroup*>(l->staging);
    auto* jobTable = reinterpret_cast<SessionJob*>(l->staging + groupBytes);
    auto* driveTable = reinterpret_cast<float4*>(l->staging + groupBytes + jobBytes);
    const double frameDt = s->config.substeps * s->config.step_duration;
    std::vector<uint32_t> wide, narrow;
    uint32_t rows = 0;
    for (uint32_t k = 0; k < ready.size(); k++) {
        const uint32_t i = ready[k];
        const uint32_t b = uint32_t(s->slot[i]);
        Request& r = s->queue[i].front();
        SessionJob& j = jobTable[k];
        j = SessionJob{};
        j.nodeFirst = sim->nodeBodyStart[b];
        j.nodeCount = sim->nodeBodyStart[b + 1] - sim->nodeBodyStart[b];
        j.recFirst = sim->recordBodyStart[b];
        j.recCount = sim->recordBodyStart[b + 1] - sim->recordBodyStart[b];
        uint32_t widest = 0;
        for (int c = 0; c < 8; c++) {
            j.cellFirst[c] = sim->colorStart[c] + sim->colourBodyStart[c][b];
            j.cellCount[c] = sim->colourBodyStart[c][b + 1] - sim->colourBodyStart[c][b];
            widest = std::max(widest, j.cellCount[c]);
        }
        j.body = b;
        j.frames = r.frames;
        j.heldBefore = s->held[i] >= 0 ? int32_t(sim->offsets[b] + uint32_t(s->held[i])) : -1;
        s->held[i] = r.drag ? int64_t(r.path.node) : int64_t(-1);
        j.held = s->held[i] >= 0 ? int32_t(sim->offsets[b] + uint32_t(s->held[i])) : -1;
        j.driveFirst = rows;
        if (r.drag) {
            // The drag starts on its curve (the grab's placement) and
            // advances one frame at a time at its speed; velocity is each
            // frame's motion over its duration (simulator.js:309-315).
            double prev[3], p[3], dp[3];
            bezier(r.path.control, 0.0, prev, dp);
            for (uint32_t f = 0; f < r.frames; f++) {
                bezier(r.path.control, r.t, p, dp);
                const double rate = std::sqrt(dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
                r.t = std::min(1.0, r.t + r.path.speed * frameDt / std::max(rate, 1e-9));
                bezier(r.path.control, r.t, p, dp);
                driveTable[2 * (rows + f)] = make_float4(float(p[0]), float(p[1]), float(p[2]), 0.0f);
                driveTable[2 * (rows + f) + 1] =
                    make_float4(float((p[0] - prev[0]) / frameDt), float((p[1] - prev[1]) / frameDt),
                                float((p[2] - prev[2]) / frameDt), 0.0f);
                for (int a = 0; a < 3; a++) prev[a] = p[a];
            }
            for (int a = 0; a < 3; a++) s->prevTarget[3 * i + a] = prev[a];
            rows += r.frames;
        }
        j.ticket = ++e->ticket;
        ticketOf[i] = j.ticket;
        (widest > s->blockCells ? wide : narrow).push_back(k);
    }
    // Wide jobs first (each a cluster), then the narrow ones, a block each.
    uint32_t groups = 0;
    for (uint32_t k : wide) {
        SessionGroup& g = groupTable[groups++];
        g.wide = 1;
        g.job[0] = k;
        for (uint32_t r = 1; r < kSessionCluster; r++) g.job[r] = kNoJob;
    }
    for (size_t at = 0; at < narrow.size(); at += kSessionCluster) {
        SessionGroup& g = groupTable[groups++];
        g.wide = 0;
        for (uint32_t r = 0; r < kSessionCluster; r++) g.job[r] = at + r < narrow.size() ? narrow[at + r] : kNoJob;
    }
    SessionLaunch L{};
    L.groups = reinterpret_cast<const SessionGroup*>(l->tables);
    L.groupCount = groups;
    L.jobs = reinterpret_cast<const SessionJob*>(l->tables + groupBytes);
    L.drive = reinterpret_cast<const float4*>(l->tables + groupBytes + jobBytes);
    L.cursor = e->cursor;
    L.fault = e->fault;
    L.done = e->doneDev;
    L.status = e->statusDev;
    L.activeCount = sim->activeCount;
    L.cellCount = sim->cellCount;
    L.surfaceCount = sim->surfaceCount;
    L.nodeCount = sim->nodeCount;
    L.bodyCount = uint32_t(s->resident.size());
    L.driveRows = rows;
    L.substeps = s->config.substeps;
    L.iterations = sim->iterations;
    L.limited = anyStretch(sim) ? 1u : 0u;
    L.contact = sim->contact && sim->surfaceCount > 0 ? 1u : 0u;
    L.warpRecords = 4;
    L.lens = stretchLengths();
    CK(cudaMemcpyAsync(l->tables, l->staging, groupBytes + jobBytes + 2 * size_t(rows) * sizeof(float4),
                       cudaMemcpyHostToDevice, l->stream),
       "upload job tables");
    CK(cudaEventRecord(l->start, l->stream), "launch sessions");
    CK(launchSessions(l->stream, sim->d, e->entries, e->sorted, L), "launch sessions");
    CK(cudaEventRecord(l->end, l->stream), "launch sessions");
    l->busy = true;
    l->launched = seconds(s);
    l->sessions = ready;
    for (uint32_t i : ready) {
        running[i] = int8_t(l - e->slot);  // the slot it runs in
        s->queue[i].front().firstTick = s->ticks;
    }
    s->ticks++;
    s->prepareSeconds += l->launched - entered;
    launched = true;
    return VSIM_OK;
}

int runSessions(vsim_server* s, RunState& st) {
    if (int rc = buildEngine(s)) return rc;
    vsim_sim* sim = s->sim;
    if (int rc = syncParams(sim)) return rc;
    CK(cudaStreamSynchronize(sim->stream), "serve sessions");
    SessionEngine* e = s->sessionEngine;
    // Sessions small enough for a block (or, if allowed, a cluster) run in
    // the session kernel; the rest in ticks of shared frames on the pool's
    // stream, alongside. The kernel sessions' drag holds are the kernel's
    // own while the run lasts, so the pool's hold list -- which the ticks
    // rewrite -- leaves their nodes alone.
    std::vector<uint8_t> inKernel(s->sessions.size(), 0), inTicks(s->sessions.size(), 0);
    for (uint32_t b = 0; b < s->resident.size(); b++) {
        uint32_t widest = 0;
        for (int c = 0; c < 8; c++) widest = std::max(widest, sim->colourBodyStart[c][b + 1] - sim->colourBodyStart[c][b]);
        const uint32_t i = s->resident[b];
        inKernel[i] = widest <= std::max(s->blockCells, s->clusterCells);
        inTicks[i] = !inKernel[i];
    }
    s->kernelHolds = inKernel;
    if (int rc = applyHolds(s)) return rc;
    // Per session: the launch slot its request runs in, -1 for none. A
    // session retired by its ticket may run again in another slot while the
    // first slot still runs others, so a slot answers only for its own.
    std::vector<int8_t> running(s->sessions.size(), -1);
    std::vector<uint32_t> ticketOf(s->sessions.size(), 0);
    bool faulted = false;
    int fault = VSIM_OK;
    // An error leaves nothing in flight behind it.
    auto bail = [&](int rc) {
        for (LaunchSlot& l : e->slot) cudaStreamSynchronize(l.stream);
        if (s->tickInFlight) finishTick(s);
        s->kernelHolds.clear();
        for (int k = 0; k < kLaunchSlots; k++) {
            LaunchSlot& l = e->slot[k];
            for (uint32_t i : l.sessions)
                if (running[i] == k) {
                    retire(s, i, seconds(s));
                    running[i] = -1;
                }
            l.sessions.clear();
            l.busy = false;
        }
        s->completed.clear();
        return rc;
    };
    while (true) {
        if (int rc = st.admitDue(s)) return bail(rc);
        // Retire the jobs that have ended: by their tickets, or all of a
        // launch once it has ended.
        bool anyRunning = false, progressed = false;
        for (int k = 0; k < kLaunchSlots; k++) {
            LaunchSlot& l = e->slot[k];
            if (!l.busy) continue;
            const cudaError_t q = cudaEventQuery(l.end);
            if (q != cudaSuccess && q != cudaErrorNotReady) return bail(cudaFail(q, "serve sessions"));
            const bool ended = q == cudaSuccess;
            const double now = seconds(s);
            for (uint32_t i : l.sessions) {
                if (running[i] != k) continue;
                const uint32_t b = uint32_t(s->slot[i]);
                const bool seen = __atomic_load_n(&e->done[b], __ATOMIC_ACQUIRE) == ticketOf[i];
                if (!seen && !ended) continue;
                const uint32_t check = seen ? e->status[b] : 0xffffffffu;
                retire(s, i, now);
                running[i] = -1;
                progressed = true;
                if (check != kFaultNone && !faulted) {
                    faulted = true;
                    fault = fail(VSIM_ERR_CUDA, "session kernel: session " + std::to_string(i) +
                                                    (seen ? " failed check " + std::to_string(check)
                                                          : " ended without its ticket"));
                }
            }
            if (ended) {
                float ms = 0;
                if (cudaEventElapsedTime(&ms, l.start, l.end) == cudaSuccess) s->frameSeconds += 1e-3 * ms;
                s->tickSeconds += now - l.launched;
                l.sessions.clear();
                l.busy = false;
            } else {
                anyRunning = true;
            }
        }
        if (faulted) return bail(fault);
        if (s->tickInFlight) {
            const cudaError_t q = cudaEventQuery(s->frameDone);
            if (q != cudaSuccess && q != cudaErrorNotReady) return bail(cudaFail(q, "serve frame"));
            if (q == cudaSuccess) {
                if (int rc = finishTick(s)) return bail(rc);
                progressed = true;
            }
        }
        if (int rc = st.collect(s)) return bail(rc);
        bool launched;
        if (int rc = launchReady(s, inKernel, running, ticketOf, launched)) return bail(rc);
        if (!s->tickInFlight) {
            uint32_t stepped = 0;
            if (int rc = startTick(s, &inTicks, &stepped)) return bail(rc);
            launched = launched || stepped > 0;
        }
        anyRunning = anyRunning || launched || s->tickInFlight;
        if (anyRunning) {
            if (!progressed && !launched) std::this_thread::yield();
            continue;
        }
        if (st.closed || st.next >= st.n) break;
        st.idle(s);
    }
    // The device pool's hold list follows what the jobs left held.
    s->kernelHolds.clear();
    return applyHolds(s);
}

}  // namespace

extern "C" {

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
    DeviceGuard guard(s->sim->device);
    RunState st{requests, n, drags, closed, closed_loop_seconds, out, capacity};
    st.frames0 = s->sessionFrames;
    st.ticks0 = s->ticks;
    st.t0 = seconds(s);
    if (closed) {
        for (size_t k = 0; k < s->resident.size(); k++) {
            if (int rc = st.submit(s, requests[st.next].session, requests[st.next], seconds(s))) return rc;
            st.next = (st.next + 1) % n;
        }
    }
    const int rc = s->engine == VSIM_SERVE_SESSIONS ? runSessions(s, st) : runFrames(s, st);
    if (rc) return rc;
    if (out) std::copy(st.done.begin(), st.done.end(), out);
    if (report) {
        report->requests = closed ? st.windowRequests : st.requestsDone;
        report->returned = uint32_t(st.done.size());
        report->frames = closed ? st.windowFrames : s->sessionFrames - st.frames0;
        report->ticks = closed ? st.windowTicks : s->ticks - st.ticks0;
        report->seconds = closed ? st.windowSeconds : seconds(s) - st.t0;
    }
    return VSIM_OK;
}

int vsim_server_set_engine(vsim_server* s, int engine, uint32_t block_cells, uint32_t cluster_cells) {
    clearError();
    if (!s) return fail(VSIM_ERR_INVALID, "server is NULL");
    if (engine != VSIM_SERVE_FRAMES && engine != VSIM_SERVE_SESSIONS) return fail(VSIM_ERR_RANGE, "unknown engine");
    s->engine = engine;
    s->blockCells = block_cells;
    s->clusterCells = cluster_cells;
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
