// Host-side logic of libvsim that needs no GPU: error state, material
// arithmetic, lattice construction, the contact grid layout and the fixed
// timestep clock, plus their C entry points.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "vsim_internal.h"

namespace vsim {

namespace {
thread_local std::string g_lastError;
}

int fail(int code, const std::string& msg) {
    g_lastError = msg;
    return code;
}

void clearError() { g_lastError.clear(); }

// material.js:66,101-108: nu clamped to [0.25, 0.49], E at least 1.
void lame(const vsim_material& m, double& mu, double& lambda) {
    const double nu = std::min(std::max(m.poisson_ratio, 0.25), 0.49);
    const double e = std::max(m.youngs_modulus, 1.0);
    mu = e / (2 * (1 + nu));
    lambda = (e * nu) / ((1 + nu) * (1 - 2 * nu));
}

// material.js:137-140.
double waveSpeed(const vsim_material& m) {
    double mu, lambda;
    lame(m, mu, lambda);
    return std::sqrt((lambda + 2 * mu) / m.density);
}

// material.js:80-85.
bool validMaxStretch(double v) { return std::isfinite(v) && (v == 0 || v > 1); }

// material.js:69-77.
vsim_material defaultMaterial() { return vsim_material{1.2e5, 0.40, 1000, 0.4, 0.6, 0.012, 0}; }

// lattice.js:166-239 and lattice.js:128-158, for one body.
int buildLattice(const vsim_body_desc& d, Lattice& L) {
    for (int a = 0; a < 3; a++) {
        if (d.cell_dims[a] == 0 || d.cell_dims[a] > 4096)
            return fail(VSIM_ERR_RANGE, "body cell_dims must be in [1, 4096] per axis");
        L.cellDims[a] = d.cell_dims[a];
        L.nodeDims[a] = d.cell_dims[a] + 1;
        L.origin[a] = d.origin[a];
    }
    if (!(d.h > 0) || !std::isfinite(d.h)) return fail(VSIM_ERR_RANGE, "body h must be finite and positive");
    if (!d.occupancy) return fail(VSIM_ERR_INVALID, "body occupancy is NULL");
    if (!(d.material.density > 0)) return fail(VSIM_ERR_RANGE, "material density must be positive");
    if (!validMaxStretch(d.material.max_stretch))
        return fail(VSIM_ERR_RANGE, "maxStretch must be zero (disabled) or a finite ratio greater than one");
    const uint64_t nodes = uint64_t(L.nodeDims[0]) * L.nodeDims[1] * L.nodeDims[2];
    if (nodes >= (1ull << 31)) return fail(VSIM_ERR_RANGE, "body has too many nodes");
    L.h = d.h;
    L.nodeCount = uint32_t(nodes);
    const uint32_t* cd = L.cellDims;
    const uint32_t* nd = L.nodeDims;
    const size_t cells = size_t(cd[0]) * cd[1] * cd[2];
    L.occupancy.assign(d.occupancy, d.occupancy + cells);

    // Rest positions: f32 of the double sum origin + i h (lattice.js:171-181).
    L.rest.resize(size_t(L.nodeCount) * 3);
    for (uint32_t k = 0; k < nd[2]; k++)
        for (uint32_t j = 0; j < nd[1]; j++)
            for (uint32_t i = 0; i < nd[0]; i++) {
                const size_t n = i + size_t(nd[0]) * (j + size_t(nd[1]) * k);
                L.rest[3 * n] = float(L.origin[0] + i * L.h);
                L.rest[3 * n + 1] = float(L.origin[1] + j * L.h);
                L.rest[3 * n + 2] = float(L.origin[2] + k * L.h);
            }

    // Lumped mass: each occupied cell puts rho h^3 / 8 on each corner, the sum
    // held in f32 as the reference's Float32Array holds it (lattice.js:185-224).
    const double cornerMass = d.material.density * L.h * L.h * L.h / 8;
    std::vector<float> mass(L.nodeCount, 0.0f);
    L.cellCount = 0;
    for (uint32_t k = 0; k < cd[2]; k++)
        for (uint32_t j = 0; j < cd[1]; j++)
            for (uint32_t i = 0; i < cd[0]; i++) {
                const uint32_t cell = i + cd[0] * (j + cd[1] * k);
                if (!L.occupancy[cell]) continue;
                L.cellCount++;
                L.cellsByColor[cellColor(i, j, k)].push_back(cell);
                for (int c = 0; c < 8; c++) {
                    const uint32_t n = (i + (c & 1)) + nd[0] * ((j + ((c >> 1) & 1)) + nd[1] * (k + ((c >> 2) & 1)));
                    mass[n] = float(double(mass[n]) + cornerMass);
                }
            }
    L.invMass.resize(L.nodeCount);
    for (uint32_t n = 0; n < L.nodeCount; n++) L.invMass[n] = mass[n] > 0 ? float(1.0 / double(mass[n])) : 0.0f;

    // Boundary nodes: some but not all of the eight incident cells occupied.
    L.surface.clear();
    for (uint32_t k = 0; k < nd[2]; k++)
        for (uint32_t j = 0; j < nd[1]; j++)
            for (uint32_t i = 0; i < nd[0]; i++) {
                int filled = 0;
                for (int c = 0; c < 8; c++) {
                    const int64_t ci = int64_t(i) + (c & 1) - 1;
                    const int64_t cj = int64_t(j) + ((c >> 1) & 1) - 1;
                    const int64_t ck = int64_t(k) + ((c >> 2) & 1) - 1;
                    if (ci < 0 || cj < 0 || ck < 0 || ci >= cd[0] || cj >= cd[1] || ck >= cd[2]) continue;
                    filled += L.occupancy[ci + cd[0] * (cj + cd[1] * ck)] ? 1 : 0;
                }
                if (filled > 0 && filled < 8) L.surface.push_back(i + nd[0] * (j + nd[1] * k));
            }
    return VSIM_OK;
}

namespace {
void layout(const double mn[3], const double mx[3], double bucket, Grid& g) {
    const double edge = bucket > 0 ? bucket : std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]});
    g.bucket = edge;
    for (int a = 0; a < 3; a++) {
        const double span = std::ceil((mx[a] - mn[a]) / edge);
        g.dims[a] = uint32_t(std::min(std::max(1.0, span), 1e9) + 2);
        g.origin[a] = mn[a] - edge;
    }
}
}  // namespace

Grid contactGrid(const vsim_tank& tank, double widest, const double lo[3], const double hi[3]) {
    Grid g;
    layout(tank.min, tank.max, widest * 2, g);
    bool finite = true;
    for (int a = 0; a < 3; a++) finite = finite && std::isfinite(tank.min[a]) && std::isfinite(tank.max[a]);
    if (!finite || !(double(g.count()) <= kGridLimit)) {
        double mn[3], mx[3];
        for (int a = 0; a < 3; a++) {
            const double pad = std::max(0.5 * (hi[a] - lo[a]), 4 * widest * 2);
            mn[a] = std::max(tank.min[a], lo[a] - pad);
            mx[a] = std::min(tank.max[a], hi[a] + pad);
        }
        layout(mn, mx, widest * 2, g);
    }
    return g;
}

// timestep.js:38-45 (the rate is validated by the caller).
double stableStepDuration(double waveRate) {
    return waveRate == 0 ? kMaxStepDuration : std::min(kMaxStepDuration, kTargetCfl / waveRate);
}

// timestep.js:99-130.
void Clock::consume(double elapsed, bool forceStep) {
    accumulator += elapsed;
    const double epsilon = stepDuration * 1e-9;
    const double available = std::floor((accumulator + epsilon) / stepDuration);
    uint32_t steps = uint32_t(std::min(available, double(maxStepsPerFrame)));
    const double droppedSteps = available - steps;
    const double consumedSteps = steps + droppedSteps;
    accumulator -= consumedSteps * stepDuration;
    if (accumulator < 0 && accumulator > -epsilon) accumulator = 0;
    if (forceStep && steps == 0) steps = 1;
    lastSteps = steps;
    lastElapsed = elapsed;
    lastDroppedTime = droppedSteps * stepDuration;
    simulatedTime += steps * stepDuration;
    totalSteps += steps;
    droppedTime += lastDroppedTime;
}

// timestep.js:407-412.
void Clock::idle() {
    lastSteps = 0;
    lastElapsed = 0;
    lastDroppedTime = 0;
}

// timestep.js:415-422.
void Clock::singleStep() {
    lastSteps = 1;
    lastElapsed = 0;
    lastDroppedTime = 0;
    simulatedTime += stepDuration;
    totalSteps++;
}

// timestep.js:425-433.
void Clock::reset() {
    accumulator = simulatedTime = droppedTime = lastElapsed = lastDroppedTime = 0;
    totalSteps = 0;
    lastSteps = 0;
}

vsim_clock_report Clock::snapshot() const {
    vsim_clock_report r;
    r.step_duration = stepDuration;
    r.max_steps_per_frame = maxStepsPerFrame;
    r.steps = lastSteps;
    r.elapsed = lastElapsed;
    r.total_steps = totalSteps;
    r.simulated_time = simulatedTime;
    r.backlog_time = accumulator;
    r.frame_dropped_time = lastDroppedTime;
    r.dropped_time = droppedTime;
    r.overloaded = lastDroppedTime > 0;
    return r;
}

}  // namespace vsim

using namespace vsim;

struct vsim_clock {
    Clock clock;
};

extern "C" {

const char* vsim_last_error(void) {
    static thread_local std::string copy;
    copy = g_lastError;
    return copy.c_str();
}

int vsim_abi_version(void) { return VSIM_ABI_VERSION; }

int vsim_stable_step_duration(double wave_rate, double* out) {
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    if (!std::isfinite(wave_rate) || wave_rate < 0)
        return fail(VSIM_ERR_RANGE, "waveRate must be a finite non-negative number");
    *out = stableStepDuration(wave_rate);
    return VSIM_OK;
}

int vsim_clock_create(double step_duration, uint32_t max_steps_per_frame, vsim_clock** out) {
    if (!out) return fail(VSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!std::isfinite(step_duration) || step_duration <= 0)
        return fail(VSIM_ERR_RANGE, "stepDuration must be a finite positive number");
    vsim_clock* c = new (std::nothrow) vsim_clock();
    if (!c) return fail(VSIM_ERR_NOMEM, "out of host memory");
    c->clock.stepDuration = step_duration;
    c->clock.maxStepsPerFrame = max_steps_per_frame == 0 ? kMaxStepsPerFrame : max_steps_per_frame;
    c->clock.reset();
    *out = c;
    return VSIM_OK;
}

int vsim_clock_destroy(vsim_clock* clock) {
    delete clock;
    return VSIM_OK;
}

int vsim_clock_consume(vsim_clock* clock, double elapsed, int force_step, vsim_clock_report* out) {
    if (!clock) return fail(VSIM_ERR_INVALID, "clock is NULL");
    if (!std::isfinite(elapsed) || elapsed < 0)
        return fail(VSIM_ERR_RANGE, "elapsed must be a finite non-negative number");
    clock->clock.consume(elapsed, force_step != 0);
    if (out) *out = clock->clock.snapshot();
    return VSIM_OK;
}

int vsim_clock_idle(vsim_clock* clock, vsim_clock_report* out) {
    if (!clock) return fail(VSIM_ERR_INVALID, "clock is NULL");
    clock->clock.idle();
    if (out) *out = clock->clock.snapshot();
    return VSIM_OK;
}

int vsim_clock_single_step(vsim_clock* clock, vsim_clock_report* out) {
    if (!clock) return fail(VSIM_ERR_INVALID, "clock is NULL");
    clock->clock.singleStep();
    if (out) *out = clock->clock.snapshot();
    return VSIM_OK;
}

int vsim_clock_set_step_duration(vsim_clock* clock, double step_duration) {
    if (!clock) return fail(VSIM_ERR_INVALID, "clock is NULL");
    if (!std::isfinite(step_duration) || step_duration <= 0)
        return fail(VSIM_ERR_RANGE, "stepDuration must be a finite positive number");
    clock->clock.stepDuration = step_duration;
    return VSIM_OK;
}

int vsim_clock_reset(vsim_clock* clock) {
    if (!clock) return fail(VSIM_ERR_INVALID, "clock is NULL");
    clock->clock.reset();
    return VSIM_OK;
}

int vsim_clock_snapshot(const vsim_clock* clock, vsim_clock_report* out) {
    if (!clock || !out) return fail(VSIM_ERR_INVALID, "NULL argument");
    *out = clock->clock.snapshot();
    return VSIM_OK;
}

int vsim_lame_parameters(const vsim_material* m, double* mu, double* lambda) {
    if (!m || !mu || !lambda) return fail(VSIM_ERR_INVALID, "NULL argument");
    lame(*m, *mu, *lambda);
    return VSIM_OK;
}

// compliance.js:30-37.
int vsim_element_compliance(const vsim_material* m, double rest_volume, double* deviatoric, double* hydrostatic,
                            double* gamma) {
    if (!m || !deviatoric || !hydrostatic || !gamma) return fail(VSIM_ERR_INVALID, "NULL argument");
    double mu, lambda;
    lame(*m, mu, lambda);
    *deviatoric = 1 / (mu * rest_volume);
    *hydrostatic = 1 / (lambda * rest_volume);
    *gamma = 1 + mu / lambda;
    return VSIM_OK;
}

// compliance.js:78-90: forty bisections of s^3 + s^2 + s = gamma - 1 on [0, 4].
double vsim_collapse_scale(double gamma) {
    double low = 0, high = 4;
    for (int i = 0; i < 40; i++) {
        const double s = (low + high) / 2;
        if (s * s * s + s * s + s < gamma - 1)
            low = s;
        else
            high = s;
    }
    return (low + high) / 2;
}

double vsim_wave_speed(const vsim_material* m) { return m ? waveSpeed(*m) : 0.0; }

}  // extern "C"
