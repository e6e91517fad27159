// vsim_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU restatement of the
// visionary-sim reference step that the GPU library is checked against.
//
// Each function follows one reference file, cited beside it, operation by
// operation and in the same evaluation order (left to right, WGSL's order for
// vector and matrix products), so that a float build of this file and a GPU
// kernel written to the same order agree bit for bit.
//
// Rounding: WGSL leaves contraction to the shader compiler, so the
// reference's own rounding differs from GPU to GPU. This restatement fixes
// one evaluation: a multiply followed by an add is fused (std::fma, one
// rounding) exactly where written below -- in dot products, matrix-vector
// products, cross products, the determinant, the Gram sums, the XPBD block
// and the position updates -- and every other operation rounds on its own.
// Build with -ffp-contract=off so the compiler fuses nothing else.
//
// Paths are relative to the reference project root.
#include "vsim_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors --

template <class T>
struct V3 {
    T x, y, z;
};

template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
// a * s + acc, fused per component.
template <class T> inline V3<T> fma3(V3<T> a, T s, V3<T> acc) {
    return {std::fma(a.x, s, acc.x), std::fma(a.y, s, acc.y), std::fma(a.z, s, acc.z)};
}
// dot: x first, then y and z fused in.
template <class T> inline T dot(V3<T> a, V3<T> b) { return std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x)); }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x))};
}

// Column-major 3x3, c[k] is column k (WGSL mat3x3f).
template <class T>
struct M3 {
    V3<T> c[3];
};

template <class T> inline M3<T> operator*(M3<T> m, T s) { return {{m.c[0] * s, m.c[1] * s, m.c[2] * s}}; }
// M * v = c0 v.x + c1 v.y + c2 v.z, summed left to right, fused.
template <class T> inline V3<T> mul(M3<T> m, V3<T> v) { return fma3(m.c[2], v.z, fma3(m.c[1], v.y, m.c[0] * v.x)); }
template <class T> inline M3<T> mul(M3<T> a, M3<T> b) { return {{mul(a, b.c[0]), mul(a, b.c[1]), mul(a, b.c[2])}}; }
template <class T> inline M3<T> transpose(M3<T> m) {
    return {{v3(m.c[0].x, m.c[1].x, m.c[2].x), v3(m.c[0].y, m.c[1].y, m.c[2].y),
             v3(m.c[0].z, m.c[1].z, m.c[2].z)}};
}
// Expansion order of mat3Determinant (packages/visionary-sim/src/sim/discretize/mat3.js:25-31).
template <class T> inline T determinant(M3<T> m) {
    const T m0 = m.c[0].x, m1 = m.c[0].y, m2 = m.c[0].z;
    const T m3 = m.c[1].x, m4 = m.c[1].y, m5 = m.c[1].z;
    const T m6 = m.c[2].x, m7 = m.c[2].y, m8 = m.c[2].z;
    const T t1 = std::fma(m4, m8, -(m7 * m5));
    const T t2 = std::fma(m1, m8, -(m7 * m2));
    const T t3 = std::fma(m1, m5, -(m4 * m2));
    return std::fma(m6, t3, std::fma(m0, t1, -(m3 * t2)));
}

// ------------------------------------------------------------ constants --

// corners.js:12-21: corner c sits at (c&1, (c>>1)&1, (c>>2)&1).
inline int cornerAxis(int c, int axis) { return (c >> axis) & 1; }

// kuhn.js:28-35.
const uint32_t KUHN_TETS[6][4] = {{0, 1, 3, 7}, {0, 5, 1, 7}, {0, 3, 2, 7},
                                  {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 6, 4, 7}};

// kuhn.js:59-69: Dm = [p1-p0, p2-p0, p3-p0] * h, column-major flat.
void kuhnRestShape(int t, double h, double out[9]) {
    const uint32_t* tet = KUHN_TETS[t];
    for (int col = 0; col < 3; col++)
        for (int axis = 0; axis < 3; axis++)
            out[col * 3 + axis] =
                double(cornerAxis(int(tet[col + 1]), axis) - cornerAxis(int(tet[0]), axis)) * h;
}

// mat3.js:25-55 (determinant and adjugate / det), computed in double.
double det9(const double* m) {
    return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
           m[6] * (m[1] * m[5] - m[4] * m[2]);
}
void inverse9(const double* m, double* out) {
    const double s = 1.0 / det9(m);
    out[0] = (m[4] * m[8] - m[7] * m[5]) * s;
    out[1] = (m[7] * m[2] - m[1] * m[8]) * s;
    out[2] = (m[1] * m[5] - m[4] * m[2]) * s;
    out[3] = (m[6] * m[5] - m[3] * m[8]) * s;
    out[4] = (m[0] * m[8] - m[6] * m[2]) * s;
    out[5] = (m[3] * m[2] - m[0] * m[5]) * s;
    out[6] = (m[3] * m[7] - m[6] * m[4]) * s;
    out[7] = (m[6] * m[1] - m[0] * m[7]) * s;
    out[8] = (m[0] * m[4] - m[3] * m[1]) * s;
}

// The unit-cube inverses as the GPU receives them: computed in double from
// f32 inputs, stored as f32 (kuhn.js:78-80 into elasticCells.js:85-107).
template <class T>
M3<T> kuhnUnitInverse(int t) {
    double dm[9], inv[9];
    kuhnRestShape(t, 1.0, dm);
    inverse9(dm, inv);
    M3<T> m;
    for (int col = 0; col < 3; col++) m.c[col] = v3(T(inv[col * 3]), T(inv[col * 3 + 1]), T(inv[col * 3 + 2]));
    return m;
}

// stretch.js:5-7: all 28 corner pairs in order, unit rest length.
struct Edge {
    int a, b;
    double len;
};
std::vector<Edge> stretchEdges() {
    std::vector<Edge> edges;
    for (int i = 0; i < 8; i++)
        for (int j = i + 1; j < 8; j++) {
            const double dx = cornerAxis(i, 0) - cornerAxis(j, 0);
            const double dy = cornerAxis(i, 1) - cornerAxis(j, 1);
            const double dz = cornerAxis(i, 2) - cornerAxis(j, 2);
            edges.push_back({i, j, std::hypot(std::hypot(dx, dy), dz)});
        }
    return edges;
}

// material.js:66,101-108.
void lame(const vsim_material& m, double& mu, double& lambda) {
    const double nu = std::min(std::max(m.poisson_ratio, 0.25), 0.49);
    const double e = std::max(m.youngs_modulus, 1.0);
    mu = e / (2 * (1 + nu));
    lambda = (e * nu) / ((1 + nu) * (1 - 2 * nu));
}

// -------------------------------------------------------------- the sim --

constexpr uint32_t BUCKET_SLOTS = 32;  // contacts.wgsl:75
constexpr double CONTACT_RADIUS_CELLS = 0.5;  // voxelLattice.js:17
constexpr double GRID_LIMIT = double(1u << 26);

struct Body {
    uint32_t cellDims[3], nodeDims[3];
    uint32_t nodeOffset, nodeCount;
    double origin[3], h;
    vsim_material material;
    std::vector<uint32_t> cellsByColor[8];  // linear cell indices (lattice.js:189-219)
    std::vector<uint8_t> occupancy;
};

template <class T>
struct BodyParams {  // what the kernels read, per body
    T h, alphaDev, alphaHyd, gamma, relaxation, maxStretch, friction, damping;
};

template <class T>
struct Sim {
    std::vector<Body> bodies;
    uint32_t nodeCount = 0;
    std::vector<V3<T>> pos, prev, vel;
    std::vector<T> invMass;   // material (Particles.invMass)
    std::vector<T> gpuMass;   // with static and held nodes zeroed (particles.js:206-215)
    std::vector<uint8_t> isStatic;
    std::vector<BodyParams<T>> params;
    // colour-major cell list over all bodies (elasticCells.js:143-163)
    std::vector<uint32_t> cellBody[8], cellLinear[8];
    // contact
    std::vector<uint32_t> sNode, sBody, sCoord;
    std::vector<T> sRadius;
    // Contact grids: one shared by every body, or one per body when the
    // bodies are isolated (never touch each other).
    struct OGrid {
        double origin[3];
        double bucket;
        uint32_t dims[3];
        size_t base;
    };
    std::vector<OGrid> grids;
    size_t bucketTotal = 0;
    bool isolated = false;
    bool contact = true, selfContact = false;
    // drive
    std::vector<uint32_t> driven;
    std::vector<V3<T>> drivenOffset;
    int law = VSIM_DRIVE_HARD;
    T responseTime = T(0.05);  // kinematicDrive.js:65
    V3<T> grabTarget{0, 0, 0}, grabVelocity{0, 0, 0};
    // frame
    double stepDuration = 1.0 / 240;
    double gravity[3] = {0, -9.81, 0};
    double tankMin[3], tankMax[3];
    uint32_t iterations = 1;
};

// Rounds a double to the precision the kernels hold it in.
template <class T> inline T asT(double v) { return T(v); }

template <class T>
void uploadParams(Sim<T>& s, uint32_t b) {
    Body& body = s.bodies[b];
    double mu, lambda;
    lame(body.material, mu, lambda);
    // compliance.js:30-37 with tetRestVolume (kuhn.js:48-50).
    const double volume = (1.0 / 6.0) * std::pow(body.h, 3.0);
    BodyParams<T>& p = s.params[b];
    p.h = asT<T>(body.h);
    p.alphaDev = asT<T>(1 / (mu * volume));
    p.alphaHyd = asT<T>(1 / (lambda * volume));
    p.gamma = asT<T>(1 + mu / lambda);
    p.relaxation = asT<T>(body.material.relaxation);
    p.maxStretch = asT<T>(body.material.max_stretch);
    p.friction = asT<T>(body.material.friction);
    p.damping = asT<T>(body.material.damping);
}

// particles.js:206-215.
template <class T>
void uploadGpuMasses(Sim<T>& s) {
    s.gpuMass = s.invMass;
    for (uint32_t n = 0; n < s.nodeCount; n++)
        if (s.isStatic[n]) s.gpuMass[n] = 0;
    if (s.law == VSIM_DRIVE_HARD)
        for (uint32_t n : s.driven) s.gpuMass[n] = 0;
}

// lattice.js:128-158.
uint32_t surfaceNodesOf(const uint32_t cd[3], const uint8_t* occ, std::vector<uint32_t>& found) {
    const uint32_t nd[3] = {cd[0] + 1, cd[1] + 1, cd[2] + 1};
    for (uint32_t k = 0; k < nd[2]; k++)
        for (uint32_t j = 0; j < nd[1]; j++)
            for (uint32_t i = 0; i < nd[0]; i++) {
                int filled = 0;
                for (int c = 0; c < 8; c++) {
                    const int64_t ci = int64_t(i) + cornerAxis(c, 0) - 1;
                    const int64_t cj = int64_t(j) + cornerAxis(c, 1) - 1;
                    const int64_t ck = int64_t(k) + cornerAxis(c, 2) - 1;
                    const bool outside = ci < 0 || cj < 0 || ck < 0 || ci >= cd[0] || cj >= cd[1] || ck >= cd[2];
                    filled += outside ? 0 : (occ[ci + cd[0] * (cj + cd[1] * ck)] ? 1 : 0);
                }
                if (filled > 0 && filled < 8) found.push_back(i + nd[0] * (j + nd[1] * k));
            }
    return uint32_t(found.size());
}

// broadphase.js:46-58.
void gridLayout(const double mn[3], const double mx[3], double bucket, double origin[3], double& edge,
                uint32_t dims[3]) {
    edge = bucket > 0 ? bucket : std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]});
    for (int a = 0; a < 3; a++) {
        dims[a] = uint32_t(std::max(1.0, std::ceil((mx[a] - mn[a]) / edge)) + 2);
        origin[a] = mn[a] - edge;
    }
}

template <class T>
int build(Sim<T>& s, const vsim_body_desc* descs, uint32_t n, const vsim_tank* tank, bool isolated) {
    s.isolated = isolated;
    s.bodies.resize(n);
    s.params.resize(n);
    for (int a = 0; a < 3; a++) {
        s.tankMin[a] = tank ? tank->min[a] : -INFINITY;
        s.tankMax[a] = tank ? tank->max[a] : INFINITY;
    }
    uint32_t offset = 0;
    for (uint32_t b = 0; b < n; b++) {
        const vsim_body_desc& d = descs[b];
        Body& body = s.bodies[b];
        for (int a = 0; a < 3; a++) {
            body.cellDims[a] = d.cell_dims[a];
            body.nodeDims[a] = d.cell_dims[a] + 1;
            body.origin[a] = d.origin[a];
        }
        body.h = d.h;
        body.material = d.material;
        body.nodeOffset = offset;
        body.nodeCount = body.nodeDims[0] * body.nodeDims[1] * body.nodeDims[2];
        const size_t cells = size_t(d.cell_dims[0]) * d.cell_dims[1] * d.cell_dims[2];
        body.occupancy.assign(d.occupancy, d.occupancy + cells);
        offset += body.nodeCount;
    }
    s.nodeCount = offset;
    s.pos.assign(offset, V3<T>{0, 0, 0});
    s.vel.assign(offset, V3<T>{0, 0, 0});
    s.invMass.assign(offset, T(0));
    s.isStatic.assign(offset, 0);

    for (uint32_t b = 0; b < n; b++) {
        Body& body = s.bodies[b];
        const uint32_t* cd = body.cellDims;
        const uint32_t* nd = body.nodeDims;
        // lattice.js:171-181: rest positions, f32 of a double sum.
        for (uint32_t k = 0; k < nd[2]; k++)
            for (uint32_t j = 0; j < nd[1]; j++)
                for (uint32_t i = 0; i < nd[0]; i++) {
                    const uint32_t node = body.nodeOffset + i + nd[0] * (j + nd[1] * k);
                    s.pos[node] = v3(asT<T>(body.origin[0] + i * body.h), asT<T>(body.origin[1] + j * body.h),
                                     asT<T>(body.origin[2] + k * body.h));
                }
        // lattice.js:185-224: lumped mass, colour groups, inverse mass.
        const double cornerMass = body.material.density * body.h * body.h * body.h / 8;
        std::vector<T> mass(body.nodeCount, T(0));
        for (uint32_t k = 0; k < cd[2]; k++)
            for (uint32_t j = 0; j < cd[1]; j++)
                for (uint32_t i = 0; i < cd[0]; i++) {
                    const uint32_t cell = i + cd[0] * (j + cd[1] * k);
                    if (!body.occupancy[cell]) continue;
                    body.cellsByColor[(i & 1) | ((j & 1) << 1) | ((k & 1) << 2)].push_back(cell);
                    for (int c = 0; c < 8; c++) {
                        const uint32_t node = (i + cornerAxis(c, 0)) +
                                              nd[0] * ((j + cornerAxis(c, 1)) + nd[1] * (k + cornerAxis(c, 2)));
                        mass[node] = asT<T>(double(mass[node]) + cornerMass);
                    }
                }
        for (uint32_t m = 0; m < body.nodeCount; m++)
            s.invMass[body.nodeOffset + m] = mass[m] > 0 ? asT<T>(1.0 / double(mass[m])) : T(0);
        for (uint32_t i = 0; i < descs[b].static_count; i++) {
            const uint32_t node = descs[b].static_nodes[i];
            if (node >= body.nodeCount) return VSIM_ERR_RANGE;
            s.isStatic[body.nodeOffset + node] = 1;
        }
        uploadParams(s, b);
    }
    s.prev = s.pos;
    uploadGpuMasses(s);

    for (int c = 0; c < 8; c++)
        for (uint32_t b = 0; b < n; b++)
            for (uint32_t cell : s.bodies[b].cellsByColor[c]) {
                s.cellBody[c].push_back(b);
                s.cellLinear[c].push_back(cell);
            }

    // bodyContact.js:325-343: surface records, radius h/2, bucket = 2 x widest.
    double widest = 0;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t b = 0; b < n; b++) {
        Body& body = s.bodies[b];
        std::vector<uint32_t> nodes;
        surfaceNodesOf(body.cellDims, body.occupancy.data(), nodes);
        const float radius = float(body.h * CONTACT_RADIUS_CELLS);
        for (uint32_t node : nodes) {
            const uint32_t i = node % body.nodeDims[0];
            const uint32_t j = (node / body.nodeDims[0]) % body.nodeDims[1];
            const uint32_t k = node / (body.nodeDims[0] * body.nodeDims[1]);
            s.sNode.push_back(body.nodeOffset + node);
            s.sBody.push_back(b);
            s.sCoord.push_back(i | (j << 10) | (k << 20));
            s.sRadius.push_back(sizeof(T) == 4 ? T(radius) : T(body.h * CONTACT_RADIUS_CELLS));
            widest = std::max(widest, double(radius));
        }
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], body.origin[a]);
            hi[a] = std::max(hi[a], body.origin[a] + body.cellDims[a] * body.h);
        }
    }
    typename Sim<T>::OGrid g{};
    double edge;
    if (s.isolated) {
        // Each body's own grid: its rest box padded by a quarter of its
        // extent (at least four cells) per side, clipped to the tank, buckets
        // one cell.
        for (uint32_t b = 0; b < n; b++) {
            const Body& body = s.bodies[b];
            double mn[3], mx[3];
            for (int a = 0; a < 3; a++) {
                const double pad = std::max(0.25 * body.cellDims[a] * body.h, 8 * body.h * CONTACT_RADIUS_CELLS);
                mn[a] = std::max(s.tankMin[a], body.origin[a] - pad);
                mx[a] = std::min(s.tankMax[a], body.origin[a] + body.cellDims[a] * body.h + pad);
            }
            gridLayout(mn, mx, body.h * CONTACT_RADIUS_CELLS * 2, g.origin, g.bucket, g.dims);
            g.base = s.bucketTotal;
            s.bucketTotal += size_t(g.dims[0]) * g.dims[1] * g.dims[2];
            s.grids.push_back(g);
        }
        return VSIM_OK;
    }
    gridLayout(s.tankMin, s.tankMax, widest * 2, g.origin, edge, g.dims);
    const double buckets = double(g.dims[0]) * g.dims[1] * g.dims[2];
    bool finite = true;
    for (int a = 0; a < 3; a++) finite = finite && std::isfinite(s.tankMin[a]) && std::isfinite(s.tankMax[a]);
    if (!finite || !(buckets <= GRID_LIMIT)) {
        // The library's rule for an unbounded or huge tank: the bodies' rest
        // box padded by half its extent (at least four buckets) per side,
        // clipped to the tank.
        double mn[3], mx[3];
        for (int a = 0; a < 3; a++) {
            const double pad = std::max(0.5 * (hi[a] - lo[a]), 4 * widest * 2);
            mn[a] = std::max(s.tankMin[a], lo[a] - pad);
            mx[a] = std::min(s.tankMax[a], hi[a] + pad);
        }
        gridLayout(mn, mx, widest * 2, g.origin, edge, g.dims);
    }
    g.bucket = edge;
    g.base = 0;
    s.bucketTotal = size_t(g.dims[0]) * g.dims[1] * g.dims[2];
    s.grids.push_back(g);
    return VSIM_OK;
}

// ------------------------------------------------------------- kernels --

// predict.wgsl:19-36.
template <class T>
void predict(Sim<T>& s, T dt, V3<T> g) {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < int64_t(s.nodeCount); n++) {
        if (s.gpuMass[n] == T(0)) continue;
        const V3<T> v = s.vel[n] + g * dt;
        const V3<T> p = s.pos[n];
        s.prev[n] = p;
        s.pos[n] = p + v * dt;
        s.vel[n] = v;
    }
}

// driveHard.wgsl:15-35 / driveCompliant.wgsl:24-41.
template <class T>
void drive(Sim<T>& s, T dt) {
    for (size_t i = 0; i < s.driven.size(); i++) {
        const uint32_t n = s.driven[i];
        const V3<T> goal = s.grabTarget + s.drivenOffset[i];
        if (s.law == VSIM_DRIVE_HARD) {
            const V3<T> here = s.pos[n];
            const V3<T> step = s.grabVelocity * dt;
            const V3<T> toGoal = goal - here;
            const V3<T> next = here + (dot(step, step) >= dot(toGoal, toGoal) ? toGoal : step);
            s.prev[n] = here;
            s.pos[n] = next;
            s.vel[n] = (next - here) / dt;
        } else {
            const V3<T> p = s.pos[n];
            const T dt2 = dt * dt;
            const T tau2 = s.responseTime * s.responseTime;
            const T frac = dt2 / (dt2 + tau2);
            s.pos[n] = p + (goal - p) * frac;
        }
    }
}

// xpbdCouple.wgsl:58-71.
template <class T>
inline void xpbdCouple(T cx, T cy, T ax, T ay, T relax, T rx, T ry, T gx, T gy, T gz, T& lx, T& ly) {
    const T stiffened = T(1) + relax;
    const T a00 = std::fma(gx, stiffened, ax);
    const T a01 = gy * stiffened;
    const T a11 = std::fma(gz, stiffened, ay);
    const T det = std::fma(a00, a11, -(a01 * a01));
    if (det < T(1e-20)) {
        lx = T(0);
        ly = T(0);
        return;
    }
    const T bx = -std::fma(rx, relax, cx);
    const T by = -std::fma(ry, relax, cy);
    lx = std::fma(a11, bx, -(a01 * by)) / det;
    ly = std::fma(a00, by, -(a01 * bx)) / det;
}

// sum_i w_i dot(a_i, b_i) over a tetrahedron's four nodes, fused.
template <class T>
inline T weighted4(T w0, T w1, T w2, T w3, T e0, T e1, T e2, T e3) {
    return std::fma(w3, e3, std::fma(w2, e2, std::fma(w1, e1, w0 * e0)));
}

// p + (d lx + h ly) w, fused.
template <class T>
inline V3<T> moved(V3<T> p, V3<T> d, V3<T> h, T lx, T ly, T w) {
    return fma3(fma3(h, ly, d * lx), w, p);
}

// project.wgsl:90-152: one Kuhn tetrahedron of a cell, in place.
template <class T>
inline void projectTet(V3<T>* p, const V3<T>* prev, const T* w, const uint32_t tet[4], const M3<T>& Bunit,
                       T restScale, T alphaDev, T alphaHyd, T gamma, T relax) {
    const uint32_t i0 = tet[0], i1 = tet[1], i2 = tet[2], i3 = tet[3];
    const T w0 = w[i0], w1 = w[i1], w2 = w[i2], w3 = w[i3];
    if (w0 + w1 + w2 + w3 == T(0)) return;
    const M3<T> B = Bunit * restScale;
    const M3<T> Bt = transpose(B);
    const V3<T> base = p[i0];
    const M3<T> F = mul(M3<T>{{p[i1] - base, p[i2] - base, p[i3] - base}}, B);
    const T cDev = std::sqrt(dot(F.c[0], F.c[0]) + dot(F.c[1], F.c[1]) + dot(F.c[2], F.c[2]));
    const T cHyd = determinant(F) - gamma;
    const T inv = cDev > T(1e-9) ? T(1) / cDev : T(0);
    const M3<T> mDev = mul(F * inv, Bt);
    const M3<T> mHyd = mul(M3<T>{{cross(F.c[1], F.c[2]), cross(F.c[2], F.c[0]), cross(F.c[0], F.c[1])}}, Bt);
    const V3<T> d1 = mDev.c[0], d2 = mDev.c[1], d3 = mDev.c[2];
    const V3<T> d0 = -(d1 + d2 + d3);
    const V3<T> h1 = mHyd.c[0], h2 = mHyd.c[1], h3 = mHyd.c[2];
    const V3<T> h0 = -(h1 + h2 + h3);
    const T gx = weighted4(w0, w1, w2, w3, dot(d0, d0), dot(d1, d1), dot(d2, d2), dot(d3, d3));
    const T gy = weighted4(w0, w1, w2, w3, dot(d0, h0), dot(d1, h1), dot(d2, h2), dot(d3, h3));
    const T gz = weighted4(w0, w1, w2, w3, dot(h0, h0), dot(h1, h1), dot(h2, h2), dot(h3, h3));
    const V3<T> x0 = p[i0] - prev[i0];
    const V3<T> x1 = p[i1] - prev[i1];
    const V3<T> x2 = p[i2] - prev[i2];
    const V3<T> x3 = p[i3] - prev[i3];
    const T rx = dot(d0, x0) + dot(d1, x1) + dot(d2, x2) + dot(d3, x3);
    const T ry = dot(h0, x0) + dot(h1, x1) + dot(h2, x2) + dot(h3, x3);
    T lx, ly;
    xpbdCouple(cDev, cHyd, alphaDev, alphaHyd, relax, rx, ry, gx, gy, gz, lx, ly);
    p[i0] = moved(p[i0], d0, h0, lx, ly, w0);
    p[i1] = moved(p[i1], d1, h1, lx, ly, w1);
    p[i2] = moved(p[i2], d2, h2, lx, ly, w2);
    p[i3] = moved(p[i3], d3, h3, lx, ly, w3);
}

template <class T>
struct FrameConsts {
    M3<T> kuhn[6];
    T edgeLen[28];
    int edgeA[28], edgeB[28];
};

template <class T>
FrameConsts<T> frameConsts() {
    FrameConsts<T> k;
    for (int t = 0; t < 6; t++) k.kuhn[t] = kuhnUnitInverse<T>(t);
    const std::vector<Edge> edges = stretchEdges();
    for (int e = 0; e < 28; e++) {
        k.edgeA[e] = edges[e].a;
        k.edgeB[e] = edges[e].b;
        k.edgeLen[e] = T(edges[e].len);
    }
    return k;
}

// project.wgsl:35-184, one colour pass.
template <class T>
void colorPass(Sim<T>& s, int color, bool limitOnly, T dt, const FrameConsts<T>& K) {
    const T invDt2 = T(1) / (dt * dt);
    const std::vector<uint32_t>& bodies = s.cellBody[color];
    const std::vector<uint32_t>& linear = s.cellLinear[color];
#pragma omp parallel for schedule(static)
    for (int64_t slot = 0; slot < int64_t(linear.size()); slot++) {
        const Body& body = s.bodies[bodies[slot]];
        const BodyParams<T>& cp = s.params[bodies[slot]];
        if (limitOnly && cp.maxStretch <= T(1)) continue;
        const uint32_t cell = linear[slot];
        const uint32_t cx = cell % body.cellDims[0];
        const uint32_t cy = (cell / body.cellDims[0]) % body.cellDims[1];
        const uint32_t cz = cell / (body.cellDims[0] * body.cellDims[1]);
        uint32_t ids[8];
        V3<T> p[8], prev[8];
        T w[8];
        for (int c = 0; c < 8; c++) {
            const uint32_t n = body.nodeOffset + (cx + cornerAxis(c, 0)) +
                               body.nodeDims[0] * ((cy + cornerAxis(c, 1)) + body.nodeDims[1] * (cz + cornerAxis(c, 2)));
            ids[c] = n;
            p[c] = s.pos[n];
            prev[c] = s.prev[n];
            w[c] = s.gpuMass[n];
        }
        if (!limitOnly) {
            const T alphaDev = cp.alphaDev * invDt2;
            const T alphaHyd = cp.alphaHyd * invDt2;
            const T relax = cp.relaxation / dt;
            const T restScale = T(1) / cp.h;
            for (int t = 0; t < 6; t++)
                projectTet(p, prev, w, KUHN_TETS[t], K.kuhn[t], restScale, alphaDev, alphaHyd, cp.gamma, relax);
        }
        if (cp.maxStretch > T(1)) {
            for (int sweep = 0; sweep < 2; sweep++)
                for (int e = 0; e < 28; e++) {
                    const int a = K.edgeA[e], b = K.edgeB[e];
                    const V3<T> delta = p[b] - p[a];
                    const T len = length(delta);
                    const T maximum = K.edgeLen[e] * cp.h * cp.maxStretch;
                    const T weight = w[a] + w[b];
                    if (len > maximum && weight > T(0)) {
                        const V3<T> correction = delta * ((len - maximum) / (len * weight));
                        p[a] = p[a] + w[a] * correction;
                        p[b] = p[b] - w[b] * correction;
                    }
                }
        }
        for (int c = 0; c < 8; c++) s.pos[ids[c]] = p[c];
    }
}

// contacts.wgsl:84-91 (gridCoord, bucketAt), evaluated in T.
template <class T>
inline const typename Sim<T>::OGrid& gridOf(const Sim<T>& s, uint32_t body) {
    return s.grids[s.isolated ? body : 0];
}

// Index into the bucket arrays: the grid's base plus its linear index.
template <class T>
inline size_t bucketOf(const Sim<T>& s, uint32_t body, V3<T> p, uint32_t coord[3]) {
    const typename Sim<T>::OGrid& g = gridOf(s, body);
    const T o[3] = {asT<T>(g.origin[0]), asT<T>(g.origin[1]), asT<T>(g.origin[2])};
    const T size = asT<T>(g.bucket);
    const T q[3] = {p.x, p.y, p.z};
    for (int a = 0; a < 3; a++) {
        const T last = T(g.dims[a]) - T(1);
        const T f = std::floor((q[a] - o[a]) / size);
        coord[a] = uint32_t(std::min(std::max(f, T(0)), last));
    }
    return g.base + coord[0] + size_t(g.dims[0]) * (coord[1] + size_t(g.dims[1]) * coord[2]);
}

// Whether records a and b may touch. The reference drops every same-body
// pair (collide.wgsl:66); with self contact on, a same-body pair is kept
// when its nodes share no cell (rest grid distance above one on some axis).
template <class T>
inline bool admitted(const Sim<T>& s, uint32_t a, uint32_t b) {
    if (s.sBody[a] != s.sBody[b]) return !s.isolated;
    if (!s.selfContact) return false;
    const uint32_t ca = s.sCoord[a], cb = s.sCoord[b];
    for (int axis = 0; axis < 3; axis++) {
        const int ia = int((ca >> (10 * axis)) & 1023u), ib = int((cb >> (10 * axis)) & 1023u);
        if (std::abs(ia - ib) > 1) return true;
    }
    return false;
}

// bin.wgsl + sort.wgsl: each bucket's live entries in ascending record order,
// at most BUCKET_SLOTS of them visible.
template <class T>
struct Binned {
    std::vector<uint32_t> start, count, entries;
};

template <class T>
Binned<T> binAll(const Sim<T>& s) {
    Binned<T> g;
    const size_t buckets = s.bucketTotal;
    const size_t S = s.sNode.size();
    std::vector<size_t> key(S);
    g.count.assign(buckets, 0);
    g.start.assign(buckets, 0);
    for (size_t r = 0; r < S; r++) {
        uint32_t coord[3];
        key[r] = bucketOf(s, s.sBody[r], s.pos[s.sNode[r]], coord);
        g.count[key[r]]++;
    }
    uint32_t run = 0;
    for (size_t b = 0; b < buckets; b++) {
        g.start[b] = run;
        run += g.count[b];
    }
    g.entries.resize(S);
    std::vector<uint32_t> fill(g.start);
    for (size_t r = 0; r < S; r++) g.entries[fill[key[r]]++] = uint32_t(r);
    return g;
}

// collide.wgsl:16-125 for record r; `emit` sees every counted hit.
template <class T, class Emit>
inline void gather(const Sim<T>& s, const Binned<T>& g, uint32_t r, V3<T>& sum, T& hits, Emit emit) {
    const uint32_t node = s.sNode[r];
    const uint32_t body = s.sBody[r];
    const T radius = s.sRadius[r];
    const T wi = s.gpuMass[node];
    const V3<T> pi = s.pos[node];
    const V3<T> movedI = pi - s.prev[node];
    const T frictionI = s.params[body].friction;
    sum = V3<T>{0, 0, 0};
    hits = T(0);
    uint32_t centre[3];
    bucketOf(s, body, pi, centre);
    const typename Sim<T>::OGrid& grid = gridOf(s, body);
    const int dims[3] = {int(grid.dims[0]), int(grid.dims[1]), int(grid.dims[2])};
    for (int dz = -1; dz <= 1; dz++) {
        const int z = int(centre[2]) + dz;
        if (z < 0 || z >= dims[2]) continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = int(centre[1]) + dy;
            if (y < 0 || y >= dims[1]) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int x = int(centre[0]) + dx;
                if (x < 0 || x >= dims[0]) continue;
                const size_t bucket = grid.base + uint32_t(x) + size_t(grid.dims[0]) * (uint32_t(y) + size_t(grid.dims[1]) * uint32_t(z));
                const uint32_t held = std::min(g.count[bucket], BUCKET_SLOTS);
                for (uint32_t k = 0; k < held; k++) {
                    const uint32_t other = g.entries[g.start[bucket] + k];
                    if (!admitted(s, r, other)) continue;
                    const uint32_t mateBody = s.sBody[other];
                    const uint32_t mate = s.sNode[other];
                    const V3<T> pj = s.pos[mate];
                    const V3<T> d = pi - pj;
                    const T dist2 = dot(d, d);
                    const T reach = radius + s.sRadius[other];
                    if (dist2 >= reach * reach) continue;
                    const T wj = s.gpuMass[mate];
                    const T total = wi + wj;
                    if (total <= T(0)) continue;
                    const T share = wi / total;
                    const T dist = std::sqrt(dist2);
                    V3<T> normal = v3(T(0), node < mate ? T(1) : T(-1), T(0));
                    if (dist > T(1e-9)) normal = d / dist;
                    const T depth = reach - dist;
                    V3<T> correction = normal * (depth * share);
                    const V3<T> sliding = movedI - (pj - s.prev[mate]);
                    const V3<T> tangent = sliding - normal * dot(sliding, normal);
                    const T slid = length(tangent);
                    if (slid > T(1e-9)) {
                        const T mu = std::min(frictionI, s.params[mateBody].friction);
                        correction = correction - tangent * (share * std::min(T(1), mu * depth / slid));
                    }
                    sum = sum + correction;
                    hits = hits + T(1);
                    emit(other);
                }
            }
        }
    }
}

// bin, sort, collide, settle (bodyContact.js:393-404).
template <class T>
void contactPass(Sim<T>& s) {
    const size_t S = s.sNode.size();
    if (!s.contact || S == 0) return;
    const Binned<T> g = binAll(s);
    std::vector<V3<T>> delta(S);
    std::vector<T> hits(S);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < int64_t(S); r++) gather(s, g, uint32_t(r), delta[r], hits[r], [](uint32_t) {});
    // settle.wgsl:20-36 with gain 1 (bodyContact.js:48).
    const T gain = T(1);
    for (size_t r = 0; r < S; r++) {
        if (hits[r] > T(0)) {
            const uint32_t node = s.sNode[r];
            const V3<T> step = delta[r] * (gain / hits[r]);
            s.pos[node] = s.pos[node] + step;
        }
    }
}

// finalize.wgsl:29-42.
template <class T>
inline V3<T> resolvePlane(V3<T> p, V3<T> prev, V3<T> normal, T depth, T friction) {
    if (depth <= T(0)) return p;
    V3<T> q = p + normal * depth;
    const V3<T> delta = q - prev;
    const V3<T> tangent = delta - normal * dot(delta, normal);
    const T len = length(tangent);
    if (len > T(1e-9)) q = q - tangent * std::min(T(1), friction * depth / len);
    return q;
}

// The per-body velocity factor exp(-damping dt) of finalize.wgsl:72. The
// library evaluates it once per body on the host the same way, in double,
// rounded to T.
template <class T>
inline T dampFactor(T damping, T dt) {
    const T arg = -damping * dt;
    return T(std::exp(double(arg)));
}

// finalize.wgsl:44-74.
template <class T>
void finalize(Sim<T>& s, T dt) {
    const V3<T> mn = v3(asT<T>(s.tankMin[0]), asT<T>(s.tankMin[1]), asT<T>(s.tankMin[2]));
    const V3<T> mx = v3(asT<T>(s.tankMax[0]), asT<T>(s.tankMax[1]), asT<T>(s.tankMax[2]));
    std::vector<T> factor(s.bodies.size());
    for (size_t b = 0; b < s.bodies.size(); b++) factor[b] = dampFactor(s.params[b].damping, dt);
#pragma omp parallel for schedule(static)
    for (int64_t bi = 0; bi < int64_t(s.bodies.size()); bi++) {
        const Body& body = s.bodies[bi];
        const T fr = s.params[bi].friction;
        for (uint32_t m = 0; m < body.nodeCount; m++) {
            const uint32_t n = body.nodeOffset + m;
            if (s.gpuMass[n] == T(0)) continue;
            const V3<T> prev = s.prev[n];
            V3<T> p = s.pos[n];
            p = resolvePlane(p, prev, v3(T(0), T(1), T(0)), mn.y - p.y, fr);
            p = resolvePlane(p, prev, v3(T(1), T(0), T(0)), mn.x - p.x, fr);
            p = resolvePlane(p, prev, v3(T(-1), T(0), T(0)), p.x - mx.x, fr);
            p = resolvePlane(p, prev, v3(T(0), T(0), T(1)), mn.z - p.z, fr);
            p = resolvePlane(p, prev, v3(T(0), T(0), T(-1)), p.z - mx.z, fr);
            s.pos[n] = p;
            V3<T> v = (p - prev) / dt;
            v = v * factor[bi];
            s.vel[n] = v;
        }
    }
}

// stepper.js:101-108 with the constraint order of simulator.js:83:
// predict, drive, elastic colours (x iterations, + 3 limit-only sweeps when
// any body limits stretch, elasticCells.js:199-214), contact, finalize.
template <class T>
void dispatch(Sim<T>& s, uint32_t steps) {
    if (steps < 1 || s.nodeCount == 0) return;
    const T dt = asT<T>(s.stepDuration);
    const V3<T> g = v3(asT<T>(s.gravity[0]), asT<T>(s.gravity[1]), asT<T>(s.gravity[2]));
    const FrameConsts<T> K = frameConsts<T>();
    bool limited = false;
    for (const auto& b : s.bodies) limited = limited || b.material.max_stretch > 1;
    for (uint32_t step = 0; step < steps; step++) {
        predict(s, dt, g);
        if (!s.driven.empty()) drive(s, dt);
        for (uint32_t it = 0; it < s.iterations; it++)
            for (int c = 0; c < 8; c++) colorPass(s, c, false, dt, K);
        if (limited)
            for (int sweep = 0; sweep < 3; sweep++)
                for (int c = 0; c < 8; c++) colorPass(s, c, true, dt, K);
        contactPass(s);
        finalize(s, dt);
    }
}

// sample.wgsl:40-80.
template <class T>
void deformationAt(const V3<T>* nodes, const uint32_t nodeDims[3], const uint32_t cellDims[3], const T origin[3],
                   T h, V3<T> rest, V3<T>& position, M3<T>& gradient) {
    const T inv = T(1) / h;
    const T r[3] = {rest.x, rest.y, rest.z};
    T local[3];
    uint32_t base[3];
    for (int a = 0; a < 3; a++) {
        const T grid = (r[a] - origin[a]) * inv;
        const T cell = std::min(std::max(std::floor(grid), T(0)), T(cellDims[a]) - T(1));
        local[a] = grid - cell;
        base[a] = uint32_t(cell);
    }
    position = V3<T>{0, 0, 0};
    V3<T> col0{0, 0, 0}, col1{0, 0, 0}, col2{0, 0, 0};
    for (int c = 0; c < 8; c++) {
        T f[3], dir[3];
        for (int a = 0; a < 3; a++) {
            const bool far = cornerAxis(c, a) == 1;
            f[a] = far ? local[a] : T(1) - local[a];
            dir[a] = far ? T(1) : T(-1);
        }
        const uint32_t ix = base[0] + cornerAxis(c, 0), iy = base[1] + cornerAxis(c, 1), iz = base[2] + cornerAxis(c, 2);
        const V3<T> p = nodes[ix + nodeDims[0] * (iy + nodeDims[1] * iz)];
        position = position + p * (f[0] * f[1] * f[2]);
        const V3<T> gv = v3(dir[0] * f[1] * f[2], dir[1] * f[0] * f[2], dir[2] * f[0] * f[1]) * inv;
        col0 = col0 + p * gv.x;
        col1 = col1 + p * gv.y;
        col2 = col2 + p * gv.z;
    }
    gradient = M3<T>{{col0, col1, col2}};
}

// covariance.wgsl:18-42; returns xx, xy, xz, yy, yz, zz.
template <class T>
void deformedCovariance(const M3<T>& F, const T q[4], const T scale[3], T out6[6]) {
    const T x = q[0], y = q[1], z = q[2], w = q[3];
    const M3<T> basis{{v3(T(1) - T(2) * (y * y + z * z), T(2) * (x * y + z * w), T(2) * (x * z - y * w)),
                       v3(T(2) * (x * y - z * w), T(1) - T(2) * (x * x + z * z), T(2) * (y * z + x * w)),
                       v3(T(2) * (x * z + y * w), T(2) * (y * z - x * w), T(1) - T(2) * (x * x + y * y))}};
    const M3<T> a{{mul(F, basis.c[0]) * scale[0], mul(F, basis.c[1]) * scale[1], mul(F, basis.c[2]) * scale[2]}};
    const M3<T> cov = mul(a, transpose(a));
    out6[0] = cov.c[0].x;
    out6[1] = cov.c[0].y;
    out6[2] = cov.c[0].z;
    out6[3] = cov.c[1].y;
    out6[4] = cov.c[1].z;
    out6[5] = cov.c[2].z;
}

// ellipsoid.wgsl:20-91 (CPU twin apps/simulator/src/render/ellipsoid.js:40-149):
// a covariance (xx, xy, xz, yy, yz, zz) taken apart into a unit quaternion
// (xyzw) and three axis lengths by four sweeps of cyclic Jacobi. Evaluation
// here and in the kernel: inverseSqrt as 1 / sqrt, normalize as q / sqrt(|q|^2)
// with |q|^2 fused as dot is, everything else one rounding per operation.
template <class T>
inline T dot4(const T q[4]) {
    return std::fma(q[3], q[3], std::fma(q[2], q[2], std::fma(q[1], q[1], q[0] * q[0])));
}

template <class T>
void ellipsoidAxes(const T cov6[6], T rotation[4], T scale[3]) {
    T a[9] = {cov6[0], cov6[1], cov6[2], cov6[1], cov6[3], cov6[4], cov6[2], cov6[4], cov6[5]};
    T q[4] = {T(0), T(0), T(0), T(1)};
    for (int sweep = 0; sweep < 4; sweep++) {
        for (int p = 0; p < 3; p++) {
            const int r = (p + 1) % 3, other = (p + 2) % 3;
            const T apr = a[r * 3 + p];
            if (apr == T(0)) continue;
            const T app = a[p * 3 + p];
            const T arr = a[r * 3 + r];
            const T theta = (arr - app) / (T(2) * apr);
            const T sign = theta >= T(0) ? T(1) : T(-1);
            const T tangent = sign / (std::fabs(theta) + std::sqrt(theta * theta + T(1)));
            const T cosine = T(1) / std::sqrt(tangent * tangent + T(1));
            const T sine = tangent * cosine;
            const T apo = a[other * 3 + p];
            const T aro = a[other * 3 + r];
            const T turnedP = cosine * apo - sine * aro;
            const T turnedR = sine * apo + cosine * aro;
            a[p * 3 + p] = app - tangent * apr;
            a[r * 3 + r] = arr + tangent * apr;
            a[r * 3 + p] = T(0);
            a[p * 3 + r] = T(0);
            a[other * 3 + p] = turnedP;
            a[p * 3 + other] = turnedP;
            a[other * 3 + r] = turnedR;
            a[r * 3 + other] = turnedR;
            // q * (half along +other, 1): ellipsoidQuaternionProduct with b
            // having one imaginary part; the zero terms are exact.
            const T half = -(sine / (T(1) + cosine));
            T b[4] = {T(0), T(0), T(0), T(1)};
            b[other] = half;
            const T prod[4] = {q[3] * b[0] + q[0] * b[3] + q[1] * b[2] - q[2] * b[1],
                               q[3] * b[1] - q[0] * b[2] + q[1] * b[3] + q[2] * b[0],
                               q[3] * b[2] + q[0] * b[1] - q[1] * b[0] + q[2] * b[3],
                               q[3] * b[3] - q[0] * b[0] - q[1] * b[1] - q[2] * b[2]};
            const T length = std::sqrt(dot4(prod));
            for (int c = 0; c < 4; c++) q[c] = prod[c] / length;
        }
    }
    for (int c = 0; c < 4; c++) rotation[c] = q[c];
    scale[0] = std::sqrt(std::max(a[0], T(0)));
    scale[1] = std::sqrt(std::max(a[4], T(0)));
    scale[2] = std::sqrt(std::max(a[8], T(0)));
}

// Back-to-front draw key: ascending key order is descending depth.
inline uint32_t depthKey(float depth) {
    uint32_t bits;
    std::memcpy(&bits, &depth, 4);
    const uint32_t ordered = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
    return ~ordered;
}

struct Handle {
    int precision;
    void* sim;
};

template <class T> Sim<T>& simOf(vo_sim* s) { return *static_cast<Sim<T>*>(reinterpret_cast<Handle*>(s)->sim); }
template <class T> const Sim<T>& simOf(const vo_sim* s) {
    return *static_cast<const Sim<T>*>(reinterpret_cast<const Handle*>(s)->sim);
}
inline int prec(const vo_sim* s) { return reinterpret_cast<const Handle*>(s)->precision; }

#define DISPATCH_T(s, ...)                   \
    do {                                     \
        if (prec(s) == 32) {                 \
            using T = float;                 \
            __VA_ARGS__;                     \
        } else {                             \
            using T = double;                \
            __VA_ARGS__;                     \
        }                                    \
    } while (0)

template <class T>
void copyOut(const std::vector<V3<T>>& from, float* to) {
    for (size_t n = 0; n < from.size(); n++) {
        to[4 * n] = float(from[n].x);
        to[4 * n + 1] = float(from[n].y);
        to[4 * n + 2] = float(from[n].z);
        to[4 * n + 3] = 0;
    }
}

template <class T>
void copyIn(const float* from, std::vector<V3<T>>& to) {
    for (size_t n = 0; n < to.size(); n++) to[n] = v3(T(from[4 * n]), T(from[4 * n + 1]), T(from[4 * n + 2]));
}

}  // namespace

extern "C" {

int vo_create(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, int precision, vo_sim** out) {
    return vo_create_ex(bodies, n, tank, precision, 0, out);
}

int vo_create_ex(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, int precision, uint32_t flags,
                 vo_sim** out) {
    if (!out || (precision != 32 && precision != 64)) return VSIM_ERR_INVALID;
    const bool isolated = (flags & VSIM_CREATE_ISOLATED) != 0;
    Handle* h = new (std::nothrow) Handle{precision, nullptr};
    if (!h) return VSIM_ERR_NOMEM;
    int rc;
    if (precision == 32) {
        auto* s = new Sim<float>();
        rc = build(*s, bodies, n, tank, isolated);
        h->sim = s;
    } else {
        auto* s = new Sim<double>();
        rc = build(*s, bodies, n, tank, isolated);
        h->sim = s;
    }
    *out = reinterpret_cast<vo_sim*>(h);
    if (rc != VSIM_OK) {
        vo_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

void vo_destroy(vo_sim* s) {
    if (!s) return;
    Handle* h = reinterpret_cast<Handle*>(s);
    if (h->precision == 32)
        delete static_cast<Sim<float>*>(h->sim);
    else
        delete static_cast<Sim<double>*>(h->sim);
    delete h;
}

void vo_set_threads(int threads) {
#ifdef _OPENMP
    omp_set_num_threads(threads < 1 ? 1 : threads);
#else
    (void)threads;
#endif
}

int vo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int vo_set_step_duration(vo_sim* s, double seconds) {
    if (!std::isfinite(seconds) || seconds <= 0) return VSIM_ERR_RANGE;
    DISPATCH_T(s, simOf<T>(s).stepDuration = seconds);
    return VSIM_OK;
}

int vo_set_gravity(vo_sim* s, const double g[3]) {
    DISPATCH_T(s, std::memcpy(simOf<T>(s).gravity, g, sizeof(double) * 3));
    return VSIM_OK;
}

int vo_set_contact(vo_sim* s, int enabled) {
    DISPATCH_T(s, simOf<T>(s).contact = enabled != 0);
    return VSIM_OK;
}

int vo_set_self_contact(vo_sim* s, int enabled) {
    DISPATCH_T(s, simOf<T>(s).selfContact = enabled != 0);
    return VSIM_OK;
}

int vo_set_iterations(vo_sim* s, uint32_t iterations) {
    if (iterations < 1) return VSIM_ERR_RANGE;
    DISPATCH_T(s, simOf<T>(s).iterations = iterations);
    return VSIM_OK;
}

// simulator.js:332-353 with VoxelLattice.setDensity (voxelLattice.js:188-195).
int vo_set_material(vo_sim* s, uint32_t body, const vsim_material* m, uint32_t fields) {
    DISPATCH_T(s, {
        Sim<T>& sim = simOf<T>(s);
        if (body >= sim.bodies.size()) return VSIM_ERR_RANGE;
        vsim_material& mat = sim.bodies[body].material;
        if (fields & VSIM_MAT_MAX_STRETCH) {
            if (!std::isfinite(m->max_stretch) || (m->max_stretch != 0 && m->max_stretch <= 1)) return VSIM_ERR_RANGE;
            mat.max_stretch = m->max_stretch;
        }
        if (fields & VSIM_MAT_YOUNGS) mat.youngs_modulus = m->youngs_modulus;
        if (fields & VSIM_MAT_POISSON) mat.poisson_ratio = m->poisson_ratio;
        if (fields & VSIM_MAT_FRICTION) mat.friction = m->friction;
        if (fields & VSIM_MAT_DAMPING) mat.damping = m->damping;
        if (fields & VSIM_MAT_RELAXATION) mat.relaxation = m->relaxation;
        if ((fields & VSIM_MAT_DENSITY) && m->density > 0 && m->density != mat.density) {
            const double ratio = mat.density / m->density;
            const Body& b = sim.bodies[body];
            for (uint32_t n = 0; n < b.nodeCount; n++)
                sim.invMass[b.nodeOffset + n] = asT<T>(double(sim.invMass[b.nodeOffset + n]) * ratio);
            mat.density = m->density;
            uploadGpuMasses(sim);
        }
        uploadParams(sim, body);
    });
    return VSIM_OK;
}

// kinematicDrive.js:155-191.
int vo_hold(vo_sim* s, const uint32_t* nodes, const float* offsets, uint32_t count) {
    DISPATCH_T(s, {
        Sim<T>& sim = simOf<T>(s);
        for (uint32_t i = 0; i < count; i++) {
            if (nodes[i] >= sim.nodeCount) return VSIM_ERR_RANGE;
            if (sim.isStatic[nodes[i]]) return VSIM_ERR_INVALID;
        }
        sim.driven.clear();
        sim.drivenOffset.clear();
        const uint32_t kept = std::min<uint32_t>(count, VSIM_MAX_DRIVEN);
        for (uint32_t i = 0; i < kept; i++) {
            sim.driven.push_back(nodes[i]);
            sim.drivenOffset.push_back(v3(T(offsets[3 * i]), T(offsets[3 * i + 1]), T(offsets[3 * i + 2])));
        }
        uploadGpuMasses(sim);
    });
    return VSIM_OK;
}

int vo_release(vo_sim* s) {
    DISPATCH_T(s, {
        Sim<T>& sim = simOf<T>(s);
        sim.driven.clear();
        sim.drivenOffset.clear();
        uploadGpuMasses(sim);
    });
    return VSIM_OK;
}

int vo_set_drive_law(vo_sim* s, int law) {
    if (law != VSIM_DRIVE_HARD && law != VSIM_DRIVE_COMPLIANT) return VSIM_ERR_INVALID;
    DISPATCH_T(s, {
        simOf<T>(s).law = law;
        uploadGpuMasses(simOf<T>(s));
    });
    return VSIM_OK;
}

int vo_set_drive_response_time(vo_sim* s, double seconds) {
    if (!std::isfinite(seconds) || seconds <= 0) return VSIM_ERR_RANGE;
    DISPATCH_T(s, simOf<T>(s).responseTime = asT<T>(seconds));
    return VSIM_OK;
}

int vo_set_grab(vo_sim* s, const double target[3], const double velocity[3]) {
    DISPATCH_T(s, {
        simOf<T>(s).grabTarget = v3(asT<T>(target[0]), asT<T>(target[1]), asT<T>(target[2]));
        simOf<T>(s).grabVelocity = v3(asT<T>(velocity[0]), asT<T>(velocity[1]), asT<T>(velocity[2]));
    });
    return VSIM_OK;
}

int vo_dispatch(vo_sim* s, uint32_t steps) {
    DISPATCH_T(s, dispatch(simOf<T>(s), steps));
    return VSIM_OK;
}

uint32_t vo_node_count(const vo_sim* s) {
    DISPATCH_T(s, return simOf<T>(s).nodeCount);
}

uint32_t vo_cell_count(const vo_sim* s) {
    DISPATCH_T(s, {
        size_t total = 0;
        for (int c = 0; c < 8; c++) total += simOf<T>(s).cellLinear[c].size();
        return uint32_t(total);
    });
}

uint32_t vo_surface_count(const vo_sim* s) {
    DISPATCH_T(s, return uint32_t(simOf<T>(s).sNode.size()));
}

uint32_t vo_body_node_offset(const vo_sim* s, uint32_t body) {
    DISPATCH_T(s, return body < simOf<T>(s).bodies.size() ? simOf<T>(s).bodies[body].nodeOffset : 0u);
}

int vo_get_state(const vo_sim* s, float* pos, float* prev, float* vel) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        if (pos) copyOut(sim.pos, pos);
        if (prev) copyOut(sim.prev, prev);
        if (vel) copyOut(sim.vel, vel);
    });
    return VSIM_OK;
}

int vo_get_state_f64(const vo_sim* s, double* pos, double* prev, double* vel) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        const std::vector<V3<T>>* from[3] = {&sim.pos, &sim.prev, &sim.vel};
        double* to[3] = {pos, prev, vel};
        for (int a = 0; a < 3; a++) {
            if (!to[a]) continue;
            for (size_t n = 0; n < from[a]->size(); n++) {
                to[a][4 * n] = double((*from[a])[n].x);
                to[a][4 * n + 1] = double((*from[a])[n].y);
                to[a][4 * n + 2] = double((*from[a])[n].z);
                to[a][4 * n + 3] = 0;
            }
        }
    });
    return VSIM_OK;
}

int vo_set_state(vo_sim* s, const float* pos, const float* prev, const float* vel) {
    DISPATCH_T(s, {
        Sim<T>& sim = simOf<T>(s);
        if (pos) copyIn(pos, sim.pos);
        if (prev) copyIn(prev, sim.prev);
        if (vel) copyIn(vel, sim.vel);
    });
    return VSIM_OK;
}

int vo_inv_mass(const vo_sim* s, float* out) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        for (uint32_t n = 0; n < sim.nodeCount; n++) out[n] = float(sim.invMass[n]);
    });
    return VSIM_OK;
}

int vo_cells(const vo_sim* s, uint32_t b, uint32_t* cells, uint32_t color_counts[8]) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        if (b >= sim.bodies.size()) return VSIM_ERR_RANGE;
        size_t at = 0;
        for (int c = 0; c < 8; c++) {
            const auto& list = sim.bodies[b].cellsByColor[c];
            color_counts[c] = uint32_t(list.size());
            if (cells) std::copy(list.begin(), list.end(), cells + at);
            at += list.size();
        }
    });
    return VSIM_OK;
}

int vo_surface(const vo_sim* s, uint32_t* nodes, uint32_t* bodies) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        if (nodes) std::copy(sim.sNode.begin(), sim.sNode.end(), nodes);
        if (bodies) std::copy(sim.sBody.begin(), sim.sBody.end(), bodies);
    });
    return VSIM_OK;
}

size_t vo_contact_pairs(const vo_sim* s, uint32_t* pairs, size_t capacity) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        const Binned<T> g = binAll(sim);
        size_t total = 0;
        for (uint32_t r = 0; r < sim.sNode.size(); r++) {
            V3<T> sum;
            T hits;
            gather(sim, g, r, sum, hits, [&](uint32_t other) {
                if (total < capacity) {
                    pairs[2 * total] = r;
                    pairs[2 * total + 1] = other;
                }
                total++;
            });
        }
        return total;
    });
}

int vo_contact_grid(const vo_sim* s, double origin[3], double* bucket, uint32_t dims[3]) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        for (int a = 0; a < 3; a++) {
            origin[a] = sim.grids[0].origin[a];
            dims[a] = sim.grids[0].dims[a];
        }
        *bucket = sim.grids[0].bucket;
    });
    return VSIM_OK;
}

int vo_splat_deform(const vo_sim* s, uint32_t b, const float* means, const float* quats, const float* scales,
                    uint32_t n, const float view_dir[3], float* out_means, float* out_cov6, uint32_t* keys) {
    DISPATCH_T(s, {
        const Sim<T>& sim = simOf<T>(s);
        if (b >= sim.bodies.size()) return VSIM_ERR_RANGE;
        const Body& body = sim.bodies[b];
        const T origin[3] = {asT<T>(body.origin[0]), asT<T>(body.origin[1]), asT<T>(body.origin[2])};
        const T h = asT<T>(body.h);
        const V3<T>* nodes = sim.pos.data() + body.nodeOffset;
        for (uint32_t i = 0; i < n; i++) {
            V3<T> position;
            M3<T> F;
            deformationAt(nodes, body.nodeDims, body.cellDims, origin, h,
                          v3(T(means[3 * i]), T(means[3 * i + 1]), T(means[3 * i + 2])), position, F);
            const T q[4] = {T(quats[4 * i]), T(quats[4 * i + 1]), T(quats[4 * i + 2]), T(quats[4 * i + 3])};
            const T sc[3] = {T(scales[3 * i]), T(scales[3 * i + 1]), T(scales[3 * i + 2])};
            T cov[6];
            deformedCovariance(F, q, sc, cov);
            if (out_means) {
                out_means[3 * i] = float(position.x);
                out_means[3 * i + 1] = float(position.y);
                out_means[3 * i + 2] = float(position.z);
            }
            if (out_cov6)
                for (int k = 0; k < 6; k++) out_cov6[6 * i + k] = float(cov[k]);
            if (keys) {
                const float px = float(position.x), py = float(position.y), pz = float(position.z);
                const float depth = px * view_dir[0] + py * view_dir[1] + pz * view_dir[2];
                keys[i] = depthKey(depth);
            }
        }
    });
    return VSIM_OK;
}

void vo_stable_sort_u32(const uint32_t* keys, uint32_t n, uint32_t key_bits, uint32_t* order) {
    const uint32_t mask = key_bits >= 32 ? 0xffffffffu : ((1u << key_bits) - 1u);
    std::iota(order, order + n, 0u);
    std::stable_sort(order, order + n, [&](uint32_t a, uint32_t b) { return (keys[a] & mask) < (keys[b] & mask); });
}

// ---- known-answer helpers --------------------------------------------

void vo_kuhn_tets(uint32_t out[24]) {
    for (int t = 0; t < 6; t++)
        for (int i = 0; i < 4; i++) out[4 * t + i] = KUHN_TETS[t][i];
}

void vo_kuhn_rest_shapes(double h, double out[54]) {
    for (int t = 0; t < 6; t++) {
        double m[9];
        kuhnRestShape(t, h, m);
        for (int i = 0; i < 9; i++) out[9 * t + i] = double(float(m[i]));
    }
}

void vo_kuhn_rest_inverses(double h, double out[54]) {
    for (int t = 0; t < 6; t++) {
        double m[9], f[9], inv[9];
        kuhnRestShape(t, h, m);
        for (int i = 0; i < 9; i++) f[i] = double(float(m[i]));  // mat3FromColumns stores f32
        inverse9(f, inv);
        for (int i = 0; i < 9; i++) out[9 * t + i] = double(float(inv[i]));
    }
}

static M3<double> m3FromFlat(const double* m) {
    return M3<double>{{v3(m[0], m[1], m[2]), v3(m[3], m[4], m[5]), v3(m[6], m[7], m[8])}};
}

void vo_project_tet_f64(const double* p, const double* prev, const double* w, const double* B, double alpha_dev,
                        double alpha_hyd, double gamma, double relax, double* out) {
    V3<double> q[4], pv[4];
    for (int i = 0; i < 4; i++) {
        q[i] = v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        pv[i] = v3(prev[3 * i], prev[3 * i + 1], prev[3 * i + 2]);
    }
    const uint32_t tet[4] = {0, 1, 2, 3};
    projectTet(q, pv, w, tet, m3FromFlat(B), 1.0, alpha_dev, alpha_hyd, gamma, relax);
    for (int i = 0; i < 4; i++) {
        out[3 * i] = q[i].x;
        out[3 * i + 1] = q[i].y;
        out[3 * i + 2] = q[i].z;
    }
}

void vo_run_free_tet_f64(double* p, const double* w, const double* B, double alpha_dev, double alpha_hyd,
                         double gamma, double relax, double dt, uint32_t substeps) {
    V3<double> q[4], v[4];
    for (int i = 0; i < 4; i++) {
        q[i] = v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        v[i] = v3(0.0, 0.0, 0.0);
    }
    const uint32_t tet[4] = {0, 1, 2, 3};
    const M3<double> Bm = m3FromFlat(B);
    for (uint32_t step = 0; step < substeps; step++) {
        V3<double> prev[4];
        for (int i = 0; i < 4; i++) {
            prev[i] = q[i];
            q[i] = q[i] + v[i] * (dt * (w[i] > 0 ? 1.0 : 0.0));
        }
        projectTet(q, prev, w, tet, Bm, 1.0, alpha_dev, alpha_hyd, gamma, relax);
        for (int i = 0; i < 4; i++) v[i] = (q[i] - prev[i]) * (1 / dt);
    }
    for (int i = 0; i < 4; i++) {
        p[3 * i] = q[i].x;
        p[3 * i + 1] = q[i].y;
        p[3 * i + 2] = q[i].z;
    }
}

void vo_tet_constraints_f64(const double* p, const double* B, double gamma, double* c_dev, double* c_hyd,
                            double* g_dev, double* g_hyd) {
    V3<double> q[4];
    for (int i = 0; i < 4; i++) q[i] = v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    const M3<double> Bm = m3FromFlat(B);
    const M3<double> Bt = transpose(Bm);
    const M3<double> F = mul(M3<double>{{q[1] - q[0], q[2] - q[0], q[3] - q[0]}}, Bm);
    const double cDev = std::sqrt(dot(F.c[0], F.c[0]) + dot(F.c[1], F.c[1]) + dot(F.c[2], F.c[2]));
    *c_dev = cDev;
    *c_hyd = determinant(F) - gamma;
    const double inv = cDev > 1e-9 ? 1 / cDev : 0;
    const M3<double> mDev = mul(F * inv, Bt);
    const M3<double> mHyd = mul(M3<double>{{cross(F.c[1], F.c[2]), cross(F.c[2], F.c[0]), cross(F.c[0], F.c[1])}}, Bt);
    const V3<double> d0 = -(mDev.c[0] + mDev.c[1] + mDev.c[2]);
    const V3<double> h0 = -(mHyd.c[0] + mHyd.c[1] + mHyd.c[2]);
    const V3<double> gd[4] = {d0, mDev.c[0], mDev.c[1], mDev.c[2]};
    const V3<double> gh[4] = {h0, mHyd.c[0], mHyd.c[1], mHyd.c[2]};
    for (int i = 0; i < 4; i++) {
        g_dev[3 * i] = gd[i].x;
        g_dev[3 * i + 1] = gd[i].y;
        g_dev[3 * i + 2] = gd[i].z;
        g_hyd[3 * i] = gh[i].x;
        g_hyd[3 * i + 1] = gh[i].y;
        g_hyd[3 * i + 2] = gh[i].z;
    }
}

int vo_resolve_pair_f64(const double* me, const double* mate, uint32_t me_index, uint32_t mate_index, double out[3]) {
    const V3<double> pi = v3(me[0], me[1], me[2]), previ = v3(me[3], me[4], me[5]);
    const V3<double> pj = v3(mate[0], mate[1], mate[2]), prevj = v3(mate[3], mate[4], mate[5]);
    const double wi = me[6], wj = mate[6];
    const V3<double> d = pi - pj;
    const double dist2 = dot(d, d);
    const double reach = me[7] + mate[7];
    out[0] = out[1] = out[2] = 0;
    if (dist2 >= reach * reach) return 0;
    const double total = wi + wj;
    if (total <= 0) return 0;
    const double share = wi / total;
    const double dist = std::sqrt(dist2);
    V3<double> normal = v3(0.0, me_index < mate_index ? 1.0 : -1.0, 0.0);
    if (dist > 1e-9) normal = d / dist;
    const double depth = reach - dist;
    V3<double> correction = normal * (depth * share);
    const V3<double> sliding = (pi - previ) - (pj - prevj);
    const V3<double> tangent = sliding - normal * dot(sliding, normal);
    const double slid = length(tangent);
    if (slid > 1e-9) {
        const double mu = std::min(me[8], mate[8]);
        correction = correction - tangent * (share * std::min(1.0, mu * depth / slid));
    }
    out[0] = correction.x;
    out[1] = correction.y;
    out[2] = correction.z;
    return 1;
}

void vo_drive_hard_f64(const double here[3], const double goal[3], const double velocity[3], double dt,
                       double position[3], double out_velocity[3]) {
    const V3<double> h = v3(here[0], here[1], here[2]);
    const V3<double> step = v3(velocity[0], velocity[1], velocity[2]) * dt;
    const V3<double> toGoal = v3(goal[0], goal[1], goal[2]) - h;
    const V3<double> next = h + (dot(step, step) >= dot(toGoal, toGoal) ? toGoal : step);
    const V3<double> v = (next - h) / dt;
    position[0] = next.x;
    position[1] = next.y;
    position[2] = next.z;
    out_velocity[0] = v.x;
    out_velocity[1] = v.y;
    out_velocity[2] = v.z;
}

void vo_drive_compliant_f64(const double p[3], const double goal[3], double dt, double response_time, double out[3]) {
    const double dt2 = dt * dt;
    const double tau2 = response_time * response_time;
    const double frac = dt2 / (dt2 + tau2);
    for (int a = 0; a < 3; a++) out[a] = p[a] + (goal[a] - p[a]) * frac;
}

void vo_stretch_pair_f64(double a[3], double b[3], double wa, double wb, double maximum) {
    const V3<double> pa = v3(a[0], a[1], a[2]), pb = v3(b[0], b[1], b[2]);
    const V3<double> delta = pb - pa;
    const double len = length(delta);
    const double weight = wa + wb;
    if (len > maximum && weight > 0) {
        const V3<double> correction = delta * ((len - maximum) / (len * weight));
        const V3<double> na = pa + wa * correction, nb = pb - wb * correction;
        a[0] = na.x, a[1] = na.y, a[2] = na.z;
        b[0] = nb.x, b[1] = nb.y, b[2] = nb.z;
    }
}

void vo_resolve_plane_f64(const double p[3], const double prev[3], const double normal[3], double depth,
                          double friction, double out[3]) {
    const V3<double> q = resolvePlane(v3(p[0], p[1], p[2]), v3(prev[0], prev[1], prev[2]),
                                      v3(normal[0], normal[1], normal[2]), depth, friction);
    out[0] = q.x;
    out[1] = q.y;
    out[2] = q.z;
}

void vo_deformation_at_f64(const double* node_pos, const uint32_t node_dims[3], const uint32_t cell_dims[3],
                           const double origin[3], double h, const double rest[3], double position[3],
                           double gradient[9]) {
    const size_t count = size_t(node_dims[0]) * node_dims[1] * node_dims[2];
    std::vector<V3<double>> nodes(count);
    for (size_t n = 0; n < count; n++) nodes[n] = v3(node_pos[3 * n], node_pos[3 * n + 1], node_pos[3 * n + 2]);
    V3<double> pos;
    M3<double> F;
    deformationAt(nodes.data(), node_dims, cell_dims, origin, h, v3(rest[0], rest[1], rest[2]), pos, F);
    position[0] = pos.x;
    position[1] = pos.y;
    position[2] = pos.z;
    for (int c = 0; c < 3; c++) {
        gradient[3 * c] = F.c[c].x;
        gradient[3 * c + 1] = F.c[c].y;
        gradient[3 * c + 2] = F.c[c].z;
    }
}

void vo_deformed_covariance_f64(const double gradient[9], const double quat[4], const double scale[3], double out[9]) {
    double c6[6];
    deformedCovariance(m3FromFlat(gradient), quat, scale, c6);
    out[0] = c6[0], out[1] = c6[1], out[2] = c6[2];
    out[3] = c6[1], out[4] = c6[3], out[5] = c6[4];
    out[6] = c6[2], out[7] = c6[4], out[8] = c6[5];
}

void vo_ellipsoid_axes_f64(const double cov6[6], double rotation[4], double scale[3]) {
    ellipsoidAxes(cov6, rotation, scale);
}

void vo_ellipsoid_axes_f32(const float* cov6, uint32_t n, float* rotation, float* scale) {
    for (uint32_t i = 0; i < n; i++) ellipsoidAxes(cov6 + 6 * size_t(i), rotation + 4 * size_t(i), scale + 3 * size_t(i));
}

void vo_stretch_edges(double out[84]) {
    const std::vector<Edge> edges = stretchEdges();
    for (int e = 0; e < 28; e++) {
        out[3 * e] = edges[e].a;
        out[3 * e + 1] = edges[e].b;
        out[3 * e + 2] = edges[e].len;
    }
}

void vo_broadphase_grid(const double mn[3], const double mx[3], double bucket_size, double origin[3], double* edge,
                        uint32_t dims[3]) {
    gridLayout(mn, mx, bucket_size, origin, *edge, dims);
}

// broadphase.js:570-577.
uint32_t vo_bucket_of(const double origin[3], double bucket, const uint32_t dims[3], const double point[3]) {
    uint32_t index = 0;
    for (int axis = 2; axis >= 0; axis--) {
        const double raw = std::floor((point[axis] - origin[axis]) / bucket);
        index = index * dims[axis] + uint32_t(std::min(double(dims[axis] - 1), std::max(0.0, raw)));
    }
    return index;
}

uint32_t vo_surface_nodes(const uint32_t cell_dims[3], const uint8_t* occupancy, uint32_t* out) {
    std::vector<uint32_t> found;
    surfaceNodesOf(cell_dims, occupancy, found);
    if (out) std::copy(found.begin(), found.end(), out);
    return uint32_t(found.size());
}

}  // extern "C"
