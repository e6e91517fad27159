// The per-item device code of a substep -- a node's prediction and closing
// pass, a cell's projection, a surface record's binning, ordering and
// contact gather -- shared by the per-pass kernels (step_kernels.cu) and the
// session kernel (session.cu), so both run the same arithmetic.
//
// Pointers here carry no __restrict__: the session kernel reads and writes
// the same arrays across its phases, so none of them may be read through
// the non-coherent path. The per-pass kernels' own __restrict__ parameters
// still tell the compiler what it may assume inside each launch.
#pragma once

#include "kernels.cuh"

namespace vsim {

// ------------------------------------------------------- Kuhn constants --

// kuhn.js:28-35: corner indices of the six tetrahedra.
__host__ __device__ constexpr int kTet(int t, int i) {
    constexpr int tets[6][4] = {{0, 1, 3, 7}, {0, 5, 1, 7}, {0, 3, 2, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 6, 4, 7}};
    return tets[t][i];
}

// The inverse rest shape of tetrahedron t of the unit cube, entry (row r,
// column c) of the column-major matrix (kuhn.js:59-80). The rest shapes are
// unimodular, so the inverse is the integer adjugate divided by det = +-1.
struct KuhnInv {
    int v[6][3][3];  // [t][column][row]
};

__host__ __device__ constexpr KuhnInv makeKuhnInv() {
    KuhnInv out{};
    for (int t = 0; t < 6; t++) {
        int m[9] = {};  // column-major Dm
        for (int col = 0; col < 3; col++)
            for (int row = 0; row < 3; row++)
                m[col * 3 + row] = ((kTet(t, col + 1) >> row) & 1) - ((kTet(t, 0) >> row) & 1);
        const int det = m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
                        m[6] * (m[1] * m[5] - m[4] * m[2]);
        const int adj[9] = {m[4] * m[8] - m[7] * m[5], m[7] * m[2] - m[1] * m[8], m[1] * m[5] - m[4] * m[2],
                            m[6] * m[5] - m[3] * m[8], m[0] * m[8] - m[6] * m[2], m[3] * m[2] - m[0] * m[5],
                            m[3] * m[7] - m[6] * m[4], m[6] * m[1] - m[0] * m[7], m[0] * m[4] - m[3] * m[1]};
        for (int col = 0; col < 3; col++)
            for (int row = 0; row < 3; row++) out.v[t][col][row] = adj[col * 3 + row] / det;
    }
    return out;
}

constexpr KuhnInv kKuhn = makeKuhnInv();

// a0 k0 s + a1 k1 s + a2 k2 s for constant k in {-1, 0, 1}, summed left to
// right as M * v is (the first product rounded, the next ones fused in),
// with the zero terms left out. A product with an exact zero is a signed
// zero, and fusing it in changes nothing but the sign of an exact-zero sum,
// so this is the full product's value with a third of the arithmetic.
template <int K>
__device__ __forceinline__ float kscale(float s, float ns) {
    return K > 0 ? s : ns;
}

template <int K0, int K1, int K2>
__device__ __forceinline__ V sparse3(V a0, V a1, V a2, float s, float ns) {
    if constexpr (K0 != 0) {
        V acc = a0 * kscale<K0>(s, ns);
        if constexpr (K1 != 0) acc = fma3(a1, kscale<K1>(s, ns), acc);
        if constexpr (K2 != 0) acc = fma3(a2, kscale<K2>(s, ns), acc);
        return acc;
    } else if constexpr (K1 != 0) {
        V acc = a1 * kscale<K1>(s, ns);
        if constexpr (K2 != 0) acc = fma3(a2, kscale<K2>(s, ns), acc);
        return acc;
    } else {
        return a2 * kscale<K2>(s, ns);
    }
}

// A * B with B = K_t s: column j is sum_k A.c[k] B[j][k].
template <int t>
__device__ __forceinline__ M timesB(const M& A, float s, float ns) {
    return M{{sparse3<kKuhn.v[t][0][0], kKuhn.v[t][0][1], kKuhn.v[t][0][2]>(A.c[0], A.c[1], A.c[2], s, ns),
              sparse3<kKuhn.v[t][1][0], kKuhn.v[t][1][1], kKuhn.v[t][1][2]>(A.c[0], A.c[1], A.c[2], s, ns),
              sparse3<kKuhn.v[t][2][0], kKuhn.v[t][2][1], kKuhn.v[t][2][2]>(A.c[0], A.c[1], A.c[2], s, ns)}};
}

// A * transpose(B): column j is sum_k A.c[k] B[k][j].
template <int t>
__device__ __forceinline__ M timesBt(const M& A, float s, float ns) {
    return M{{sparse3<kKuhn.v[t][0][0], kKuhn.v[t][1][0], kKuhn.v[t][2][0]>(A.c[0], A.c[1], A.c[2], s, ns),
              sparse3<kKuhn.v[t][0][1], kKuhn.v[t][1][1], kKuhn.v[t][2][1]>(A.c[0], A.c[1], A.c[2], s, ns),
              sparse3<kKuhn.v[t][0][2], kKuhn.v[t][1][2], kKuhn.v[t][2][2]>(A.c[0], A.c[1], A.c[2], s, ns)}};
}

// xpbdCouple.wgsl:58-71.
__device__ __forceinline__ void couple(float cx, float cy, float ax, float ay, float relax, float rx, float ry, float gx,
                                       float gy, float gz, float& lx, float& ly) {
    const float stiffened = 1.0f + relax;
    const float a00 = fmaf(gx, stiffened, ax);
    const float a01 = gy * stiffened;
    const float a11 = fmaf(gz, stiffened, ay);
    const float det = fmaf(a00, a11, -(a01 * a01));
    if (det < 1e-20f) {
        lx = 0.0f;
        ly = 0.0f;
        return;
    }
    const float bx = -fmaf(rx, relax, cx);
    const float by = -fmaf(ry, relax, cy);
    lx = fmaf(a11, bx, -(a01 * by)) / det;
    ly = fmaf(a00, by, -(a01 * bx)) / det;
}

// sum_i w_i e_i over a tetrahedron's four nodes, fused.
__device__ __forceinline__ float weighted4(float w0, float w1, float w2, float w3, float e0, float e1, float e2,
                                           float e3) {
    return fmaf(w3, e3, fmaf(w2, e2, fmaf(w1, e1, w0 * e0)));
}

// p + (d lx + h ly) w, fused.
__device__ __forceinline__ V moved(V p, V d, V h, float lx, float ly, float w) {
    return fma3(fma3(h, ly, d * lx), w, p);
}

// project.wgsl:75-153, tetrahedron t of the cell held in registers.
template <int t>
__device__ __forceinline__ void projectTet(V (&p)[8], const V (&prev)[8], const float (&w)[8], float s, float ns,
                                           float alphaDev, float alphaHyd, float gamma, float relax) {
    constexpr int i0 = kTet(t, 0), i1 = kTet(t, 1), i2 = kTet(t, 2), i3 = kTet(t, 3);
    const float w0 = w[i0], w1 = w[i1], w2 = w[i2], w3 = w[i3];
    if (w0 + w1 + w2 + w3 == 0.0f) return;
    const V base = p[i0];
    const M F = timesB<t>(M{{p[i1] - base, p[i2] - base, p[i3] - base}}, s, ns);
    const float cDev = sqrtf(dot(F.c[0], F.c[0]) + dot(F.c[1], F.c[1]) + dot(F.c[2], F.c[2]));
    const float cHyd = determinant(F) - gamma;
    const float inv = cDev > 1e-9f ? 1.0f / cDev : 0.0f;
    const M mDev = timesBt<t>(F * inv, s, ns);
    const M mHyd = timesBt<t>(M{{cross(F.c[1], F.c[2]), cross(F.c[2], F.c[0]), cross(F.c[0], F.c[1])}}, s, ns);
    const V d1 = mDev.c[0], d2 = mDev.c[1], d3 = mDev.c[2];
    const V d0 = -(d1 + d2 + d3);
    const V h1 = mHyd.c[0], h2 = mHyd.c[1], h3 = mHyd.c[2];
    const V h0 = -(h1 + h2 + h3);
    const float gx = weighted4(w0, w1, w2, w3, dot(d0, d0), dot(d1, d1), dot(d2, d2), dot(d3, d3));
    const float gy = weighted4(w0, w1, w2, w3, dot(d0, h0), dot(d1, h1), dot(d2, h2), dot(d3, h3));
    const float gz = weighted4(w0, w1, w2, w3, dot(h0, h0), dot(h1, h1), dot(h2, h2), dot(h3, h3));
    const V x0 = p[i0] - prev[i0];
    const V x1 = p[i1] - prev[i1];
    const V x2 = p[i2] - prev[i2];
    const V x3 = p[i3] - prev[i3];
    const float rx = dot(d0, x0) + dot(d1, x1) + dot(d2, x2) + dot(d3, x3);
    const float ry = dot(h0, x0) + dot(h1, x1) + dot(h2, x2) + dot(h3, x3);
    float lx, ly;
    couple(cDev, cHyd, alphaDev, alphaHyd, relax, rx, ry, gx, gy, gz, lx, ly);
    p[i0] = moved(p[i0], d0, h0, lx, ly, w0);
    p[i1] = moved(p[i1], d1, h1, lx, ly, w1);
    p[i2] = moved(p[i2], d2, h2, lx, ly, w2);
    p[i3] = moved(p[i3], d3, h3, lx, ly, w3);
}

// The constants of a cell's body that project.wgsl:64-73 derives.
struct CellConsts {
    float alphaDev, alphaHyd, gamma, relax, restScale, h, maxStretch;
};

__device__ __forceinline__ CellConsts cellConsts(const DevBody* b) {
    return CellConsts{b->alphaDev, b->alphaHyd, b->gamma, b->relax, b->restScale, b->h, b->maxStretch};
}

// project.wgsl:35-184 on one cell held in registers: the six tetrahedra in
// Kuhn order (unless LIMIT_ONLY), then, with maxStretch > 1, two sweeps of
// the unilateral length limit over all 28 corner pairs (project.wgsl:162-179).
template <bool LIMIT_ONLY>
__device__ __forceinline__ void solveCell(V (&p)[8], const V (&prev)[8], const float (&w)[8], const CellConsts& k,
                                          const StretchLengths& lens) {
    if (!LIMIT_ONLY) {
        const float s = k.restScale, ns = -s;
        projectTet<0>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
        projectTet<1>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
        projectTet<2>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
        projectTet<3>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
        projectTet<4>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
        projectTet<5>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax);
    }
    if (k.maxStretch > 1.0f) {
        for (int sweep = 0; sweep < 2; sweep++) {
#pragma unroll
            for (int a = 0; a < 8; a++) {
#pragma unroll
                for (int bb = a + 1; bb < 8; bb++) {
                    const V delta = p[bb] - p[a];
                    const float len = length(delta);
                    const float maximum = lens.len[__popc(a ^ bb) - 1] * k.h * k.maxStretch;
                    const float weight = w[a] + w[bb];
                    if (len > maximum && weight > 0.0f) {
                        const V correction = delta * ((len - maximum) / (len * weight));
                        p[a] = p[a] + w[a] * correction;
                        p[bb] = p[bb] - w[bb] * correction;
                    }
                }
            }
        }
    }
}

// projectTet with the cell split over the four lanes of a quad (lanes
// 4k..4k+3 of a warp, `quad` their shuffle mask, q the lane's place): every
// lane holds the cell and runs the tetrahedron's spine -- F, its norm, the
// determinant, the gradient columns, the 2x2 solve -- as projectTet does;
// lane q takes corner q's dot products and update, and the products reach
// every lane for the reference's left-to-right chains. Same values, same
// order: the result equals projectTet's bit for bit.
template <int t>
__device__ __forceinline__ void projectTetQuad(V (&p)[8], const V (&prev)[8], const float (&w)[8], float s, float ns,
                                               float alphaDev, float alphaHyd, float gamma, float relax,
                                               uint32_t q, uint32_t quad) {
    constexpr int i0 = kTet(t, 0), i1 = kTet(t, 1), i2 = kTet(t, 2), i3 = kTet(t, 3);
    const float w0 = w[i0], w1 = w[i1], w2 = w[i2], w3 = w[i3];
    if (w0 + w1 + w2 + w3 == 0.0f) return;
    const V base = p[i0];
    const M F = timesB<t>(M{{p[i1] - base, p[i2] - base, p[i3] - base}}, s, ns);
    const float cDev = sqrtf(dot(F.c[0], F.c[0]) + dot(F.c[1], F.c[1]) + dot(F.c[2], F.c[2]));
    const float cHyd = determinant(F) - gamma;
    const float inv = cDev > 1e-9f ? 1.0f / cDev : 0.0f;
    const M mDev = timesBt<t>(F * inv, s, ns);
    const M mHyd = timesBt<t>(M{{cross(F.c[1], F.c[2]), cross(F.c[2], F.c[0]), cross(F.c[0], F.c[1])}}, s, ns);
    const V d1 = mDev.c[0], d2 = mDev.c[1], d3 = mDev.c[2];
    const V d0 = -(d1 + d2 + d3);
    const V h1 = mHyd.c[0], h2 = mHyd.c[1], h3 = mHyd.c[2];
    const V h0 = -(h1 + h2 + h3);
    auto pick = [&](V a0, V a1, V a2, V a3) { return q == 0 ? a0 : q == 1 ? a1 : q == 2 ? a2 : a3; };
    const V d = pick(d0, d1, d2, d3), h = pick(h0, h1, h2, h3);
    const V x = pick(p[i0], p[i1], p[i2], p[i3]) - pick(prev[i0], prev[i1], prev[i2], prev[i3]);
    const float mine[5] = {dot(d, d), dot(d, h), dot(h, h), dot(d, x), dot(h, x)};
    float e[5][4];
#pragma unroll
    for (int k = 0; k < 5; k++)
#pragma unroll
        for (int l = 0; l < 4; l++) e[k][l] = __shfl_sync(quad, mine[k], l, 4);
    const float gx = weighted4(w0, w1, w2, w3, e[0][0], e[0][1], e[0][2], e[0][3]);
    const float gy = weighted4(w0, w1, w2, w3, e[1][0], e[1][1], e[1][2], e[1][3]);
    const float gz = weighted4(w0, w1, w2, w3, e[2][0], e[2][1], e[2][2], e[2][3]);
    const float rx = e[3][0] + e[3][1] + e[3][2] + e[3][3];
    const float ry = e[4][0] + e[4][1] + e[4][2] + e[4][3];
    float lx, ly;
    couple(cDev, cHyd, alphaDev, alphaHyd, relax, rx, ry, gx, gy, gz, lx, ly);
    const float wq = q == 0 ? w0 : q == 1 ? w1 : q == 2 ? w2 : w3;
    const V moved_ = moved(pick(p[i0], p[i1], p[i2], p[i3]), d, h, lx, ly, wq);
    auto from = [&](int l) {
        return mk(__shfl_sync(quad, moved_.x, l, 4), __shfl_sync(quad, moved_.y, l, 4),
                  __shfl_sync(quad, moved_.z, l, 4));
    };
    p[i0] = from(0);
    p[i1] = from(1);
    p[i2] = from(2);
    p[i3] = from(3);
}

// solveCell<false> with the six tetrahedra split over a quad's lanes; the
// stretch sweeps that follow run in every lane on the same values.
__device__ __forceinline__ void solveCellQuad(V (&p)[8], const V (&prev)[8], const float (&w)[8],
                                              const CellConsts& k, const StretchLengths& lens, uint32_t q,
                                              uint32_t quad) {
    const float s = k.restScale, ns = -s;
    projectTetQuad<0>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    projectTetQuad<1>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    projectTetQuad<2>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    projectTetQuad<3>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    projectTetQuad<4>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    projectTetQuad<5>(p, prev, w, s, ns, k.alphaDev, k.alphaHyd, k.gamma, k.relax, q, quad);
    solveCell<true>(p, prev, w, k, lens);  // the stretch sweeps only
}

// The eight corner nodes of a cell entry (corner-0 node, body, y stride, z
// stride), in corners.js order.
__device__ __forceinline__ void cornerNodes(uint4 e, uint32_t (&ids)[8]) {
    const uint32_t nx = e.z, nxy = e.w, n0 = e.x;
    ids[0] = n0;
    ids[1] = n0 + 1;
    ids[2] = n0 + nx;
    ids[3] = n0 + nx + 1;
    ids[4] = n0 + nxy;
    ids[5] = n0 + nxy + 1;
    ids[6] = n0 + nxy + nx;
    ids[7] = n0 + nxy + nx + 1;
}

// driveHard.wgsl:15-35 and driveCompliant.wgsl:24-41 for node n, whose
// state is P (its position just predicted, or as it stands where the hard
// law holds it with w = 0), toward target + offset moving at `velocity`.
// Runs inside the pass that predicts the substep, for the node that pass has
// just handled: the state it reads is the one the reference's drive pass,
// the next in its order, would read.
__device__ __forceinline__ void driveNode(const FrameParams* fp, V target, V velocity, V offset, uint32_t n, float4 P,
                                          float4* pos, float4* prev, float4* vel) {
    const float dt = fp->dt;
    const V goal = target + offset;
    if (fp->law == VSIM_DRIVE_HARD) {
        const V here = xyz(P);
        const V step = velocity * dt;
        const V toGoal = goal - here;
        const V next = here + (dot(step, step) >= dot(toGoal, toGoal) ? toGoal : step);
        prev[n] = withW(here, 0.0f);
        pos[n] = withW(next, P.w);
        vel[n] = withW((next - here) / dt, 0.0f);
    } else {
        const V p = xyz(P);
        const float dt2 = dt * dt;
        const float tau2 = fp->responseTime * fp->responseTime;
        const float frac = dt2 / (dt2 + tau2);
        pos[n] = withW(p + (goal - p) * frac, P.w);
    }
}

// driveNode for driven record d: the record carries its offset and, in
// offsets.w, its body; the target is the scene's single grab target, or with
// perBodyGrab the body's own row of `grabs`.
__device__ __forceinline__ void applyDrive(const FrameParams* fp, const float4* offsets, const float4* grabs,
                                           int32_t d, uint32_t n, float4 P, float4* pos, float4* prev, float4* vel) {
    const float4 off = offsets[d];
    const uint32_t body = __float_as_uint(off.w);
    V target = mk(fp->grabTarget[0], fp->grabTarget[1], fp->grabTarget[2]);
    V velocity = mk(fp->grabVelocity[0], fp->grabVelocity[1], fp->grabVelocity[2]);
    if (fp->perBodyGrab) {
        target = xyz(grabs[2 * body]);
        velocity = xyz(grabs[2 * body + 1]);
    }
    driveNode(fp, target, velocity, xyz(off), n, P, pos, prev, vel);
}

// The drive's tables, for the passes that predict (DRIVE variants only).
struct DriveTables {
    const int32_t* drivenOf;  // per node: its row in the driven records, -1 for none
    const float4* offsets;    // per driven record: offset from the target, body as bits
    const float4* grabs;      // per body: drive target, drive target velocity
};

// finalize.wgsl:29-42.
__device__ __forceinline__ V resolvePlane(V p, V prev, V normal, float depth, float friction) {
    if (depth <= 0.0f) return p;
    V q = p + normal * depth;
    const V delta = q - prev;
    const V tangent = delta - normal * dot(delta, normal);
    const float len = length(tangent);
    if (len > 1e-9f) q = q - tangent * fminf(1.0f, friction * depth / len);
    return q;
}

// contacts.wgsl:84-91, in the body's grid; returns the bucket's index in the
// bucket arrays (the grid's base plus its linear index).
__device__ __forceinline__ uint32_t bucketOf(const DevBody* b, V p, int coord[3]) {
    const float q[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float last = float(b->gridDims[a]) - 1.0f;
        const float f = floorf((q[a] - b->gridOrigin[a]) / b->bucket);
        coord[a] = int(fminf(fmaxf(f, 0.0f), last));
    }
    return b->gridBase + uint32_t(coord[0]) + b->gridDims[0] * (uint32_t(coord[1]) + b->gridDims[1] * uint32_t(coord[2]));
}

constexpr uint32_t kIdle = 0xffffffffu;  // key and rank of a record whose body sits out the frame

// Whether records a and b may touch: the reference drops every same-body
// pair (collide.wgsl:66); with self contact on, a same-body pair counts when
// its nodes share no cell (rest grid distance above one on some axis).
__device__ __forceinline__ bool admitted(uint4 a, uint4 b, uint32_t selfContact) {
    if (a.y != b.y) return true;
    if (!selfContact) return false;
#pragma unroll
    for (int axis = 0; axis < 3; axis++) {
        const int ia = int((a.z >> (10 * axis)) & 1023u), ib = int((b.z >> (10 * axis)) & 1023u);
        if (abs(ia - ib) > 1) return true;
    }
    return false;
}

struct Contactor {
    uint4 me;
    V pi, movedI;
    float radius, wi, frictionI;
    uint32_t node;
};

// The per-hit arithmetic of collide.wgsl:70-118 for a candidate that passed
// the three skips (M: its motion over the substep, its body's friction);
// returns the correction to add.
__device__ __forceinline__ V contactCorrection(const Contactor& c, uint4 them, float4 Q, float4 M, float dist2) {
    const uint32_t mate = them.x;
    const V pj = xyz(Q);
    const V d = c.pi - pj;
    const float reach = c.radius + __uint_as_float(them.w);
    const float share = c.wi / (c.wi + Q.w);
    const float dist = sqrtf(dist2);
    V normal = mk(0.0f, c.node < mate ? 1.0f : -1.0f, 0.0f);
    if (dist > 1e-9f) normal = d / dist;
    const float depth = reach - dist;
    V correction = normal * (depth * share);
    const V sliding = c.movedI - xyz(M);
    const V tangent = sliding - normal * dot(sliding, normal);
    const float slid = length(tangent);
    if (slid > 1e-9f) {
        const float mu = fminf(c.frictionI, M.w);
        correction = correction - tangent * (share * fminf(1.0f, mu * depth / slid));
    }
    return correction;
}

// The reference's three skips, as written (a NaN distance is not skipped).
__device__ __forceinline__ bool contactHit(const Contactor& c, uint4 them, float4 Q, uint32_t selfContact,
                                           float& dist2) {
    const V d = c.pi - xyz(Q);
    dist2 = dot(d, d);
    const float reach = c.radius + __uint_as_float(them.w);
    return admitted(c.me, them, selfContact) && !(dist2 >= reach * reach) && !(c.wi + Q.w <= 0.0f);
}

// n / d with m = reciprocal64(d).
__device__ __forceinline__ uint32_t divBy(uint32_t n, uint64_t m) { return m ? uint32_t(__umul64hi(m, uint64_t(n))) : n; }

constexpr uint32_t kCollideBlock = 256;

// ------------------------------------------------------------- per item --

// predict.wgsl:19-36 for node n; returns its state as the drive sees it.
__device__ __forceinline__ float4 predictNode(const FrameParams* fp, uint32_t n, float4* pos, float4* prev,
                                              float4* vel) {
    float4 P = pos[n];
    if (P.w != 0.0f) {
        const float dt = fp->dt;
        const V g = mk(fp->gx, fp->gy, fp->gz);
        const V v = xyz(vel[n]) + g * dt;
        const V p = xyz(P);
        P = withW(p + v * dt, P.w);
        prev[n] = withW(p, 0.0f);
        pos[n] = P;
        vel[n] = withW(v, 0.0f);
    }
    return P;
}

// project.wgsl:35-184 on the cell `entry` (corner-0 node, body, y stride,
// z stride): its eight corners gathered, solved, written back.
template <bool LIMIT_ONLY>
__device__ __forceinline__ void solveCellAt(uint4 entry, const CellConsts& k, float4* pos, const float4* prevState,
                                            const StretchLengths& lens) {
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
    solveCell<LIMIT_ONLY>(p, prev, w, k, lens);
#pragma unroll
    for (int c = 0; c < 8; c++) pos[ids[c]] = withW(p[c], w[c]);
}

// finalize.wgsl:44-74 for node n (friction and velocity factor of its
// body). With CONTACT it first does what settle.wgsl:20-36 does for a node
// with surface record `record` -- apply its averaged correction, empty its
// bucket. With PREDICT it continues into the next substep's
// predict.wgsl:19-36, and calls drive(n, state) where the drive would take
// the node next.
template <bool CONTACT, bool PREDICT, class Drive>
__device__ __forceinline__ void finalizeNode(const FrameParams* fp, uint32_t n, float friction, float damp,
                                             int32_t record, float4* pos, float4* prevState, float4* vel,
                                             const float4* delta, const uint32_t* key, uint32_t* count,
                                             Drive&& drive) {
    float4 P = pos[n];
    if (CONTACT) {
        const int32_t r = record;
        if (r >= 0) {
            const float4 d = delta[r];
            if (d.w > 0.0f) {
                const V step = xyz(d) * (1.0f / d.w);
                P = withW(xyz(P) + step, P.w);
                if (P.w == 0.0f) pos[n] = P;
            }
            count[key[r]] = 0;
        }
    }
    if (P.w == 0.0f) {
        // held by the hard law: the next substep's drive takes it from here
        if (PREDICT) drive(n, P);
        return;
    }
    const V prev = xyz(prevState[n]);
    const float fr = friction;
    const V mn = mk(fp->tankMin[0], fp->tankMin[1], fp->tankMin[2]);
    const V mx = mk(fp->tankMax[0], fp->tankMax[1], fp->tankMax[2]);
    V p = xyz(P);
    p = resolvePlane(p, prev, mk(0.0f, 1.0f, 0.0f), mn.y - p.y, fr);
    p = resolvePlane(p, prev, mk(1.0f, 0.0f, 0.0f), mn.x - p.x, fr);
    p = resolvePlane(p, prev, mk(-1.0f, 0.0f, 0.0f), p.x - mx.x, fr);
    p = resolvePlane(p, prev, mk(0.0f, 0.0f, 1.0f), mn.z - p.z, fr);
    p = resolvePlane(p, prev, mk(0.0f, 0.0f, -1.0f), p.z - mx.z, fr);
    const float dt = fp->dt;
    V v = (p - prev) / dt;
    v = v * damp;
    if (PREDICT) {
        const V g = mk(fp->gx, fp->gy, fp->gz);
        const V v2 = v + g * dt;
        const float4 next = withW(p + v2 * dt, P.w);
        prevState[n] = withW(p, 0.0f);
        pos[n] = next;
        vel[n] = withW(v2, 0.0f);
        drive(n, next);
    } else {
        pos[n] = withW(p, P.w);
        vel[n] = withW(v, 0.0f);
    }
}

// bin.wgsl:9-23 for live record r (node, body in rec): its bucket and its
// arrival rank there.
__device__ __forceinline__ void binRecord(uint32_t r, uint4 rec, const DevBody* bodies, const float4* pos,
                                          uint32_t* key, uint32_t* rank, uint32_t* count) {
    int coord[3];
    const uint32_t b = bucketOf(bodies + rec.y, xyz(pos[rec.x]), coord);
    key[r] = b;
    rank[r] = atomicAdd(&count[b], 1u);
}


struct ContactArrays {
    const DevBody* bodies;
    const uint4* surf;
    const uint32_t* key;
    const uint32_t* rank;
    const uint32_t* start;
    const uint32_t* count;
    const uint4* sMeta;
    const float4* sPos;
    const float4* sMoved;
    const uint32_t* sRec;
    const uint32_t* sKey;
    float4* delta;
};

// sort.wgsl:14-53 for binned record r (see canonKernel): a record of a
// bucket of at most kBucketSlots entries copies itself to its place; in a
// larger bucket the first-arriving record orders and copies them all.
__device__ __forceinline__ void canonRecord(uint32_t r, const ContactArrays& a, uint32_t* entries,
                                            const SortedEntries& out, const float4* pos, const float4* prevState) {
    const uint32_t b = a.key[r];
    const uint32_t n = a.count[b];
    const uint32_t base = a.start[b];
    uint32_t* e = entries + base;
    auto copyOut = [&](uint32_t at, uint32_t record, uint4 rec) {
        const float4 P = pos[rec.x], R = prevState[rec.x];
        out.sMeta[at] = rec;
        out.sPos[at] = P;
        out.sMoved[at] = withW(xyz(P) - xyz(R), a.bodies[rec.y].friction);
        out.sRec[at] = record;
        out.sKey[at] = b;
    };
    if (n <= kBucketSlots) {
        const uint4 mine = a.surf[r];
        uint32_t place = 0;
        for (uint32_t j = 0; j < n; j++) place += e[j] < r ? 1u : 0u;
        copyOut(base + place, r, mine);
        return;
    }
    if (a.rank[r] != 0) return;
    const uint32_t m = kBucketSlots;
    for (uint32_t i = 1; i < m; i++) {
        const uint32_t v = e[i];
        uint32_t at = i;
        while (at > 0 && e[at - 1] > v) {
            e[at] = e[at - 1];
            at--;
        }
        e[at] = v;
    }
    // Past capacity, keep the lowest kBucketSlots in the visible prefix.
    for (uint32_t i = m; i < n; i++) {
        const uint32_t v = e[i];
        if (v >= e[m - 1]) continue;
        e[i] = e[m - 1];
        uint32_t at = m - 1;
        while (at > 0 && e[at - 1] > v) {
            e[at] = e[at - 1];
            at--;
        }
        e[at] = v;
    }
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t other = e[k];
        copyOut(base + k, other, a.surf[other]);
    }
}

// Entry i of the bucket order: its record r, position, motion and bucket as
// canonRecord copied them (positions have not moved since), five
// independent loads; `centre` gets the bucket's coordinates, from the
// bucket binRecord gave it -- integer division by the grid's dimensions
// rather than bucketOf's three float divides.
__device__ __forceinline__ Contactor contactorAt(uint32_t i, const ContactArrays& a, uint32_t& r, int centre[3]) {
    Contactor c;
    r = a.sRec[i];
    c.me = a.sMeta[i];
    c.node = c.me.x;
    c.radius = __uint_as_float(c.me.w);
    const float4 P = a.sPos[i], M = a.sMoved[i];
    c.wi = P.w;
    c.pi = xyz(P);
    c.movedI = xyz(M);
    c.frictionI = M.w;
    const DevBody* grid = a.bodies + c.me.y;
    const uint32_t linear = a.sKey[i] - grid->gridBase;
    const uint32_t z = divBy(linear, grid->divXY);
    const uint32_t rest = linear - z * (grid->gridDims[0] * grid->gridDims[1]);
    const uint32_t y = divBy(rest, grid->divX);
    centre[0] = int(rest - y * grid->gridDims[0]);
    centre[1] = int(y);
    centre[2] = int(z);
    return c;
}

// Neighbour bucket q of a bucket (q = dx + 3 dy + 9 dz, offsets + 1).
__device__ __forceinline__ uint32_t neighbourBucket(const DevBody* grid, const int centre[3], int q, bool& inside) {
    const int x = centre[0] + q % 3 - 1, y = centre[1] + (q / 3) % 3 - 1, z = centre[2] + q / 9 - 1;
    const int dims[3] = {int(grid->gridDims[0]), int(grid->gridDims[1]), int(grid->gridDims[2])};
    inside = x >= 0 && x < dims[0] && y >= 0 && y < dims[1] && z >= 0 && z < dims[2];
    return grid->gridBase + uint32_t(x) + uint32_t(dims[0]) * (uint32_t(y) + uint32_t(dims[1]) * uint32_t(z));
}

// collide.wgsl:16-125 for entry i of the bucket order, by one thread: its
// candidates in the reference's order, each hit added to the sum in turn.
// emit(r, at) is called for every counted hit.
template <bool EMIT, class Emit>
__device__ __forceinline__ void collideThread(uint32_t i, const ContactArrays& a, uint32_t selfContact,
                                              Emit&& emit) {
    uint32_t r;
    int centre[3];
    const Contactor c = contactorAt(i, a, r, centre);
    const DevBody* grid = a.bodies + c.me.y;
    uint32_t live = 0;  // which neighbour buckets hold entries: 27 independent loads
#pragma unroll
    for (int q = 0; q < 27; q++) {
        bool inside;
        const uint32_t b = neighbourBucket(grid, centre, q, inside);
        if (inside && a.count[b] != 0) live |= 1u << q;
    }
    V sum = mk(0.0f, 0.0f, 0.0f);
    float hits = 0.0f;
    while (live) {
        const int q = __ffs(live) - 1;
        live &= live - 1;
        bool inside;
        const uint32_t b = neighbourBucket(grid, centre, q, inside);
        const uint32_t n = a.count[b];
        const uint32_t held = n < kBucketSlots ? n : kBucketSlots;
        const uint32_t at = a.start[b];
        for (uint32_t k = 0; k < held; k++) {
            const uint4 them = a.sMeta[at + k];
            const float4 Q = a.sPos[at + k], M = a.sMoved[at + k];
            float dist2;
            if (!contactHit(c, them, Q, selfContact, dist2)) continue;
            sum = sum + contactCorrection(c, them, Q, M, dist2);
            hits = hits + 1.0f;
            if (EMIT) emit(r, at + k);
        }
    }
    if (!EMIT) a.delta[r] = withW(sum, hits);
}

// The same for entry i by a whole warp (every lane calls it with the same
// i): lane q < 27 sizes neighbour bucket q, a warp scan turns the sizes into
// offsets, and the candidates are dealt to the lanes 32 at a time, each
// finding its run as the last one starting at or before it. `starting` is
// the warp's 32 words of shared memory. Hits are added in candidate order.
template <bool EMIT, class Emit>
__device__ __forceinline__ void collideWarp(uint32_t i, const ContactArrays& a, uint32_t selfContact,
                                            uint32_t* starting, Emit&& emit) {
    constexpr unsigned kAll = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t r;
    int centre[3];
    const Contactor c = contactorAt(i, a, r, centre);
    const DevBody* grid = a.bodies + c.me.y;
    uint32_t held = 0, first = 0;
    if (lane < 27) {
        bool inside;
        const uint32_t b = neighbourBucket(grid, centre, int(lane), inside);
        if (inside) {
            // loaded together (start[b] is stale and unused when empty)
            const uint32_t n = a.count[b];
            first = a.start[b];
            held = n < kBucketSlots ? n : kBucketSlots;
        }
    }
    // Inclusive prefix of the run lengths: lane q's run is [end - held, end).
    uint32_t end = held;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(kAll, end, d);
        if (lane >= uint32_t(d)) end += v;
    }
    const uint32_t candidates = __shfl_sync(kAll, end, 31);
    V sum = mk(0.0f, 0.0f, 0.0f);
    float hits = 0.0f;
    uint32_t carry = 0;  // the run holding the round's first candidate, if it began earlier
    for (uint32_t round = 0; round < candidates; round += 32) {
        const uint32_t cand = round + lane;
        // The run holding the candidate: the last run to start at or before
        // it. Runs that start in this round mark their positions.
        const uint32_t begin = end - held;
        uint32_t bit = 0;
        if (held && begin >= round && begin < round + 32) {
            bit = 1u << (begin - round);
            starting[begin - round] = lane;
        }
        const uint32_t starts = __reduce_or_sync(kAll, bit);
        __syncwarp();
        const uint32_t below = starts & (0xffffffffu >> (31 - lane));
        const uint32_t lo = below ? starting[31 - __clz(below)] : carry;
        carry = __shfl_sync(kAll, lo, 31);
        __syncwarp();  // the next round rewrites `starting`
        const uint32_t runEnd = __shfl_sync(kAll, end, lo);
        const uint32_t runHeld = __shfl_sync(kAll, held, lo);
        const uint32_t runFirst = __shfl_sync(kAll, first, lo);
        const uint32_t at = runFirst + (cand - (runEnd - runHeld));
        bool hit = false;
        V correction = mk(0.0f, 0.0f, 0.0f);
        if (cand < candidates) {
            const uint4 them = a.sMeta[at];
            const float4 Q = a.sPos[at], M = a.sMoved[at];
            float dist2;
            if (contactHit(c, them, Q, selfContact, dist2)) {
                hit = true;
                correction = contactCorrection(c, them, Q, M, dist2);
                if (EMIT) emit(r, at);
            }
        }
        // Candidate order = lane order.
        uint32_t mask = __ballot_sync(kAll, hit);
        while (mask) {
            const int l = __ffs(mask) - 1;
            mask &= mask - 1;
            const V add = mk(__shfl_sync(kAll, correction.x, l), __shfl_sync(kAll, correction.y, l),
                             __shfl_sync(kAll, correction.z, l));
            sum = sum + add;
            hits = hits + 1.0f;
        }
    }
    if (!EMIT && lane == 0) a.delta[r] = withW(sum, hits);
}

}  // namespace vsim
