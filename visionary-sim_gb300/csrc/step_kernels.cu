// The substep kernels of the solver: prediction, the kinematic drive, the
// 8-colour stable Neo-Hookean projection, body contact and the closing pass.
//
// Node state lives in HBM as three float4 arrays in the reference's dense
// node order (pos, prev, vel; state.wgsl:16-19). pos.w carries the node's
// inverse mass as the solver sees it (the reference's separate nodeInvMass
// buffer, particles.js:206-215), so one 16-byte load brings a node's
// position and weight together; every kernel that writes pos keeps w.
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

void kuhnTable(float out[54]) {
    for (int t = 0; t < 6; t++)
        for (int col = 0; col < 3; col++)
            for (int row = 0; row < 3; row++) out[t * 9 + col * 3 + row] = float(kKuhn.v[t][col][row]);
}

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

// ------------------------------------------------------------- kernels --

// driveHard.wgsl:15-35 and driveCompliant.wgsl:24-41 for driven record d,
// node n, whose state is P (its position just predicted, or as it stands
// where the hard law holds it with w = 0). The record carries its body in
// offsets.w; the target is the scene's single grab target, or with
// perBodyGrab the body's own row of `grabs`. Runs inside the pass that
// predicts the substep, for the node that pass has just handled: the state
// it reads is the one the reference's drive pass, the next in its order,
// would read.
__device__ __forceinline__ void applyDrive(const FrameParams* __restrict__ fp, const float4* __restrict__ offsets,
                                           const float4* __restrict__ grabs, int32_t d, uint32_t n, float4 P,
                                           float4* __restrict__ pos, float4* __restrict__ prev,
                                           float4* __restrict__ vel) {
    const float4 off = offsets[d];
    const uint32_t body = __float_as_uint(off.w);
    const float dt = fp->dt;
    V target = mk(fp->grabTarget[0], fp->grabTarget[1], fp->grabTarget[2]);
    V velocity = mk(fp->grabVelocity[0], fp->grabVelocity[1], fp->grabVelocity[2]);
    if (fp->perBodyGrab) {
        target = xyz(grabs[2 * body]);
        velocity = xyz(grabs[2 * body + 1]);
    }
    const V goal = target + xyz(off);
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

// The drive's tables, for the passes that predict (DRIVE variants only).
struct DriveTables {
    const int32_t* drivenOf;  // per node: its row in the driven records, -1 for none
    const float4* offsets;    // per driven record: offset from the target, body as bits
    const float4* grabs;      // per body: drive target, drive target velocity
};

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
        const uint32_t n = q.n;
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
        if (DRIVE && q.driven >= 0) applyDrive(fp, drive.offsets, drive.grabs, q.driven, n, P, pos, prev, vel);
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
        uint32_t ids[8];
        cornerNodes(q.entry, ids);
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
        solveCell<LIMIT_ONLY>(p, prev, w, q.k, lens);
#pragma unroll
        for (int c = 0; c < 8; c++) pos[ids[c]] = withW(p[c], w[c]);
    });
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
        const uint32_t n = q.n;
        float4 P = pos[n];
        if (CONTACT) {
            const int32_t r = q.record;
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
            if (DRIVE && PREDICT && q.driven >= 0) applyDrive(fp, drive.offsets, drive.grabs, q.driven, n, P, pos,
                                                               prevState, vel);
            return;
        }
        const V prev = xyz(prevState[n]);
        const float fr = q.friction;
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
        v = v * q.damp;
        if (PREDICT) {
            const V g = mk(fp->gx, fp->gy, fp->gz);
            const V v2 = v + g * dt;
            const float4 next = withW(p + v2 * dt, P.w);
            prevState[n] = withW(p, 0.0f);
            pos[n] = next;
            vel[n] = withW(v2, 0.0f);
            if (DRIVE && q.driven >= 0) applyDrive(fp, drive.offsets, drive.grabs, q.driven, n, next, pos, prevState,
                                                   vel);
        } else {
            pos[n] = withW(p, P.w);
            vel[n] = withW(v, 0.0f);
        }
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
        int coord[3];
        const uint32_t b = bucketOf(bodies + rec.y, xyz(pos[rec.x]), coord);
        key[r] = b;
        rank[r] = atomicAdd(&count[b], 1u);
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
    forEachItem(work, [&](uint32_t r) {
        const uint32_t b = key[r];
        if (b == kIdle) return;
        const uint32_t n = count[b];
        const uint32_t base = start[b];
        uint32_t* e = entries + base;
        auto copyOut = [&](uint32_t at, uint32_t record, uint4 rec) {
            const float4 P = pos[rec.x], R = prevState[rec.x];
            sMeta[at] = rec;
            sPos[at] = P;
            sMoved[at] = withW(xyz(P) - xyz(R), bodies[rec.y].friction);
            sRec[at] = record;
            sKey[at] = b;
        };
        if (n <= kBucketSlots) {
            const uint4 mine = surf[r];
            uint32_t place = 0;
            for (uint32_t j = 0; j < n; j++) place += e[j] < r ? 1u : 0u;
            copyOut(base + place, r, mine);
            return;
        }
        if (rank[r] != 0) return;
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
            copyOut(base + k, other, surf[other]);
        }
    });
}

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

template <bool EMIT>
__global__ void __launch_bounds__(kCollideBlock, 5) collideKernel(
    const FrameParams* __restrict__ fp, uint32_t items, uint32_t warpModeBelow, const uint32_t* __restrict__ cursor,
    const DevBody* __restrict__ bodies, const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
    const uint4* __restrict__ sMeta, const float4* __restrict__ sPos, const float4* __restrict__ sMoved,
    const uint32_t* __restrict__ sRec, const uint32_t* __restrict__ sKey, float4* __restrict__ delta,
    uint32_t* __restrict__ pairs, uint32_t capacity, unsigned long long* __restrict__ pairCount) {
    pdlWait();
    pdlLaunchNext();
    constexpr unsigned kAll = 0xffffffffu;
    const uint32_t total = min(items, *cursor);
    const uint32_t selfContact = fp->selfContact;
    const uint32_t thread = blockIdx.x * blockDim.x + threadIdx.x;
    // Entry i of the bucket order: its record r, position, motion and bucket
    // as canonKernel copied them (positions have not moved since), five
    // independent loads.
    auto setup = [&](uint32_t i, uint32_t& r, int centre[3]) {
        Contactor c;
        r = sRec[i];
        c.me = sMeta[i];
        c.node = c.me.x;
        c.radius = __uint_as_float(c.me.w);
        const float4 P = sPos[i], M = sMoved[i];
        c.wi = P.w;
        c.pi = xyz(P);
        c.movedI = xyz(M);
        c.frictionI = M.w;
        const DevBody* grid = bodies + c.me.y;
        // The record's bucket coordinates, from the bucket binKernel gave it:
        // integer division by the grid's dimensions rather than bucketOf's
        // three float divides.
        const uint32_t linear = sKey[i] - grid->gridBase;
        const uint32_t z = divBy(linear, grid->divXY);
        const uint32_t rest = linear - z * (grid->gridDims[0] * grid->gridDims[1]);
        const uint32_t y = divBy(rest, grid->divX);
        centre[0] = int(rest - y * grid->gridDims[0]);
        centre[1] = int(y);
        centre[2] = int(z);
        return c;
    };
    // Neighbour bucket q of the record's bucket (q = dx + 3 dy + 9 dz, offsets + 1).
    auto neighbour = [&](const DevBody* grid, const int centre[3], int q, bool& inside) {
        const int x = centre[0] + q % 3 - 1, y = centre[1] + (q / 3) % 3 - 1, z = centre[2] + q / 9 - 1;
        const int dims[3] = {int(grid->gridDims[0]), int(grid->gridDims[1]), int(grid->gridDims[2])};
        inside = x >= 0 && x < dims[0] && y >= 0 && y < dims[1] && z >= 0 && z < dims[2];
        return grid->gridBase + uint32_t(x) + uint32_t(dims[0]) * (uint32_t(y) + uint32_t(dims[1]) * uint32_t(z));
    };
    auto emit = [&](uint32_t r, uint32_t at) {
        const unsigned long long slot = atomicAdd(pairCount, 1ull);
        if (slot < capacity) {
            pairs[2 * slot] = r;
            pairs[2 * slot + 1] = sRec[at];
        }
    };

    if (total >= warpModeBelow) {
        for (uint32_t i = thread; i < total; i += gridDim.x * blockDim.x) {
            uint32_t r;
            int centre[3];
            const Contactor c = setup(i, r, centre);
            const DevBody* grid = bodies + c.me.y;
            uint32_t live = 0;  // which neighbour buckets hold entries: 27 independent loads
#pragma unroll
            for (int q = 0; q < 27; q++) {
                bool inside;
                const uint32_t b = neighbour(grid, centre, q, inside);
                if (inside && count[b] != 0) live |= 1u << q;
            }
            V sum = mk(0.0f, 0.0f, 0.0f);
            float hits = 0.0f;
            while (live) {
                const int q = __ffs(live) - 1;
                live &= live - 1;
                bool inside;
                const uint32_t b = neighbour(grid, centre, q, inside);
                const uint32_t n = count[b];
                const uint32_t held = n < kBucketSlots ? n : kBucketSlots;
                const uint32_t at = start[b];
                for (uint32_t k = 0; k < held; k++) {
                    const uint4 them = sMeta[at + k];
                    const float4 Q = sPos[at + k], M = sMoved[at + k];
                    float dist2;
                    if (!contactHit(c, them, Q, selfContact, dist2)) continue;
                    sum = sum + contactCorrection(c, them, Q, M, dist2);
                    hits = hits + 1.0f;
                    if (EMIT) emit(r, at + k);
                }
            }
            if (!EMIT) delta[r] = withW(sum, hits);
        }
        return;
    }

    // Per warp: the neighbour bucket (lane) whose run starts at each candidate
    // position of the current round.
    __shared__ uint32_t runAt[kCollideBlock / 32][32];
    const uint32_t lane = threadIdx.x & 31;
    uint32_t* starting = runAt[threadIdx.x >> 5];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = thread >> 5; i < total; i += warps) {
        uint32_t r;
        int centre[3];
        const Contactor c = setup(i, r, centre);
        const DevBody* grid = bodies + c.me.y;
        uint32_t held = 0, first = 0;
        if (lane < 27) {
            bool inside;
            const uint32_t b = neighbour(grid, centre, int(lane), inside);
            if (inside) {
                // loaded together (start[b] is stale and unused when empty)
                const uint32_t n = count[b];
                first = start[b];
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
            // The run holding the candidate: the last run to start at or
            // before it. Runs that start in this round mark their positions.
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
                const uint4 them = sMeta[at];
                const float4 Q = sPos[at], M = sMoved[at];
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
        if (!EMIT && lane == 0) delta[r] = withW(sum, hits);
    }
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
    // a warp each while fewer than 2048 per SM, else a thread each.
    const uint32_t cg = std::min(blocks(recordItems, 8), 64 * c.sms);
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
