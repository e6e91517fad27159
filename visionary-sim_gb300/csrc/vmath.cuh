// Device vector arithmetic in the reference's evaluation order (WGSL: left
// to right, `dot` as (x + y) + z, `M * v` as c0 v.x + c1 v.y + c2 v.z).
//
// Rounding is fixed, not left to the compiler: every translation unit that
// includes this is compiled with -fmad=false, so a multiply and an add fuse
// only where fmaf is written -- in dot, cross, M * v and the determinant
// here, and at the named places of the solver kernels -- and everything else
// rounds once per operation. The CPU restatement of the solver fuses at the
// same places (std::fma); together with IEEE division and square root
// (nvcc's defaults) the kernels' results equal it bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace vsim {

struct V {
    float x, y, z;
};

__device__ __forceinline__ V mk(float x, float y, float z) { return V{x, y, z}; }
__device__ __forceinline__ V xyz(float4 a) { return V{a.x, a.y, a.z}; }

// fma3 issues x and y as one packed FP32x2 fused multiply-add (sm_100 and
// later), which rounds each lane to nearest exactly as fmaf does. Adds,
// subtractions and multiplies stay scalar: their packed forms round each
// lane exactly as the scalar operations do (checked bit for bit on the GPU,
// subnormal and signed-zero operands included), but using them made the
// compiler keep the colour pass's cell in local memory (a 144-byte stack
// frame in every colour-pass kernel).
__device__ __forceinline__ float2 xyOf(V a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ V withXy(float2 xy, float z) { return V{xy.x, xy.y, z}; }
__device__ __forceinline__ V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator-(V a) { return V{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V operator*(V a, float s) { return V{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V operator*(float s, V a) { return V{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V operator/(V a, float s) { return V{a.x / s, a.y / s, a.z / s}; }
// a * s + acc per component, one rounding each.
__device__ __forceinline__ V fma3(V a, float s, V acc) {
    return withXy(__ffma2_rn(xyOf(a), make_float2(s, s), xyOf(acc)), fmaf(a.z, s, acc.z));
}
// x first, then y and z fused in.
__device__ __forceinline__ float dot(V a, V b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ float length(V a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V cross(V a, V b) {
    return V{fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x))};
}

// Column-major 3x3: c[k] is column k.
struct M {
    V c[3];
};

__device__ __forceinline__ M operator*(const M& m, float s) { return M{{m.c[0] * s, m.c[1] * s, m.c[2] * s}}; }
__device__ __forceinline__ V mul(const M& m, V v) { return fma3(m.c[2], v.z, fma3(m.c[1], v.y, m.c[0] * v.x)); }
// Expansion order of the reference's mat3Determinant (mat3.js:25-31).
__device__ __forceinline__ float determinant(const M& m) {
    const float m0 = m.c[0].x, m1 = m.c[0].y, m2 = m.c[0].z;
    const float m3 = m.c[1].x, m4 = m.c[1].y, m5 = m.c[1].z;
    const float m6 = m.c[2].x, m7 = m.c[2].y, m8 = m.c[2].z;
    const float t1 = fmaf(m4, m8, -(m7 * m5));
    const float t2 = fmaf(m1, m8, -(m7 * m2));
    const float t3 = fmaf(m1, m5, -(m4 * m2));
    return fmaf(m6, t3, fmaf(m0, t1, -(m3 * t2)));
}

__device__ __forceinline__ float4 withW(V p, float w) { return make_float4(p.x, p.y, p.z, w); }

// Programmatic dependent launch: wait for the preceding kernel in the stream
// (its writes visible) before touching memory, and let the next kernel's
// launch begin while this one runs. Both are no-ops without the launch
// attribute.
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdlLaunchNext() { asm volatile("griddepcontrol.launch_dependents;" :::); }

}  // namespace vsim
