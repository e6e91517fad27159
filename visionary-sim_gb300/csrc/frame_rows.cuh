// A Gaussian's rotation matrix as the reference's voxeliser holds it
// (mat3.js:71-87, mat3FromQuat, into a Float32Array: every entry formed in
// JavaScript doubles from the float32 quaternion, then rounded to float32),
// computed in float.
//
// In double the products of two float32 values are exact, so an entry is
//   off the diagonal:  float(2 RN_d(a b +- c d))
//   on the diagonal:   float(RN_d(1 - 2 RN_d(a a + b b)))
// Here the sums are carried exactly as float pairs (each product split by a
// fused multiply-add into its rounded value and its exact error, sums by
// TwoSum), a float candidate A is formed, and A is taken only when the
// distance from the exact value to A, plus how far the double roundings can
// move it, stays under half the smaller gap between A and its float
// neighbours: then the double path rounds to A as well. Otherwise (a
// product or the result outside [2^-60, 2^60], a value too close to a
// rounding boundary) the entry is not certified and the caller forms the
// frame in double. Zero products are exact and handled as the double
// arithmetic handles them, signed zeros included.
//
// Every operation is a single IEEE float operation or fmaf, so the host
// compiler (with contraction off) and the device give the same results; the
// CPU test compiles this header against the double formula.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define VSIM_FRAME_HD __host__ __device__ __forceinline__
#else
#define VSIM_FRAME_HD inline
#endif

namespace vsim {
namespace frame {

// Half the smaller gap between a and its float neighbours, for |a| in
// [2^-60, 2^100] (a power of two has the finer gap below it).
VSIM_FRAME_HD float halfGap(float a) {
    uint32_t u;
    std::memcpy(&u, &a, 4);
    u &= 0x7fffffffu;
    const uint32_t exponent = u >> 23, mantissa = u & 0x7fffffu;
    const uint32_t ulpBits = (exponent - 23u) << 23;  // 2^(e - 23): the gap above
    float ulp;
    std::memcpy(&ulp, &ulpBits, 4);
    return mantissa == 0 ? ulp * 0.25f : ulp * 0.5f;
}

// s + e = a + b exactly (Knuth's TwoSum).
VSIM_FRAME_HD void twoSum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

VSIM_FRAME_HD bool productInRange(float p) {
    const float m = std::fabs(p);
    return m >= 0x1p-60f && m <= 0x1p60f;
}

// a b + c d = s + r + eps, |eps| <= err; false when a nonzero product is out
// of range (its split would not be exact).
VSIM_FRAME_HD bool productSum(float a, float b, float c, float d, float& s, float& r, float& err) {
    const float p1 = a * b, p2 = c * d;
    const bool zero1 = a == 0.0f || b == 0.0f, zero2 = c == 0.0f || d == 0.0f;
    if ((!zero1 && !productInRange(p1)) || (!zero2 && !productInRange(p2))) return false;
    const float e1 = zero1 ? 0.0f : std::fma(a, b, -p1);  // exact: p1 + e1 = a b
    const float e2 = zero2 ? 0.0f : std::fma(c, d, -p2);
    float t;
    twoSum(p1, p2, s, t);
    const float r1 = t + e1;
    r = r1 + e2;
    // two roundings, each within 2^-24 of its result (2^-140 for subnormals)
    err = (0x1p-24f * (std::fabs(r1) + std::fabs(r)) + 0x1p-140f) * 1.0001f;
    return true;
}

// float(2 RN_d(a b + c d)) into out; false if not certified.
VSIM_FRAME_HD bool offDiagonal(float a, float b, float c, float d, float& out) {
    const bool zero1 = a == 0.0f || b == 0.0f, zero2 = c == 0.0f || d == 0.0f;
    if (zero1 || zero2) {
        // A zero product adds nothing but its sign: the sum is the other
        // product, exact in double, so one rounding to float; two zeros
        // add as signed zeros do in double.
        const float p1 = a * b, p2 = c * d;
        if (zero1 && zero2) {
            out = 2.0f * (p1 + p2);
            return true;
        }
        const float p = zero1 ? p2 : p1;
        if (!productInRange(p)) return false;
        out = 2.0f * p;
        return true;
    }
    float s, r, err;
    if (!productSum(a, b, c, d, s, r, err)) return false;
    float A, eA;
    twoSum(s, r, A, eA);  // s + r = A + eA exactly
    const float m = std::fabs(A);
    if (!(m >= 0x1p-60f && m <= 0x1p60f)) return false;
    // |S - A| <= |eA| + err; the double sum is within 2^-53 |S| of S
    const float bound = (std::fabs(eA) + err + 0x1p-50f * m) * 1.0001f;
    if (!(bound < halfGap(A))) return false;
    out = 2.0f * A;
    return true;
}

// float(RN_d(1 - 2 RN_d(a a + b b))) into out; false if not certified.
VSIM_FRAME_HD bool diagonal(float a, float b, float& out) {
    if (a == 0.0f && b == 0.0f) {
        out = 1.0f;  // 1 - 2 (+0): squares of zeros are +0
        return true;
    }
    float s, r, err;
    if (!productSum(a, a, b, b, s, r, err)) return false;
    // V = 1 - 2 S2 = (1 - 2 s) - 2 r - 2 eps; 1 - 2 s = u + tu exactly
    float u, tu;
    twoSum(1.0f, -2.0f * s, u, tu);
    const float vr = tu - 2.0f * r;  // within 2^-24 |vr| of tu - 2 r
    float A, eA;
    twoSum(u, vr, A, eA);
    const float m = std::fabs(A);
    if (!(m >= 0x1p-60f && m <= 0x1p60f)) return false;
    // |V - A| <= |eA| + 2^-24 |vr| + 2 err; the double path's two roundings
    // move V by under 2^-52 S2 + 2^-53 |V| (S2 <= |s| + |r| + err)
    const float bound =
        (std::fabs(eA) + 0x1p-24f * std::fabs(vr) + 2.0f * err + 0x1p-51f * (std::fabs(s) + std::fabs(r) + m)) *
        1.0001f;
    if (!(bound < halfGap(A))) return false;
    out = A;
    return true;
}

// The column-major entries of mat3FromQuat for the quaternion (x, y, z, w),
// each rounded to float32 as the reference stores it; false if any entry is
// not certified (then form them in double).
VSIM_FRAME_HD bool rowsInFloat(float x, float y, float z, float w, float col[9]) {
    bool ok = diagonal(y, z, col[0]);
    ok = ok && offDiagonal(x, y, z, w, col[1]);
    ok = ok && offDiagonal(x, z, y, -w, col[2]);
    ok = ok && offDiagonal(x, y, z, -w, col[3]);
    ok = ok && diagonal(x, z, col[4]);
    ok = ok && offDiagonal(y, z, x, w, col[5]);
    ok = ok && offDiagonal(x, z, y, w, col[6]);
    ok = ok && offDiagonal(y, z, x, -w, col[7]);
    ok = ok && diagonal(x, y, col[8]);
    return ok;
}

}  // namespace frame
}  // namespace vsim
