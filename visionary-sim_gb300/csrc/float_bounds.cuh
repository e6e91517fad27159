// The cloud voxeliser's float decisions that stand in for double ones, with
// the double reference they must agree with, usable on the host and the
// device alike: every operation is a single IEEE operation (contraction
// off on both), so a host test checks the device's arithmetic.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>

#ifdef __CUDACC__
#define VSIM_BOUNDS_HD __host__ __device__ __forceinline__
#else
#define VSIM_BOUNDS_HD inline
#endif

namespace vsim {
namespace bounds {

// JavaScript's Math.hypot as V8 evaluates it (its published math builtin):
// infinity if any argument is infinite, else NaN if any is NaN, else 0 when
// all are 0; otherwise the magnitudes over the largest, squared and summed in
// argument order with Kahan compensation, square root times the largest.
VSIM_BOUNDS_HD double hypotV8(double a, double b, double c) {
    a = std::fabs(a);
    b = std::fabs(b);
    c = std::fabs(c);
    if (std::isinf(a) || std::isinf(b) || std::isinf(c)) return std::numeric_limits<double>::infinity();
    if (std::isnan(a) || std::isnan(b) || std::isnan(c)) return std::numeric_limits<double>::quiet_NaN();
    const double top = std::fmax(a, std::fmax(b, c));
    if (top == 0.0) return 0.0;
    const double v[3] = {a, b, c};
    double total = 0.0, compensation = 0.0;
    for (int r = 0; r < 3; r++) {
        // x / x is exactly 1 and 0 / x exactly 0: those divisions are skipped
        const double n = v[r] == top ? 1.0 : v[r] == 0.0 ? 0.0 : v[r] / top;
        const double summand = n * n - compensation;
        const double preliminary = total + summand;
        compensation = (preliminary - total) - summand;
        total = preliminary;
    }
    return std::sqrt(total) * top;
}

// The reach estimate, sqrtf of the float sum of the float products'
// squares, is within 2^-21 of V8's hypot of the double products (relative):
// the float products are within 2^-22.4 of the double ones (float(sigma),
// the radius and the product each rounded once), their squares and two sums
// add under 2^-21, the square root halves that, and V8's own evaluation is
// within 2^-50 of the exact hypot. kReachSlack, 8 times that, brackets the
// exact reach:
//   hf (1 - kReachSlack) <= reach <= hf (1 + kReachSlack),
// both products rounded in double well inside the slack. It holds while
// every nonzero product lies in [2^-60, 2^60] (squares and sums stay normal
// floats) and the radii are 0 or in [2^-100, 2^100].
constexpr double kReachSlack = 0x1p-18;

// The estimate along world axis a from the frame (column-major float32
// entries) and the radii float(sigma) * scale; NaN where out of its range.
VSIM_BOUNDS_HD float reachEstimate(const float col[9], const float r[3], int a) {
    float sum = 0.0f;
    for (int k = 0; k < 3; k++) {
        const float c = col[3 * k + a];
        const float v = c * r[k];
        if (c != 0.0f && r[k] != 0.0f && !(std::fabs(v) >= 0x1p-60f && std::fabs(v) <= 0x1p60f))
            return std::numeric_limits<float>::quiet_NaN();
        sum += v * v;
    }
    return std::sqrt(sum);
}

// A radius float(sigma) * scale for the estimate, NaN where out of its
// range.
VSIM_BOUNDS_HD float radiusEstimate(float sigmaF, float scale) {
    const float r = sigmaF * scale;
    const float m = std::fabs(r);
    return (r == 0.0f || (m >= 0x1p-100f && m <= 0x1p100f)) ? r : std::numeric_limits<float>::quiet_NaN();
}

// The cell floor(RN(RN(x - origin) / h)) of cloudVolume.js:384-386, for x =
// RN(c + s) with s anywhere in [s1, s2] (c the position, s a signed
// half-reach or 0), decided in float when every such x shares one cell.
// With co = float(c - float(origin)), e(s) = (co + s) * invH: the float
// origin, the two sums and the product each round within 2^-24 of their
// magnitude, invH within 2^-24 of 1 / h, so e is within 5 2^-24 M of (c +
// s - origin) / h, M = (|origin| + |c| + |co| + |s|) / h bounding every
// magnitude in cells; the double path's quotient is within 3 2^-53 M of it
// too. delta = 2^-20 M (plus 2^-100 for subnormal roundings) covers both,
// and e and the double quotient are monotone in s, so one floor of e(s1) -
// delta and e(s2) + delta is the floor of every x's quotient. False when
// they differ or leave float's exact integers.
VSIM_BOUNDS_HD bool floatCell(float co, float s1, float s2, float invH, float delta, int64_t& cell) {
    const float a = std::floor((co + s1) * invH - delta), b = std::floor((co + s2) * invH + delta);
    if (a != b || !(std::fabs(a) < 0x1p22f)) return false;
    cell = int64_t(a);
    return true;
}

// delta of floatCell for a position c and half-reach bound `wide` (0 for the
// centre), with originMag = max(|float(origin)|, 2^-100).
VSIM_BOUNDS_HD float cellDelta(float originMag, float c, float co, float wide, float invH) {
    return 0x1p-20f * (originMag + std::fabs(c) + std::fabs(co) + wide) * invH + 0x1p-100f;
}

}  // namespace bounds
}  // namespace vsim
