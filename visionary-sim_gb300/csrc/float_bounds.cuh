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


// The float reciprocal, correctly rounded (the device's rcp.rn; on the host
// the IEEE quotient 1 / x, the same value).
VSIM_BOUNDS_HD float rcpRn(float x) {
#ifdef __CUDA_ARCH__
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

struct GridView {
    uint32_t dims[3];
    double origin[3];
    double h;
    float invH;  // float(1 / h), 0 outside [2^-40, 2^40]
    float hF;    // float(h)
    float originF[3];    // float(origin)
    float originMag[3];  // max(|float(origin)|, 2^-100)
    bool floatBound;     // h in [2^-30, 2^30] and |origin| <= 2^40 on every axis
    uint32_t cells;
};

// One Gaussian as an ellipsoid (cloudVolume.js:195-210): the column-major
// rotation as the reference's Float32Array holds it, the half-axes in the
// Gaussian's frame.
struct Ellipsoid {
    double col[9];
    double radius[3];
};

// One of a cell's nine sample points (its eight corners in corners.js:12-21
// order, then its centre) tested against the ellipsoid in the reference's
// double arithmetic and order (cloudVolume.js:255-273).
VSIM_BOUNDS_HD void sampleOffset(int s, double& ox, double& oy, double& oz) {
    ox = s == 8 ? 0.5 : double(s & 1);
    oy = s == 8 ? 0.5 : double((s >> 1) & 1);
    oz = s == 8 ? 0.5 : double((s >> 2) & 1);
}

VSIM_BOUNDS_HD bool sampleInside(const GridView& g, int64_t i, int64_t j, int64_t k, int s, const double c[3],
                             const Ellipsoid& e) {
    double ox, oy, oz;
    sampleOffset(s, ox, oy, oz);
    const double dx = g.origin[0] + (double(i) + ox) * g.h - c[0];
    const double dy = g.origin[1] + (double(j) + oy) * g.h - c[1];
    const double dz = g.origin[2] + (double(k) + oz) * g.h - c[2];
    double sum = 0.0;
    for (int a = 0; a < 3; a++) {
        const double t = (e.col[3 * a] * dx + e.col[3 * a + 1] * dy + e.col[3 * a + 2] * dz) / e.radius[a];
        sum += t * t;
    }
    return sum <= 1.0;
}

struct Box {
    int64_t lo[3], hi[3];
    VSIM_BOUNDS_HD int64_t extent(int a) const { return hi[a] - lo[a] + 1; }
    VSIM_BOUNDS_HD int64_t cells() const { return extent(0) * extent(1) * extent(2); }
};

// The sample test in float, with a bound on how far its sum of squares can
// be from the double evaluation's; a sample whose float sum is further than
// the bound from 1 is decided by it, every other one is evaluated in double.
// Same answers, far fewer double operations (a double division costs tens
// of float operations on this part). The bound, per Gaussian and box:
//   offset: float(base) + off * float(h), with base = origin + lo h - c (in
//     double) and off = i - lo + ox exact, against the double sequence
//     origin + (i + ox) h - c: within 2^-22 X + A, where X = |base| +
//     (extent + 1) h bounds |base|, off h and the offset, and A = 2^-50
//     (|origin| + |c| + (|lo| + extent + 1) h) the double sequence's own
//     rounding;
//   dot with column a (float entries, exact): the propagated offset errors
//     plus 2^-22 sum_k |col| X_k for its own three roundings;
//   t = dot / r: that over r (held x4 in `err`, a factor of 4 to spare),
//     plus 2^-23 |t| for the float reciprocal and product (taken x4);
//   sum of squares: sum_a (2|t_a| + e_a) e_a, plus 2^-21 s for its roundings,
//     plus a floor of 2^-20 so that 1 +- the bound is never rounded away.
// A Gaussian whose bound is not small (err >= 1e-3), whose half-axes or cell
// are outside [1e-30, 1e30], or whose box is wider than 2^20 cells is tested
// in double throughout.
struct FloatTest {
    float base[3];
    float h;
    float col[9];
    float inv[3];
    float err[3];
};

VSIM_BOUNDS_HD bool floatTestOf(const GridView& g, const Box& b, const double c[3], const Ellipsoid& e, FloatTest& f) {
    if (!(g.h > 1e-30 && g.h < 1e30)) return false;
    double X[3], ex[3];
    for (int a = 0; a < 3; a++) {
        if (b.extent(a) > (1 << 20)) return false;
        const double base = (g.origin[a] + double(b.lo[a]) * g.h) - c[a];
        const double span = double(b.extent(a) + 1) * g.h;
        X[a] = std::fabs(base) + span;
        ex[a] = 0x1p-22 * X[a] + 0x1p-50 * (std::fabs(g.origin[a]) + std::fabs(c[a]) + std::fabs(double(b.lo[a])) * g.h + span);
        f.base[a] = float(base);
    }
    f.h = float(g.h);
    for (int q = 0; q < 9; q++) f.col[q] = float(e.col[q]);
    for (int a = 0; a < 3; a++) {
        const double r = e.radius[a];
        if (!(r > 1e-30 && r < 1e30)) return false;
        // the float reciprocal of float(r): within 2^-23 of 1 / r, inside the
        // 2^-21 |t| allowance
        f.inv[a] = rcpRn(float(r));
        double dotErr = 0.0;
        for (int k = 0; k < 3; k++) dotErr += std::fabs(e.col[3 * a + k]) * (ex[k] + 0x1p-22 * X[k]);
        // above 4 dotErr / r: the reciprocal's error and every rounding of
        // this product are covered by the (1 + 2^-20)
        const double err = 4.0 * dotErr * double(f.inv[a]) * (1.0 + 0x1p-20);
        if (!(err < 1e-3)) return false;
        f.err[a] = float(err);
    }
    return true;
}

// floatTestOf with the bound's terms summed in float instead of double, from
// the frame rows the bounds pass kept (f.col, exactly floatTestOf's), the
// position as float (exact) and the radius as float(sigma) * scale (within
// 2^-23 of float(r), so its reciprocal stays inside the 2^-21 |t|
// allowance). All terms are sums and products of magnitudes, so each float
// rounding (2^-24 relative, about a dozen along any chain) lowers them by
// under 2^-20 in all, which the final (1 + 2^-16) more than restores;
// magnitudes under 2^-100 are counted as 2^-100. Only the base offsets are
// formed in double, as floatTestOf forms them. Inside the ranges checked
// here (and g.floatBound's: h in [2^-30, 2^30], |origin| <= 2^40) no term is
// a subnormal float or overflows (the smallest, 2^-50 h, is above 2^-80; the
// error after the reciprocal above 2^-113); elsewhere floatTestOf decides.
// Conversions from double cost FP64-pipe time on this part: there are four
// a Gaussian.
VSIM_BOUNDS_HD bool floatTestInFloat(const GridView& g, const Box& b, const double c[3], const float cf[3],
                                     const float col[9], double sigma, float sigmaF, const float scale[3],
                                     FloatTest& f) {
    float rf[3];
    bool ok = g.floatBound;
    for (int a = 0; a < 3; a++) {
        rf[a] = sigmaF * scale[a];
        ok = ok && std::fabs(cf[a]) <= 0x1p40f && b.extent(a) <= (1 << 20) && rf[a] >= 0x1p-30f && rf[a] <= 0x1p30f;
    }
    for (int q = 0; q < 9; q++) {
        const float m = std::fabs(col[q]);
        ok = ok && (m == 0.0f || (m >= 0x1p-30f && m <= 0x1p30f));
    }
    if (!ok) {
        Ellipsoid e;
        for (int q = 0; q < 9; q++) e.col[q] = col[q];
        for (int a = 0; a < 3; a++) e.radius[a] = sigma * double(scale[a]);
        return floatTestOf(g, b, c, e, f);
    }
    const float h = g.hF;
    float X[3], ex[3];
    for (int a = 0; a < 3; a++) {
        const double base = (g.origin[a] + double(b.lo[a]) * g.h) - c[a];
        f.base[a] = float(base);
        const float span = float(int32_t(b.extent(a) + 1)) * h;
        X[a] = std::fmax(std::fabs(f.base[a]), 0x1p-100f) + span;
        const float lo = float(int32_t(b.lo[a]));
        ex[a] = 0x1p-22f * X[a] + 0x1p-50f * (g.originMag[a] + std::fmax(std::fabs(cf[a]), 0x1p-100f) + std::fabs(lo) * h + span);
    }
    f.h = h;
    for (int q = 0; q < 9; q++) f.col[q] = col[q];
    for (int a = 0; a < 3; a++) {
        f.inv[a] = rcpRn(rf[a]);
        float dotErr = 0.0f;
        for (int k = 0; k < 3; k++) dotErr += std::fabs(f.col[3 * a + k]) * (ex[k] + 0x1p-22f * X[k]);
        const float err = 4.0f * dotErr * f.inv[a] * (1.0f + 0x1p-16f);
        if (!(err < 1e-3f)) return false;
        f.err[a] = err;
    }
    return true;
}

// 1 inside, 0 outside, -1 too close to call in float.
VSIM_BOUNDS_HD int floatSample(const FloatTest& f, float ox, float oy, float oz) {
    const float dx = f.base[0] + ox * f.h, dy = f.base[1] + oy * f.h, dz = f.base[2] + oz * f.h;
    float sum = 0.0f, bound = 0.0f;
    for (int a = 0; a < 3; a++) {
        const float t = (f.col[3 * a] * dx + f.col[3 * a + 1] * dy + f.col[3 * a + 2] * dz) * f.inv[a];
        const float at = std::fabs(t);
        const float et = f.err[a] + 0x1p-21f * at;
        sum += t * t;
        bound += (2.0f * at + et) * et;
    }
    bound += 0x1p-20f * sum + 0x1p-20f;
    if (sum > 1.0f + bound) return 0;
    if (sum < 1.0f - bound) return 1;
    return -1;
}

}  // namespace bounds
}  // namespace vsim
