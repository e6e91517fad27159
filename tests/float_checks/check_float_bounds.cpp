// Checks the cloud voxeliser's float stand-ins (csrc/float_bounds.cuh)
// against the double arithmetic they replace:
//   reach: wherever reachEstimate gives an estimate hf, V8's hypot of the
//     double products lies in [hf (1 - slack), hf (1 + slack)], and also
//     between the float-rounded bounds the stamp uses;
//   cells: wherever floatCell decides a cell for position c and signed
//     half-reach s in [s1, s2], floor(RN(RN(RN(c + s) - origin) / h)) in
//     double is that cell for s1, s2 and points between them, including
//     positions placed within a few ulps of cell boundaries;
//   samples: wherever the float sample test decides, the double evaluation
//     of the sample decides the same, with ellipsoids scaled so their
//     surface passes within a few ulps of a sample, and with grids small
//     enough that the bound is summed in double (floatTestOf).
// Prints the counts; exits 1 on any disagreement.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "float_bounds.cuh"
#include "frame_rows.cuh"

using namespace vsim;

static uint64_t state = 0x2545f4914f6cdd1dull;
static uint64_t next() {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}
static double uniform() { return double(next() >> 11) * 0x1p-53; }

static void frameInDouble(float x, float y, float z, float w, float col[9]) {
    const double X = x, Y = y, Z = z, W = w;
    col[0] = float(1.0 - 2.0 * (Y * Y + Z * Z));
    col[1] = float(2.0 * (X * Y + Z * W));
    col[2] = float(2.0 * (X * Z - Y * W));
    col[3] = float(2.0 * (X * Y - Z * W));
    col[4] = float(1.0 - 2.0 * (X * X + Z * Z));
    col[5] = float(2.0 * (Y * Z + X * W));
    col[6] = float(2.0 * (X * Z + Y * W));
    col[7] = float(2.0 * (Y * Z - X * W));
    col[8] = float(1.0 - 2.0 * (X * X + Y * Y));
}

static int64_t doubleCell(float c, double s, double origin, double h) {
    const double x = double(c) + s;
    return int64_t(std::floor((x - origin) / h));
}

int main(int argc, char** argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    long reachChecked = 0, reachBad = 0, cellDecided = 0, cellTried = 0, cellBad = 0;
    const double sigmas[] = {1.0, 2.0, 2.5, 3.0};
    for (long n = 0; n < cases; n++) {
        // a Gaussian: random rotation (unit or not), scales log-uniform
        float q[4];
        double len = 0, v[4];
        for (int k = 0; k < 4; k++) {
            v[k] = uniform() * 2 - 1;
            len += v[k] * v[k];
        }
        const double norm = (next() % 4 == 0) ? 1.0 + uniform() : std::sqrt(len);
        for (int k = 0; k < 4; k++) q[k] = float(v[k] / norm);
        float col[9];
        frameInDouble(q[0], q[1], q[2], q[3], col);
        const double sigma = sigmas[next() % 4];
        float scale[3], rf[3];
        double r[3];
        for (int a = 0; a < 3; a++) {
            scale[a] = float(std::exp(std::log(1e-5) + uniform() * std::log(1e4)));
            r[a] = sigma * double(scale[a]);
            rf[a] = bounds::radiusEstimate(float(sigma), scale[a]);
        }
        for (int a = 0; a < 3; a++) {
            const float hf = bounds::reachEstimate(col, rf, a);
            if (std::isnan(hf)) continue;
            const double exact = bounds::hypotV8(double(col[a]) * r[0], double(col[3 + a]) * r[1], double(col[6 + a]) * r[2]);
            const double lo = double(hf) * (1.0 - bounds::kReachSlack), hi = double(hf) * (1.0 + bounds::kReachSlack);
            const float narrowF = hf * float(1.0 - bounds::kReachSlack), wideF = hf * float(1.0 + bounds::kReachSlack);
            reachChecked++;
            if (!(lo <= exact && exact <= hi && double(narrowF) <= exact && exact <= double(wideF))) {
                if (reachBad < 5) std::printf("reach outside bracket: hf %a exact %a\n", hf, exact);
                reachBad++;
            }
            // the box edges of this reach in a grid: origin, cell size, position
            const double h = std::exp(std::log(1e-4) + uniform() * std::log(1e3));
            const double origin = (uniform() * 2 - 1) * 2.0;
            const float invH = float(1.0 / h);
            if (!(invH >= 0x1p-40f && invH <= 0x1p40f)) continue;
            double place = origin + (uniform() * 300.0) * h;
            if (next() % 2) {
                // put c + wide within a few ulps of a cell boundary
                const double boundary = origin + std::floor(uniform() * 300.0) * h;
                place = boundary - double(wideF) + (uniform() * 2 - 1) * 4e-7 * h;
            }
            const float c = float(place);
            const float originF = float(origin);
            const float originMag = std::fmax(std::fabs(originF), 0x1p-100f);
            const float co = c - originF;
            const float delta = bounds::cellDelta(originMag, c, co, wideF, invH);
            const float edges[2][2] = {{-wideF, -narrowF}, {narrowF, wideF}};
            for (int e = 0; e < 2; e++) {
                int64_t cell;
                cellTried++;
                if (!bounds::floatCell(co, edges[e][0], edges[e][1], invH, delta, cell)) continue;
                cellDecided++;
                const double probes[4] = {edges[e][0], edges[e][1], (e ? 1.0 : -1.0) * exact,
                                          edges[e][0] + uniform() * (edges[e][1] - edges[e][0])};
                for (double s : probes) {
                    if (doubleCell(c, s, origin, h) != cell) {
                        if (cellBad < 5)
                            std::printf("cell mismatch: c %a s %a origin %a h %a float %lld double %lld\n", c, s,
                                        origin, h, (long long)cell, (long long)doubleCell(c, s, origin, h));
                        cellBad++;
                    }
                }
            }
        }
    }
    // samples: the float test of a box against the double evaluation
    long samples = 0, sampleDecided = 0, sampleBad = 0;
    const long gaussians = cases / 20 + 1;
    for (long n = 0; n < gaussians; n++) {
        double v[4], len = 0;
        for (int k = 0; k < 4; k++) {
            v[k] = uniform() * 2 - 1;
            len += v[k] * v[k];
        }
        len = std::sqrt(len);
        float q[4];
        for (int k = 0; k < 4; k++) q[k] = float(v[k] / len);
        float col[9];
        frameInDouble(q[0], q[1], q[2], q[3], col);
        // a grid: h, origin; tiny h now and then takes the double-summed bound
        const double h = (next() % 16 == 0) ? 1e-10 * (1 + uniform()) : std::exp(std::log(1e-4) + uniform() * std::log(1e2));
        bounds::GridView g{};
        for (int a = 0; a < 3; a++) {
            g.dims[a] = 400;
            g.origin[a] = (uniform() * 2 - 1) * 0.5;
        }
        g.h = h;
        const float invH = float(1.0 / h);
        g.invH = invH >= 0x1p-40f && invH <= 0x1p40f ? invH : 0.0f;
        g.hF = float(h);
        g.floatBound = h >= 0x1p-30 && h <= 0x1p30;
        for (int a = 0; a < 3; a++) {
            g.originF[a] = float(g.origin[a]);
            g.originMag[a] = std::fmax(std::fabs(g.originF[a]), 0x1p-100f);
            g.floatBound = g.floatBound && std::fabs(g.origin[a]) <= 0x1p40;
        }
        g.cells = 400u * 400u * 400u;
        // the centre at a random place; the radii chosen so the surface
        // passes within a few ulps of a sample point half the time
        float cf[3];
        double c[3];
        for (int a = 0; a < 3; a++) {
            cf[a] = float(g.origin[a] + (50 + uniform() * 300) * h);
            c[a] = cf[a];
        }
        const double sigma = 2.0;
        float scale[3];
        for (int a = 0; a < 3; a++) scale[a] = float(h * (0.3 + uniform() * 1.5) / sigma);
        bounds::Ellipsoid e;
        for (int qq = 0; qq < 9; qq++) e.col[qq] = col[qq];
        for (int a = 0; a < 3; a++) e.radius[a] = sigma * double(scale[a]);
        bounds::Box b;
        for (int a = 0; a < 3; a++) {
            const double half = bounds::hypotV8(e.col[a] * e.radius[0], e.col[3 + a] * e.radius[1], e.col[6 + a] * e.radius[2]);
            b.lo[a] = int64_t(std::floor(((c[a] - half) - g.origin[a]) / h));
            b.hi[a] = int64_t(std::floor(((c[a] + half) - g.origin[a]) / h));
        }
        if (next() % 2) {
            // scale the ellipsoid so its surface meets one sample exactly
            // (the sum there 1 up to rounding), then nudge by a few ulps
            const int64_t i = b.lo[0] + int64_t(next() % uint64_t(b.extent(0)));
            const int64_t j = b.lo[1] + int64_t(next() % uint64_t(b.extent(1)));
            const int64_t k = b.lo[2] + int64_t(next() % uint64_t(b.extent(2)));
            double ox, oy, oz;
            bounds::sampleOffset(int(next() % 9), ox, oy, oz);
            const double d[3] = {g.origin[0] + (double(i) + ox) * h - c[0], g.origin[1] + (double(j) + oy) * h - c[1],
                                 g.origin[2] + (double(k) + oz) * h - c[2]};
            double sum = 0;
            for (int a = 0; a < 3; a++) {
                const double t = (e.col[3 * a] * d[0] + e.col[3 * a + 1] * d[1] + e.col[3 * a + 2] * d[2]) / e.radius[a];
                sum += t * t;
            }
            if (sum > 0) {
                const double f = std::sqrt(sum) * (1 + (uniform() * 2 - 1) * 1e-7);
                for (int a = 0; a < 3; a++) {
                    scale[a] = float(scale[a] * f);
                    e.radius[a] = sigma * double(scale[a]);
                }
            }
        }
        bounds::FloatTest f;
        const bool fast = bounds::floatTestInFloat(g, b, c, cf, col, sigma, float(sigma), scale, f);
        if (!fast) continue;
        for (int64_t k = b.lo[2]; k <= b.hi[2]; k++)
            for (int64_t j = b.lo[1]; j <= b.hi[1]; j++)
                for (int64_t i = b.lo[0]; i <= b.hi[0]; i++)
                    for (int sIdx = 0; sIdx < 9; sIdx++) {
                        double ox, oy, oz;
                        bounds::sampleOffset(sIdx, ox, oy, oz);
                        const int got = bounds::floatSample(f, float(i - b.lo[0]) + float(ox), float(j - b.lo[1]) + float(oy),
                                                            float(k - b.lo[2]) + float(oz));
                        samples++;
                        if (got < 0) continue;
                        sampleDecided++;
                        const bool want = bounds::sampleInside(g, i, j, k, sIdx, c, e);
                        if ((got == 1) != want) {
                            if (sampleBad < 5) std::printf("sample mismatch: float %d double %d\n", got, int(want));
                            sampleBad++;
                        }
                    }
    }
    std::printf("reach checked %ld bad %ld; cells tried %ld decided %ld bad %ld; samples %ld decided %ld bad %ld\n",
                reachChecked, reachBad, cellTried, cellDecided, cellBad, samples, sampleDecided, sampleBad);
    return reachBad || cellBad || sampleBad ? 1 : 0;
}
