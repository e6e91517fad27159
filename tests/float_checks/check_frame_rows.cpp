// Checks vsim::frame::rowsInFloat (csrc/frame_rows.cuh) against the double
// formula of mat3.js:71-87 followed by a float32 rounding, bit for bit, on
// random unit and non-unit quaternions and on special values. Prints the
// cases, the certified share and the mismatches; exits 1 on any mismatch.
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <cstdlib>

#include "frame_rows.cuh"

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next() {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}
static double uniform() { return double(next() >> 11) * 0x1p-53; }

static void reference(float x, float y, float z, float w, float col[9]) {
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

int main(int argc, char** argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 2000000;
    const float specials[] = {0.0f, -0.0f, 1.0f, -1.0f, 0.5f, -0.5f, 0.70710677f, 1e-30f, -1e-30f,
                              1e-10f, 3e-19f, 1e30f, 2.0f, 0x1p-24f, 1.0f - 0x1p-24f, 0.25f, 0.75f};
    const int ns = sizeof specials / sizeof specials[0];
    long certified = 0, mismatches = 0, total = 0;
    for (long n = 0; n < cases; n++) {
        float q[4];
        const int kind = int(next() % 8);
        if (kind < 4) {  // unit quaternion
            double v[4], len = 0;
            for (int k = 0; k < 4; k++) {
                v[k] = uniform() * 2 - 1;
                len += v[k] * v[k];
            }
            len = __builtin_sqrt(len);
            for (int k = 0; k < 4; k++) q[k] = float(v[k] / len);
        } else if (kind < 6) {  // unnormalised, scale 2^-20 .. 2^20
            const double scale = __builtin_ldexp(1.0, int(next() % 41) - 20);
            for (int k = 0; k < 4; k++) q[k] = float((uniform() * 2 - 1) * scale);
        } else {  // specials mixed with random components
            for (int k = 0; k < 4; k++) q[k] = (next() & 1) ? specials[next() % ns] : float(uniform() * 2 - 1);
        }
        float got[9], want[9];
        reference(q[0], q[1], q[2], q[3], want);
        total++;
        if (!vsim::frame::rowsInFloat(q[0], q[1], q[2], q[3], got)) continue;
        certified++;
        if (std::memcmp(got, want, sizeof got) != 0) {
            if (mismatches < 10)
                std::printf("mismatch q=(%a %a %a %a)\n", q[0], q[1], q[2], q[3]);
            mismatches++;
        }
    }
    std::printf("cases %ld certified %ld (%.5f) mismatches %ld\n", total, certified, double(certified) / total, mismatches);
    return mismatches ? 1 : 0;
}
