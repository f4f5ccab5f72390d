// Checks the integer emulations of atag_device.cuh against the operations
// they replace, bit for bit, on the host:
//   * hypot_f against the FP64 formula: random significands at every
//     exponent difference, integer-valued inputs (the int64 conversions of
//     fit_line), Pythagorean triples (exact roots) and constructed half-way
//     cases (roots that are float midpoints);
//   * i64_to_f32_rn / u64_to_f32_rn against C++ conversions: random values
//     of every bit length, values next to rounding boundaries and ties.
// Prints "<cases> <mismatches>" and exits non-zero on a mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../sycl-apriltag-test_gb300/csrc/atag_device.cuh"

using atag::hypot_f;
using atag::hypot_f_fp64;
using atag::i64_to_f32_rn;
using atag::u2f;
using atag::u64_to_f32_rn;

static unsigned long long g_state = 0x9E3779B97F4A7C15ull;
static unsigned long long rnd() {
    g_state ^= g_state << 13;
    g_state ^= g_state >> 7;
    g_state ^= g_state << 17;
    return g_state;
}

static long long cases = 0, bad = 0;
static void check_conv(long long v) {
    cases += 2;
    float g = i64_to_f32_rn(v), w = (float)v;
    if (memcmp(&g, &w, 4) != 0) {
        if (bad < 10) printf("mismatch i64 %lld got=%a want=%a\n", v, g, w);
        bad++;
    }
    unsigned long long u = (unsigned long long)v;
    g = u64_to_f32_rn(u);
    w = (float)u;
    if (memcmp(&g, &w, 4) != 0) {
        if (bad < 10) printf("mismatch u64 %llu got=%a want=%a\n", u, g, w);
        bad++;
    }
}
static void check(float a, float b) {
    cases++;
    float g = hypot_f(a, b), w = hypot_f_fp64(a, b);
    uint32_t gu, wu;
    memcpy(&gu, &g, 4);
    memcpy(&wu, &w, 4);
    if (gu != wu) {
        if (bad < 10) printf("mismatch a=%a b=%a got=%a want=%a\n", a, b, g, w);
        bad++;
    }
}

int main(int argc, char** argv) {
    long long n = argc > 1 ? atoll(argv[1]) : 2000000;
    // random significands, exponent differences 0..70, both orders and signs
    for (long long i = 0; i < n; i++) {
        unsigned long long r = rnd();
        uint32_t ea = 60 + (uint32_t)(r % 120), diff = (uint32_t)((r >> 8) % 71);
        uint32_t eb = ea > diff ? ea - diff : 1;
        uint32_t ua = (ea << 23) | (uint32_t)(rnd() & 0x7FFFFF), ub = (eb << 23) | (uint32_t)(rnd() & 0x7FFFFF);
        if (r & (1ull << 40)) ua |= 0x80000000u;
        if (r & (1ull << 41)) ub |= 0x80000000u;
        check(u2f(ua), u2f(ub));
        check(u2f(ub), u2f(ua));
    }
    // integer-valued inputs as produced by (float)int64 in fit_line
    for (long long i = 0; i < n; i++) {
        int sh = (int)(rnd() % 63);
        long long x = (long long)(rnd() >> (sh + 1)), y = (long long)(rnd() >> (rnd() % 64));
        if (rnd() & 1) x = -x;
        check((float)x, (float)y);
        check((float)(x % 100000), (float)(y % 1000));
    }
    // small integers exhaustively
    for (int x = 0; x < 1500; x++)
        for (int y = 0; y < 1500; y++) check((float)x, (float)y);
    // Pythagorean triples (exact roots), scaled
    for (long long m = 2; m < 3000; m++)
        for (long long k = 1; k < m; k += 7) {
            long long a = m * m - k * k, b = 2 * m * k;
            check((float)a, (float)b);
            check((float)a * 0x1p-40f, (float)b * 0x1p-40f);
        }
    // exact roots that are float half-way points: primitive triples
    // (m^2 - n^2, 2mn, m^2 + n^2) with an odd 25-bit hypotenuse and legs
    // below 2^24 (ties, rounded to even)
    long long ties = 0;
    for (long long m = 2900; m < 4200; m++)
        for (long long k = 1 + (m & 1); k < m; k += 2) {
            long long a = m * m - k * k, b = 2 * m * k, c = m * m + k * k;
            if (c <= (1ll << 24) || c >= (1ll << 25) || a >= (1ll << 24) || b >= (1ll << 24)) continue;
            check((float)a, (float)b);
            check((float)b * 0x1p-30f, (float)a * 0x1p-30f);
            ties++;
        }
    if (ties < 1000) {
        printf("too few half-way cases: %lld\n", ties);
        return 2;
    }
    // roots at float half-way points: c = odd 25-bit, c^2 = a^2 + b^2 with
    // a = c^2 - 1 split as (c^2-1) = (a-b)(a+b) is rare, so instead take
    // a just below c and b = sqrt(c^2 - a^2) when that is an integer
    for (long long c = (1ll << 24) + 1; c < (1ll << 24) + 200001; c += 2) {
        long long c2 = c * c;
        for (long long a = c - 1; a > c - 40; a--) {
            long long b2 = c2 - a * a;
            long long b = (long long)__builtin_sqrt((double)b2);
            while (b * b > b2) b--;
            while ((b + 1) * (b + 1) <= b2) b++;
            if (b * b == b2 && a < (1ll << 24) && b < (1ll << 24)) check((float)a, (float)b);
            // neighbours of the tie
            check((float)a, (float)b + 1.0f);
        }
    }
    // 64-bit integer conversions
    for (long long i = 0; i < n; i++) {
        unsigned long long r = rnd();
        check_conv((long long)(r >> (rnd() % 64)));
        check_conv(-(long long)(r >> (1 + rnd() % 63)));
    }
    for (int L = 0; L < 64; L++)
        for (long long d = -3; d <= 3; d++) {
            unsigned long long b = 1ull << L;
            check_conv((long long)(b + d));
            for (int k = 1; k < 40 && k < L; k++) {
                unsigned long long t = b | (1ull << (k - 1)) | (rnd() & ((1ull << (k - 1)) - 1));
                check_conv((long long)(t + d));
                check_conv((long long)((b | (1ull << (k - 1))) + d));  // exact ties at bit k-1
            }
        }
    check_conv(0);
    check_conv((long long)0x8000000000000000ull);
    check_conv(0x7FFFFFFFFFFFFFFFll);
    printf("%lld %lld\n", cases, bad);
    return bad ? 1 : 0;
}
