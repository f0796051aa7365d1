// Checks the integer FP64 -> FP32 rounding of fjsph_gb300/csrc/split.cuh against the compiler's
// conversions: hi = (float)x and lo = (float)(x - (double)hi), bit for bit, over random doubles of
// every exponent, both signs, rounding ties and the carry into the exponent; and the FP32 -> FP64
// widening over every FP32 bit pattern.  Exit status 0 on
// agreement; prints the first mismatch otherwise.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>

#include "../../fjsph_gb300/csrc/split.cuh"

static uint32_t fbits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}
static double dfrom(uint64_t u) {
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

static int check(double x) {
    float h, l;
    fjsph::split_f32(x, h, l);
    const float h0 = (float)x;
    const float l0 = (float)(x - (double)h0);
    const float t = fjsph::to_f32(x);
    if (fbits(h) != fbits(h0) || fbits(l) != fbits(l0) || fbits(t) != fbits(h0)) {
        if (h0 != h0 && h != h) return 0; /* NaN payloads */
        std::printf("mismatch x=%.17g hi %08x/%08x lo %08x/%08x to_f32 %08x\n", x, fbits(h), fbits(h0), fbits(l),
                    fbits(l0), fbits(t));
        return 1;
    }
    return 0;
}

static int check_widen(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    const double w = fjsph::to_f64(f), w0 = (double)f;
    uint64_t u, u0;
    std::memcpy(&u, &w, 8);
    std::memcpy(&u0, &w0, 8);
    if (u != u0) {
        if (w0 != w0 && w != w) return 0; /* NaN payloads */
        std::printf("widen mismatch bits=%08x %016llx/%016llx\n", b, (unsigned long long)u, (unsigned long long)u0);
        return 1;
    }
    return 0;
}

int main() {
    std::mt19937_64 rng(12345);
    long bad = 0, n = 0;
    /* every FP32 bit pattern, widened */
    for (uint64_t b = 0; b <= 0xFFFFFFFFull; b += 1) {
        bad += check_widen((uint32_t)b);
        if (bad > 5) return 1;
    }
    for (int e = 0; e < 2048; ++e) {
        for (int k = 0; k < 4000; ++k) {
            uint64_t m = rng() & 0xFFFFFFFFFFFFFull;
            if (k % 8 == 1) m = (m & ~0x1FFFFFFFull) | 0x10000000ull; /* exact tie */
            if (k % 8 == 2) m = 0xFFFFFFFFFFFFFull;                    /* carry into the exponent */
            if (k % 8 == 3) m = (m & ~0x1FFFFFFFull) | 0x0FFFFFFFull;  /* just below the tie */
            if (k % 8 == 4) m = (m & ~0x1FFFFFFFull) | 0x10000001ull;  /* just above the tie */
            if (k % 8 == 5) m = m & ~0x1FFFFFFFull;                    /* exactly representable */
            for (int s = 0; s < 2; ++s) {
                const uint64_t u = ((uint64_t)s << 63) | ((uint64_t)e << 52) | m;
                bad += check(dfrom(u));
                ++n;
                if (bad > 5) return 1;
            }
        }
    }
    bad += check(0.0) + check(-0.0) + check(1e-320) + check(3.4028235677973366e38) + check(-3.4028235677973366e38);
    std::printf("%ld values, %ld mismatches\n", n, bad);
    return bad ? 1 : 0;
}
