// Compares the library's sin/cos and sin alone (binary32 double-float paths + rounding test,
// falling back to binary64) with the binary64 paths alone over many arguments; prints
// mismatches and the share of arguments that needed the binary64 path. Built and run by tests/test_math_paths.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "dl_math.cuh"

int main(int argc, char **argv) {
    unsigned long long n = argc > 1 ? strtoull(argv[1], nullptr, 10) : 1000000ull;
    unsigned long long mismatch = 0, fallback = 0;
    uint64_t state = 12345;
    for (unsigned long long i = 0; i < n; ++i) {
        state = dl::splitmix64(state);
        float x;
        switch (i % 4) {
            case 0: x = (float)((state >> 40) * (1.0 / 16777216.0)) * 6.2831855f; break;        // [0, tau)
            case 1: x = (float)((state >> 40) * (1.0 / 16777216.0)) * 3.1415927f - 0.78539819f; break;
            case 2: x = (float)((state >> 40) * (1.0 / 16777216.0)) * 16.0f - 8.0f; break;
            default: {
                // any bit pattern with a magnitude in [2^-20, 8), either sign
                uint32_t mant = (uint32_t)(state >> 41) & 0x7FFFFFu;
                uint32_t ex = 107u + (uint32_t)((state >> 20) % 23u);  // exponents -20 .. 2
                uint32_t bits = (ex << 23) | mant | ((uint32_t)(state & 1u) << 31);
                std::memcpy(&x, &bits, 4);
            }
        }
        float s, c;
        dl::sincos_f(x, s, c);
        double sd, cd;
        dl::sincos_d((double)x, sd, cd);
        float s64 = (float)sd, c64 = (float)cd;
        if (std::memcmp(&s, &s64, 4) || std::memcmp(&c, &c64, 4)) {
            if (mismatch < 10) std::printf("mismatch x=%a fast=(%a,%a) b64=(%a,%a)\n", x, s, c, s64, c64);
            ++mismatch;
        }
        float s_only = dl::sin_f(x);  // the sin-only path
        if (std::memcmp(&s_only, &s64, 4)) {
            if (mismatch < 10) std::printf("sin mismatch x=%a fast=%a b64=%a\n", x, s_only, s64);
            ++mismatch;
        }
        // count fallbacks by re-running the fast path's reduction and test
        float k = rintf(x * 0.6366197466850281f);
        dl::FF r = dl::ff_two_sum(x - k * dl::kPio2F1, -(k * dl::kPio2F2));
        r = dl::ff_fast_sum(r.h, r.l - k * dl::kPio2F3);
        dl::FF sv, cv;
        dl::ff_sincos_poly(r, sv, cv);
        float t;
        if ((k != 0.0f && fabsf(r.h) <= 1.52587890625e-05f) || !dl::ff_rounds_to(sv, t) || !dl::ff_rounds_to(cv, t)) ++fallback;
    }
    std::printf("checked %llu mismatches %llu binary64_fallbacks %llu\n", n, mismatch, fallback);

    return mismatch ? 1 : 0;
}
