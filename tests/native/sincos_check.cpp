// Compares the library's sin/cos, sin alone and acos (binary32 double-float paths + rounding
// test, falling back to binary64) with the binary64 paths alone over many arguments; prints
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

    // acos: the double-float path against acos_d over [-1, 1]: uniform arguments, arguments near
    // -1, -1/2, 1/2 and 1, and arbitrary bit patterns of magnitude below 1
    unsigned long long amismatch = 0, afallback = 0;
    for (unsigned long long i = 0; i < n; ++i) {
        state = dl::splitmix64(state);
        double u = (state >> 11) * (1.0 / 9007199254740992.0);
        float x;
        switch (i % 4) {
            case 0: x = (float)(u * 2.0 - 1.0); break;
            case 1: {
                const float centers[4] = {-1.0f, -0.5f, 0.5f, 1.0f};
                x = centers[(state >> 3) & 3] + (float)((u - 0.5) * 1e-3);
                if (x > 1.0f) x = 1.0f;
                if (x < -1.0f) x = -1.0f;
                break;
            }
            case 2: x = 1.0f - (float)(u * u * u * 1e-2); break;
            default: {
                uint32_t bits = ((uint32_t)(state >> 32) & 0x3F7FFFFFu) | ((uint32_t)(state & 1u) << 31);
                std::memcpy(&x, &bits, 4);
            }
        }
        float fast = dl::acos_f(x), ref = dl::acos_d(x);
        if (std::memcmp(&fast, &ref, 4)) {
            if (amismatch < 10) std::printf("acos mismatch x=%a fast=%a b64=%a\n", x, fast, ref);
            ++amismatch;
        }
        // count fallbacks by re-running the double-float evaluation and its test
        float a = fabsf(x), t = (1.0f - a) * 0.5f, out;
        dl::FF r;
        if (a <= 0.5f) {
            r = dl::ff_add(dl::FF{1.5707963705062866f, -4.371138828673793e-08f},
                           dl::ff_neg(dl::ff_asin_poly(dl::FF{x, 0.0f})));
        } else if (t == 0.0f) {
            continue;  // +-1: exact constants
        } else {
            float sq = sqrtf(t);
            dl::FF as = dl::ff_asin_poly(dl::ff_fast_sum(sq, fmaf(-sq, sq, t) / (sq + sq)));
            dl::FF twice{as.h + as.h, as.l + as.l};
            r = x > 0.0f ? twice : dl::ff_add(dl::FF{3.1415927410125732f, -8.742277657347586e-08f}, dl::ff_neg(twice));
        }
        if (!dl::ff_rounds_to(r, out)) ++afallback;
    }
    std::printf("acos checked %llu mismatches %llu binary64_fallbacks %llu\n", n, amismatch, afallback);
    return mismatch || amismatch ? 1 : 0;
}
