// The library's acos_approx (dl_math.cuh, the angle of the bounce gather's slerp) against the
// oracle's restatement of glam's acos_approx, bit for bit, over every binary32 in [-1, 1] with a
// stride, plus the neighbourhoods of -1, 0 and 1. Built and run by tests/test_math_paths.py.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "dl_math.cuh"
#include "oracle_bounce.hpp"

int main() {
    unsigned long long checked = 0, mismatch = 0;
    auto check = [&](float x) {
        float a = dl::acos_approx(x), b = oracle::acos_approx(x);
        ++checked;
        if (std::memcmp(&a, &b, 4)) {
            if (mismatch < 10) std::printf("mismatch x=%a lib=%a oracle=%a\n", x, a, b);
            ++mismatch;
        }
    };
    // magnitudes 0 .. 1 (bit patterns 0 .. 0x3F800000), both signs
    for (uint32_t bits = 0; bits <= 0x3F800000u; bits += 61) {
        float x;
        std::memcpy(&x, &bits, 4);
        check(x);
        check(-x);
    }
    for (uint32_t k = 0; k < 100000; ++k) {
        uint32_t one = 0x3F800000u - k, zero = k;
        float x, z;
        std::memcpy(&x, &one, 4);
        std::memcpy(&z, &zero, 4);
        check(x);
        check(-x);
        check(z);
        check(-z);
    }
    std::printf("acos_approx checked %llu mismatches %llu\n", checked, mismatch);
    return mismatch ? 1 : 0;
}
