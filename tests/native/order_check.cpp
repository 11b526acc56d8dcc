// The coherent sky sample order (dl_host.cpp): a permutation of 0 .. n-1 whose consecutive
// groups of 16 fall in one 4 x 4 block of the (0, m, 2)-net's cells. Built and run by
// tests/test_math_paths.py.
#include <cstdio>
#include <vector>

#include "dl_host.hpp"

int main() {
    int failures = 0;
    for (uint32_t n : {16u, 64u, 256u, 1024u, 4096u}) {
        std::vector<uint16_t> order = dl::sky_sample_order(n);
        std::vector<int> seen(n, 0);
        for (uint16_t j : order) ++seen[j];
        for (uint32_t j = 0; j < n; ++j) failures += seen[j] != 1;
        uint32_t m = 0;
        while ((1u << m) < n) ++m;
        uint32_t px = (m + 1) / 2, py = m / 2;
        for (uint32_t g = 0; g + 16 <= n; g += 16) {
            uint32_t x0 = ~0u, x1 = 0, y0 = ~0u, y1 = 0;
            for (uint32_t k = g; k < g + 16; ++k) {
                uint32_t j = order[k];
                uint32_t cx = dl::rev_bits(j) >> (32 - px), cy = dl::sobol2(j) >> (32 - py);
                x0 = cx < x0 ? cx : x0; x1 = cx > x1 ? cx : x1;
                y0 = cy < y0 ? cy : y0; y1 = cy > y1 ? cy : y1;
            }
            failures += (x1 - x0 > 3) || (y1 - y0 > 3);
        }
    }
    failures += !dl::sky_sample_order(100).empty() + !dl::sky_sample_order(8).empty();
    std::printf("order failures %d\n", failures);
    return failures ? 1 : 0;
}
