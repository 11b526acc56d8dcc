// The coherent sky sample order (dl_host.cpp): a permutation of 0 .. n-1 whose consecutive
// groups of 16 fall in one 4 x 4 block of the (0, m, 2)-net's cells; and its shift-aligned form
// (sample_cells). Built and run by tests/test_math_paths.py.
#include <cstdio>
#include <vector>

#include "dl_host.hpp"

// The reference's loop for the second coordinate (spread.rs:43-53), against the library's
// closed form.
static uint32_t sobol2_loop(uint32_t index) {
    uint32_t value = 0, dir = 1u << 31;
    for (; index != 0; index >>= 1, dir ^= dir >> 1)
        if (index & 1u) value ^= dir;
    return value;
}

int main() {
    int failures = 0;
    for (uint64_t i = 0; i < (1ull << 32); i += i < (1u << 22) ? 1 : 4099)
        failures += dl::sobol2((uint32_t)i) != sobol2_loop((uint32_t)i);
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
    // the shift-aligned order (dl::sample_cells, used as the device's shifted_sample): for any
    // shift a permutation, rank r's shifted point in cell r or the next on each axis
    uint64_t state = 0x9E3779B97F4A7C15ull;
    auto next_unit = [&state] {
        state = state * 6364136223846793005ull + 1442695040888963407ull;
        return (float)(uint32_t)(state >> 40) * (1.0f / 16777216.0f);
    };
    for (uint32_t n : {16u, 32u, 128u, 256u, 2048u, 4096u}) {
        dl::SampleCells c = dl::sample_cells(n);
        uint32_t m = 0;
        while ((1u << m) < n) ++m;
        const uint32_t xb = (m + 1) / 2, yb = m / 2, nx = 1u << xb, ny = 1u << yb;
        std::vector<int> cell_seen(n, 0);
        for (uint16_t j : c.samples) ++cell_seen[j];
        for (uint32_t j = 0; j < n; ++j) failures += cell_seen[j] != 1;
        for (int trial = 0; trial < 64; ++trial) {
            float ox = trial == 0 ? 0.0f : next_unit(), oy = trial == 0 ? 0.999999f : next_unit();
            uint32_t sx = (uint32_t)(ox * (float)nx), sy = (uint32_t)(oy * (float)ny);
            sx = sx < nx - 1 ? sx : nx - 1;
            sy = sy < ny - 1 ? sy : ny - 1;
            std::vector<int> seen(n, 0);
            for (uint32_t r = 0; r < n; ++r) {
                uint32_t cx = c.cells[r] & 0xFFu, cy = c.cells[r] >> 8;
                uint32_t j = c.samples[((cy - sy) & (ny - 1)) << xb | ((cx - sx) & (nx - 1))];
                ++seen[j];
                dl::f2 p = dl::spread(j, dl::f2{ox, oy}, true);
                uint32_t px = (uint32_t)(p.x * (float)nx), py = (uint32_t)(p.y * (float)ny);
                failures += ((px - cx) & (nx - 1)) > 1 || ((py - cy) & (ny - 1)) > 1;
            }
            for (uint32_t j = 0; j < n; ++j) failures += seen[j] != 1;
        }
    }
    failures += !dl::sample_cells(100).cells.empty();
    std::printf("order failures %d\n", failures);
    return failures ? 1 : 0;
}
