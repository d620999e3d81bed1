// CPU check of the shuffled two-block tensor-core pass (fused_tc.cu): for
// random tile geometries, tc_shuffle_layout's row layouts and swaps,
// replayed on tile coordinates exactly as the kernel's warp shuffles move
// registers, leave every thread (row) holding the second block's row in the
// second block's gate order (its jgate table), and each tile coordinate once.
// Exit status 1 on any failure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/kernels.h"

using namespace q1g;

int main()
{
    std::mt19937 rng(7);
    int bad = 0, tried = 0, laid = 0;
    for (int trial = 0; trial < 4000; ++trial) {
        // two blocks of five gate bits among the 12 tile bits, overlapping
        // in 0..4 bits (their union at most 10)
        std::vector<int> all(12);
        for (int j = 0; j < 12; ++j) all[j] = j;
        std::shuffle(all.begin(), all.end(), rng);
        const int overlap = (int)(rng() % 5);
        std::vector<int> g0(all.begin(), all.begin() + 5), g1;
        for (int i = 0; i < overlap; ++i) g1.push_back(g0[i]);
        for (int j = 5; (int)g1.size() < 5; ++j) g1.push_back(all[j]);
        std::shuffle(g0.begin(), g0.end(), rng);
        std::shuffle(g1.begin(), g1.end(), rng);
        TcBlockGeom b0{}, b1{};
        for (int g = 0; g < 32; ++g) {
            uint32_t c0 = 0, c1 = 0;
            for (int k = 0; k < 5; ++k)
                if ((g >> k) & 1) {
                    c0 |= 1u << g0[k];
                    c1 |= 1u << g1[k];
                }
            b0.jgate[g] = c0;
            b1.jgate[g] = c1;
        }
        int32_t swap_lane[5];
        int reg1[5];
        ++tried;
        if (!tc_shuffle_layout(b0, b1, swap_lane, reg1)) {
            ++bad;
            continue;
        }
        ++laid;
        auto rowc = [](const TcBlockGeom& b, int t) {
            uint32_t c = 0;
            for (int r = 0; r < 7; ++r)
                if ((t >> r) & 1) c |= b.jrow_bit[r];
            return c;
        };
        // x[t][j]: the tile coordinate thread t holds in register j
        std::vector<std::vector<uint32_t>> x(128, std::vector<uint32_t>(32));
        for (int t = 0; t < 128; ++t)
            for (int j = 0; j < 32; ++j) x[t][j] = rowc(b0, t) | b0.jgate[j];
        for (int a = 0; a < 5; ++a) {
            const int bl = swap_lane[a];
            if (bl < 0) continue;
            std::vector<std::vector<uint32_t>> y = x;
            for (int t = 0; t < 128; ++t) {
                const int lane = t & 31, partner = t ^ (1 << bl);
                const bool up = (lane >> bl) & 1;
                for (int j = 0; j < 32; ++j) {
                    if (j & (1 << a)) continue;
                    const int j1 = j | (1 << a);
                    // what the partner sends: its x[j] if it is up, else its x[j1]
                    const bool pup = ((partner & 31) >> bl) & 1;
                    const uint32_t got = pup ? x[partner][j] : x[partner][j1];
                    if (up) y[t][j] = got;
                    else y[t][j1] = got;
                }
            }
            x = y;
        }
        std::vector<int> seen(4096, 0);
        for (int t = 0; t < 128; ++t)
            for (int j = 0; j < 32; ++j) {
                if (x[t][j] != (rowc(b1, t) | b1.jgate[j])) ++bad;
                if (x[t][j] < 4096) ++seen[x[t][j]];
            }
        for (int c = 0; c < 4096; ++c)
            if (seen[c] != 1) ++bad;
        // block 1's register order is the gate order of its image
        for (int k = 0; k < 5; ++k)
            if (b1.jgate[1 << k] != 1u << reg1[k]) ++bad;
    }
    std::printf("bad %d tried %d laid %d\n", bad, tried, laid);
    return bad ? 1 : 0;
}
