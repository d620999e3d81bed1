// CPU check of the swap-run pass layout (swap_run_layout in libq1gpu.so):
// the kernel's steps are replayed on the host on states of 10 to 14 qubits
// for random sets of disjoint swaps, and the result must be the direct
// permutation out[pi(i)] = in[i] (every amplitude written once).  The
// staged offsets of the copies fill each stage once, and the permuted reads
// of one phase of a warp (16 lanes of 8 bytes, 8 lanes of 16 bytes) hit
// distinct bank groups.  Prints "bad <count> ..."; exit status 1 on any
// failure.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/kernels.h"

using namespace q1g;

int main()
{
    std::mt19937 rng(11);
    long bad = 0, layouts = 0;
    for (int trial = 0; trial < 400; ++trial) {
        const int nbits = 10 + (int)(rng() % 5);
        const int amp_bytes = (trial % 2) ? 16 : 8, C = amp_bytes == 8 ? 4 : 3;
        // random disjoint pairs, often including the lowest and highest positions
        std::vector<int> pos(nbits);
        for (int p = 0; p < nbits; ++p) pos[p] = p;
        std::shuffle(pos.begin(), pos.end(), rng);
        if (trial % 3 == 0)   // the QFT pattern: p <-> nbits-1-p
            for (int p = 0; p < nbits; ++p) pos[p] = p < nbits / 2 ? p : nbits - 1 - (p - nbits / 2);
        const int npairs = trial % 3 == 0 ? nbits / 2 : 1 + (int)(rng() % (nbits / 2));
        std::vector<int> pa, pb;
        for (int k = 0; k < npairs; ++k) {
            if (trial % 3 == 0) {
                pa.push_back(k);
                pb.push_back(nbits - 1 - k);
            } else {
                pa.push_back(pos[2 * k]);
                pb.push_back(pos[2 * k + 1]);
            }
        }
        auto tp = std::make_unique<SwapTile>();
        SwapTile& t = *tp;
        if (!swap_run_layout(t, pa.data(), pb.data(), npairs, nbits, amp_bytes)) {
            continue;   // no tile closed under the swaps: the plan applies them one by one
        }
        ++layouts;
        int perm[64];
        for (int p = 0; p < 64; ++p) perm[p] = p;
        for (int k = 0; k < npairs; ++k) {
            perm[pa[k]] = pb[k];
            perm[pb[k]] = pa[k];
        }
        auto pi = [&](uint64_t i) {
            uint64_t r = 0;
            for (int p = 0; p < nbits; ++p)
                if ((i >> p) & 1) r |= uint64_t(1) << perm[p];
            return r;
        };
        const uint64_t N = uint64_t(1) << nbits;
        std::vector<uint64_t> in(N), out(N, ~uint64_t(0)), expect(N);
        for (uint64_t i = 0; i < N; ++i) in[i] = i * 2654435761u + 7;
        for (uint64_t i = 0; i < N; ++i) expect[pi(i)] = in[i];
        std::vector<int> writes(N, 0);
        // stage offsets fill the stage once
        std::vector<int> seen(1024, 0);
        for (int l = 0; l < 1024; ++l) {
            if (t.wphys[l] >= 1024 || t.rphys[l] >= 1024) ++bad;
            else ++seen[t.wphys[l]];
        }
        for (int l = 0; l < 1024; ++l)
            if (seen[l] != 1) ++bad;
        // permuted reads and copies of one phase: distinct bank groups
        const int phase = 1 << C;
        for (int m = 0; m < 32; ++m)
            for (int h = 0; h < 32 / phase; ++h) {
                uint32_t rc = 0, wc = 0;
                for (int l = phase * h; l < phase * h + phase; ++l) {
                    rc |= 1u << (t.rphys[32 * m + l] & (phase - 1));
                    wc |= 1u << (t.wphys[32 * m + l] & (phase - 1));
                }
                if (rc != (1u << phase) - 1 || wc != (1u << phase) - 1) ++bad;
            }
        // replay the kernel over all tiles
        const uint64_t tiles = N >> 10;
        std::vector<uint64_t> A(1024), Bv(1024);
        for (uint64_t ti = 0; ti < tiles; ++ti) {
            const uint64_t base = expand_index(ti, t.tile_map);
            uint64_t base2 = base;
            for (int k = 0; k < t.nouter; ++k)
                if (((base >> t.pa[k]) ^ (base >> t.pb[k])) & 1)
                    base2 ^= (uint64_t(1) << t.pa[k]) | (uint64_t(1) << t.pb[k]);
            if (base2 < base) continue;
            const bool two = base2 != base;
            for (int m = 0; m < 32; ++m) {
                uint64_t g = 0;
                for (int b = 0; b < 5; ++b)
                    if ((m >> b) & 1) g |= t.gbit[b];
                for (int lane = 0; lane < 32; ++lane) {
                    if (base + g + lane >= N || base2 + g + lane >= N) {
                        ++bad;
                        continue;
                    }
                    A[t.wphys[32 * m + lane]] = in[base + g + lane];
                    if (two) Bv[t.wphys[32 * m + lane]] = in[base2 + g + lane];
                }
            }
            for (int m = 0; m < 32; ++m) {
                uint64_t g = 0;
                for (int b = 0; b < 5; ++b)
                    if ((m >> b) & 1) g |= t.gbit[b];
                for (int lane = 0; lane < 32; ++lane) {
                    const uint32_t r = t.rphys[32 * m + lane];
                    out[base2 + g + lane] = A[r];
                    ++writes[base2 + g + lane];
                    if (two) {
                        out[base + g + lane] = Bv[r];
                        ++writes[base + g + lane];
                    }
                }
            }
        }
        for (uint64_t i = 0; i < N; ++i)
            if (writes[i] != 1 || out[i] != expect[i]) ++bad;
    }
    // fewer than 10 qubits, or pairs that are not disjoint: no layout
    auto tp = std::make_unique<SwapTile>();
    const int a1[2] = {0, 1}, b1[2] = {5, 5};
    if (swap_run_layout(*tp, a1, b1, 2, 12, 8)) ++bad;
    const int a2[1] = {0}, b2[1] = {8};
    if (swap_run_layout(*tp, a2, b2, 1, 9, 8)) ++bad;
    std::printf("bad %ld layouts %ld\n", bad, layouts);
    return bad || layouts < 200 ? 1 : 0;
}
