// CPU check of the batch executor's warp-tile layout (batch_tile_layout in
// libq1gpu.so): over every tile of small states, slot (m, lane) addresses
// cover each amplitude once; the staged offsets of the slots fill the warp's
// 1024-entry stage once; the 2^tb staged offsets a unit reads hold one
// amplitude with every gate state at its offs[] offset; and the 16 units a
// half warp reads for one gate state, like the 16 slots a half warp copies,
// lie in 16 different 8-byte bank pairs.  Prints "bad <count> ...";
// exit status 1 on any failure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/kernels.h"

namespace q1g {
void batch_tile_layout(BatchOp& op, const int* pos, int tb, int nbits);
}
using namespace q1g;

int main()
{
    std::mt19937 rng(7);
    long bad = 0, layouts = 0;
    for (int trial = 0; trial < 4000; ++trial) {
        const int nbits = trial < 3000 ? 10 + (int)(rng() % 5) : 15 + (int)(rng() % 12);
        const int tb = 1 + (int)(rng() % 4);
        std::vector<int> pos;
        while ((int)pos.size() < tb) {
            // low positions more often: they are the ones that need the stage
            const int p = (rng() % 2) ? (int)(rng() % std::min(nbits, 8)) : (int)(rng() % nbits);
            if (std::find(pos.begin(), pos.end(), p) == pos.end()) pos.push_back(p);
        }
        BatchOp op{};
        uint64_t gmask = 0;
        for (int p : pos) gmask |= uint64_t(1) << p;
        for (int s = 0; s < (1 << tb); ++s) {
            uint64_t o = 0;
            for (int j = 0; j < tb; ++j)
                if ((s >> (tb - 1 - j)) & 1) o |= uint64_t(1) << pos[j];
            op.offs[s] = o;
        }
        batch_tile_layout(op, pos.data(), tb, nbits);
        if (!op.tiled) {
            ++bad;
            continue;
        }
        ++layouts;
        const uint64_t N = uint64_t(1) << nbits;
        const uint64_t ntiles = N >> kBatchTileBits;
        auto plane = [&](int lane) { return (uint32_t)(lane & 15) ^ ((lane & 16) ? op.lane16 : 0u); };
        uint32_t goff[32], soff[32];
        for (int m = 0; m < 32; ++m) {
            goff[m] = 0;
            soff[m] = 0;
            for (int b = 0; b < 5; ++b)
                if ((m >> b) & 1) {
                    goff[m] |= op.gbit[b];
                    soff[m] ^= op.sbit[b];
                }
        }
        // stage slot of every (m, lane), and its amplitude in a given tile
        std::vector<int> seen_stage(1024, 0);
        std::vector<uint32_t> slot_m(1024), slot_lane(1024);
        for (int m = 0; m < 32; ++m)
            for (int lane = 0; lane < 32; ++lane) {
                const uint32_t st = soff[m] ^ plane(lane);
                if (st >= 1024) { ++bad; continue; }
                ++seen_stage[st];
                slot_m[st] = m;
                slot_lane[st] = lane;
            }
        for (int k = 0; k < 1024; ++k)
            if (seen_stage[k] != 1) ++bad;
        // 16-byte copies (pairs16): the pair (2i, 2i+1) of every slot is adjacent and
        // 16-byte aligned in the stage and in the state; set exactly when position 0
        // is not a gate position
        if (op.pairs16 != ((gmask & 1) ? 0 : 1)) ++bad;
        if (op.pairs16) {
            for (int b = 0; b < 5; ++b)
                if ((op.gbit[b] & 1) || (op.sbit[b] & 1)) ++bad;
            for (int lane = 0; lane < 32; ++lane) {
                const uint32_t p16 = (uint32_t)((2 * lane) & 15) ^ ((lane & 8) ? op.lane16 : 0u);
                for (int mm = 0; mm < 16; ++mm) {
                    const int m = 2 * mm + (lane >> 4), i = lane & 15;
                    const uint32_t st = soff[m] ^ p16;
                    if ((st & 1) || st != (soff[m] ^ plane(2 * i)) || (st ^ 1u) != (soff[m] ^ plane(2 * i + 1)))
                        ++bad;
                }
            }
        }
        // copies of a half warp: 16 distinct bank pairs
        for (int m = 0; m < 32; ++m)
            for (int h = 0; h < 2; ++h) {
                uint32_t banks = 0;
                for (int l = 16 * h; l < 16 * h + 16; ++l) banks |= 1u << ((soff[m] ^ plane(l)) & 15);
                if (banks != 0xffffu) ++bad;
            }
        auto amp = [&](uint64_t tile, uint32_t st) {
            return expand_index(tile, op.tile_map) + slot_lane[st] + goff[slot_m[st]];
        };
        // every amplitude once (exhaustive on small states, sampled tiles on large ones)
        if (nbits <= 14) {
            std::vector<uint8_t> hit(N, 0);
            for (uint64_t t = 0; t < ntiles; ++t)
                for (uint32_t st = 0; st < 1024; ++st) {
                    const uint64_t a = amp(t, st);
                    if (a >= N) { ++bad; continue; }
                    hit[a]++;
                }
            for (uint64_t a = 0; a < N; ++a)
                if (hit[a] != 1) ++bad;
        } else {
            for (int r = 0; r < 4; ++r) {
                const uint64_t t = rng() % ntiles;
                for (uint32_t st = 0; st < 1024; ++st)
                    if (amp(t, st) >= N) ++bad;
            }
        }
        // units: the staged offsets of (w, s) hold one amplitude with every gate state
        const int nw = 1 << (kBatchTileBits - tb);
        const uint64_t t = rng() % ntiles;
        std::vector<uint64_t> bases;
        for (int w = 0; w < nw; ++w) {
            uint32_t pw = 0;
            for (int b = 0; b < kBatchTileBits - tb; ++b)
                if ((w >> b) & 1) pw ^= op.wbit[b];
            const uint64_t a0 = amp(t, pw ^ op.gsoff[0]);
            if (a0 & gmask) ++bad;
            for (int s = 0; s < (1 << tb); ++s) {
                const uint32_t st = pw ^ op.gsoff[s];
                if (st >= 1024 || amp(t, st) != (a0 | op.offs[s])) ++bad;
            }
            bases.push_back(a0);
        }
        std::sort(bases.begin(), bases.end());
        if (std::adjacent_find(bases.begin(), bases.end()) != bases.end()) ++bad;
        // reads of a half warp (units k * 32 + 16h .. +15) for one gate state: 16 bank pairs
        for (int k = 0; k < nw / 32; ++k)
            for (int h = 0; h < 2; ++h)
                for (int s = 0; s < (1 << tb); ++s) {
                    uint32_t banks = 0;
                    for (int l = 16 * h; l < 16 * h + 16; ++l) {
                        const int w = k * 32 + l;
                        uint32_t pw = 0;
                        for (int b = 0; b < kBatchTileBits - tb; ++b)
                            if ((w >> b) & 1) pw ^= op.wbit[b];
                        banks |= 1u << ((pw ^ op.gsoff[s]) & 15);
                    }
                    if (banks != 0xffffu) ++bad;
                }
    }
    // states below the tile size keep the per-thread path
    BatchOp small{};
    const int p0[1] = {0};
    batch_tile_layout(small, p0, 1, kBatchTileBits - 1);
    if (small.tiled) ++bad;
    std::printf("bad %ld layouts %ld\n", bad, layouts);
    return bad ? 1 : 0;
}
