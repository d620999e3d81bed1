// CPU check of the warp-tile layout (warp_tile_layout in libq1gpu.so) for
// both tile shapes: complex64 (1024 amplitudes, 16 per stage row) and
// complex128 (512 amplitudes, 8 per row).  Over every tile of small states,
// slot (m, lane) addresses cover each amplitude once; the staged offsets of
// the slots fill the warp's stage once; the 2^tb staged offsets a unit reads
// hold one amplitude with every gate state at its offs[] offset; the units
// one phase of a warp reads for one gate state (16 lanes of 8 bytes, 8 lanes
// of 16 bytes), like the slots one phase copies, lie in distinct bank
// groups; and where pairs16 is set, amplitude pairs (2i, 2i+1) stay adjacent
// and 16-byte aligned.  The batch executor's wrapper (batch_tile_layout)
// gives the complex64 layout.  Prints "bad <count> ..."; exit status 1 on
// any failure.
#include <algorithm>
#include <cstdio>
#include <cstring>
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
    for (int trial = 0; trial < 6000; ++trial) {
        const bool c128 = trial % 2 == 1;
        const int tile_bits = c128 ? 9 : 10, C = c128 ? 3 : 4, phase = 1 << C;
        const int ntile = 1 << tile_bits, nslots = 1 << (tile_bits - 5);
        const int nbits = trial < 4500 ? tile_bits + (int)(rng() % 5) : 15 + (int)(rng() % 12);
        const int tb = 1 + (int)(rng() % 4);
        std::vector<int> pos;
        while ((int)pos.size() < tb) {
            // low positions more often: they are the ones that need the stage
            const int p = (rng() % 2) ? (int)(rng() % std::min(nbits, 8)) : (int)(rng() % nbits);
            if (std::find(pos.begin(), pos.end(), p) == pos.end()) pos.push_back(p);
        }
        uint64_t gmask = 0;
        for (int p : pos) gmask |= uint64_t(1) << p;
        uint64_t offs[16];
        for (int s = 0; s < (1 << tb); ++s) {
            uint64_t o = 0;
            for (int j = 0; j < tb; ++j)
                if ((s >> (tb - 1 - j)) & 1) o |= uint64_t(1) << pos[j];
            offs[s] = o;
        }
        WarpTile w;
        if (c128) {
            warp_tile_layout(w, pos.data(), tb, offs, nbits, 9, 3);
        } else {
            BatchOp op{};
            std::memcpy(op.offs, offs, sizeof(offs));
            batch_tile_layout(op, pos.data(), tb, nbits);
            w = op.tile;
        }
        if (!w.tiled || w.tile_bits != tile_bits) {
            ++bad;
            continue;
        }
        ++layouts;
        const uint64_t N = uint64_t(1) << nbits;
        const uint64_t ntiles = N >> tile_bits;
        auto lphys = [&](int lane) {
            uint32_t p = 0;
            for (int b = 0; b < 5; ++b)
                if ((lane >> b) & 1) p ^= w.lphys[b];
            return p;
        };
        std::vector<uint32_t> goff(nslots), soff(nslots);
        for (int m = 0; m < nslots; ++m) {
            goff[m] = 0;
            soff[m] = 0;
            for (int b = 0; b < tile_bits - 5; ++b)
                if ((m >> b) & 1) {
                    goff[m] |= w.gbit[b];
                    soff[m] ^= w.sbit[b];
                }
        }
        // stage slot of every (m, lane)
        std::vector<int> seen(ntile, 0);
        std::vector<uint32_t> slot_m(ntile), slot_lane(ntile);
        for (int m = 0; m < nslots; ++m)
            for (int lane = 0; lane < 32; ++lane) {
                const uint32_t st = soff[m] ^ lphys(lane);
                if (st >= (uint32_t)ntile) {
                    ++bad;
                    continue;
                }
                ++seen[st];
                slot_m[st] = m;
                slot_lane[st] = lane;
            }
        for (int k = 0; k < ntile; ++k)
            if (seen[k] != 1) ++bad;
        // copies of one phase (consecutive lanes): distinct bank groups in one row
        for (int m = 0; m < nslots; ++m)
            for (int h = 0; h < 32 / phase; ++h) {
                uint32_t cols = 0;
                for (int l = phase * h; l < phase * h + phase; ++l) cols |= 1u << ((soff[m] ^ lphys(l)) & (phase - 1));
                if (cols != (1u << phase) - 1) ++bad;
            }
        auto amp = [&](uint64_t tile, uint32_t st) {
            return expand_index(tile, w.tile_map) + slot_lane[st] + goff[slot_m[st]];
        };
        // every amplitude once (exhaustive on small states, sampled tiles on large ones)
        if (nbits <= 14) {
            std::vector<uint8_t> hit(N, 0);
            for (uint64_t t = 0; t < ntiles; ++t)
                for (uint32_t st = 0; st < (uint32_t)ntile; ++st) {
                    const uint64_t a = amp(t, st);
                    if (a >= N) {
                        ++bad;
                        continue;
                    }
                    hit[a]++;
                }
            for (uint64_t a = 0; a < N; ++a)
                if (hit[a] != 1) ++bad;
        } else {
            for (int r = 0; r < 4; ++r) {
                const uint64_t t = rng() % ntiles;
                for (uint32_t st = 0; st < (uint32_t)ntile; ++st)
                    if (amp(t, st) >= N) ++bad;
            }
        }
        // units: the staged offsets of (unit, s) hold one amplitude with every gate state
        const int nw = 1 << (tile_bits - tb);
        const uint64_t t = rng() % ntiles;
        std::vector<uint64_t> bases;
        auto unit_phys = [&](int u) {
            uint32_t pw = 0;
            for (int b = 0; b < tile_bits - tb; ++b)
                if ((u >> b) & 1) pw ^= w.wbit[b];
            return pw;
        };
        for (int u = 0; u < nw; ++u) {
            const uint32_t pw = unit_phys(u);
            const uint64_t a0 = amp(t, pw ^ w.gsoff[0]);
            if (a0 & gmask) ++bad;
            for (int s = 0; s < (1 << tb); ++s) {
                const uint32_t st = pw ^ w.gsoff[s];
                if (st >= (uint32_t)ntile || amp(t, st) != (a0 | offs[s])) ++bad;
            }
            bases.push_back(a0);
        }
        std::sort(bases.begin(), bases.end());
        if (std::adjacent_find(bases.begin(), bases.end()) != bases.end()) ++bad;
        // reads of one phase (units k * 32 + consecutive lanes) for one gate state
        for (int k = 0; k < std::max(1, nw / 32); ++k)
            for (int h = 0; h < 32 / phase; ++h)
                for (int s = 0; s < (1 << tb); ++s) {
                    uint32_t cols = 0;
                    int n = 0;
                    for (int l = phase * h; l < phase * h + phase && k * 32 + l < nw; ++l, ++n)
                        cols |= 1u << ((unit_phys(k * 32 + l) ^ w.gsoff[s]) & (phase - 1));
                    if (n == phase && cols != (1u << phase) - 1) ++bad;
                }
        // pairs16 (complex64 only): set exactly when position 0 is not a gate position;
        // pair (2i, 2i+1) of every slot adjacent and 16-byte aligned in the stage
        if (w.pairs16 != ((!c128 && !(gmask & 1)) ? 1 : 0)) ++bad;
        if (w.pairs16) {
            for (int b = 0; b < tile_bits - 5; ++b)
                if ((w.gbit[b] & 1) || (w.sbit[b] & 1)) ++bad;
            for (int lane = 0; lane < 32; ++lane) {
                uint32_t p16 = 0;
                for (int b = 0; b < 4; ++b)
                    if ((lane >> b) & 1) p16 ^= w.lphys[b + 1];
                for (int mm = 0; mm < nslots / 2; ++mm) {
                    const int m = 2 * mm + (lane >> 4), i = lane & 15;
                    const uint32_t st = soff[m] ^ p16;
                    if ((st & 1) || st != (soff[m] ^ lphys(2 * i)) || (st ^ 1u) != (soff[m] ^ lphys(2 * i + 1)))
                        ++bad;
                }
            }
        }
    }
    // states below the tile size keep the per-thread paths
    BatchOp small{};
    const int p0[1] = {0};
    batch_tile_layout(small, p0, 1, 9);
    if (small.tile.tiled) ++bad;
    WarpTile w8;
    const uint64_t o1[2] = {0, 1};
    warp_tile_layout(w8, p0, 1, o1, 8, 9, 3);
    if (w8.tiled) ++bad;
    std::printf("bad %ld layouts %ld\n", bad, layouts);
    return bad ? 1 : 0;
}
