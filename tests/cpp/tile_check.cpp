// CPU check of the tensor-core pass geometry in libq1gpu.so (built by
// tests/test_host_logic.py against the library): tc_tile_box maps every box
// element to the amplitude its tile coordinate denotes, and tc_choose_padding
// lays a staged tile out without overlaps, inside the stage, with copy
// pieces that never straddle a padding gap.  Exit status 1 on any failure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/kernels.h"

using namespace q1g;

static uint32_t staged(uint32_t x, uint32_t pad) { return 8u * x + ((pad < 31 ? (x >> pad) : 0u) << 4); }

int main()
{
    std::mt19937 rng(1);
    int bad = 0, usable = 0, trials = 0;
    for (int trial = 0; trial < 3000; ++trial) {
        const int nbits = 12 + (int)(rng() % 20);
        const uint64_t ncols = (rng() % 3 == 0) ? 1 + rng() % 5 : 1;
        std::vector<int> T;
        const int nb = 1 + (int)(rng() % 2);
        for (int b = 0; b < nb * 5 && (int)T.size() < 10; ++b) {
            const int p = (int)(rng() % nbits);
            if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
        }
        for (int p = 0; (int)T.size() < 12 && p < nbits; ++p)
            if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
        std::sort(T.begin(), T.end());
        const TcTileBox b = tc_tile_box(T.data(), nbits, ncols);
        ++trials;
        if (!b.usable) continue;
        ++usable;
        IndexMap tm{};
        tm.nz = 12;
        for (int j = 0; j < 12; ++j) tm.zpos[j] = T[j];
        const uint64_t ntiles = (ncols << nbits) >> 12;
        uint64_t elems = 1;
        for (int d = 0; d < 5; ++d) elems *= b.box[d];
        if (elems != 4096 || b.tmask[0] != 0) ++bad;
        for (int d = 1; d < 5; ++d)
            if (b.gstride[d] % 16 || b.gstride[d] >= (uint64_t(1) << 40)) ++bad;
        for (int k = 0; k < 4; ++k) {
            uint64_t t = k == 0 ? 0 : (k == 1 ? ntiles - 1 : rng() % ntiles);
            const uint64_t base = expand_index(t, tm);
            uint64_t off = 0;
            for (int d = 0; d < 5; ++d) {
                const uint64_t c = (uint32_t)(t >> b.tshift[d]) & b.tmask[d];
                if (c + b.box[d] > b.gdim[d]) ++bad;
                off += c * (d ? b.gstride[d] / 8 : 1);
            }
            if (off != base) ++bad;
            uint64_t x = 0;
            for (uint64_t e4 = 0; e4 < b.box[4]; ++e4)
                for (uint64_t e3 = 0; e3 < b.box[3]; ++e3)
                    for (uint64_t e2 = 0; e2 < b.box[2]; ++e2)
                        for (uint64_t e1 = 0; e1 < b.box[1]; ++e1)
                            for (uint64_t e0 = 0; e0 < b.box[0]; ++e0, ++x) {
                                const uint64_t o = off + e0 + e1 * b.gstride[1] / 8 + e2 * b.gstride[2] / 8 +
                                                   e3 * b.gstride[3] / 8 + e4 * b.gstride[4] / 8;
                                uint64_t want = base;
                                for (int j = 0; j < 12; ++j)
                                    if ((x >> j) & 1) want |= uint64_t(1) << T[j];
                                if (o != want) ++bad;
                            }
        }
    }
    // padding: one and two blocks on random gate positions of a 12-bit tile
    int padded = 0;
    for (int trial = 0; trial < 400; ++trial) {
        TcOffsets o{};
        o.nblocks = 1 + (uint32_t)(rng() % 2);
        o.run_bits = 7 + (uint32_t)(rng() % 6);
        for (uint32_t b = 0; b < o.nblocks; ++b) {
            std::vector<int> g;
            while (g.size() < 5) {
                const int p = (int)(rng() % 12);
                if (std::find(g.begin(), g.end(), p) == g.end()) g.push_back(p);
            }
            std::sort(g.begin(), g.end());
            TcBlockGeom& G = o.blk[b];
            int r = 0;
            for (int j = 0; j < 12; ++j)
                if (std::find(g.begin(), g.end(), j) == g.end()) G.jrow_bit[r++] = 1u << j;
            for (int s = 0; s < 32; ++s) {
                uint32_t jc = 0;
                for (int i = 0; i < 5; ++i)
                    if ((s >> i) & 1) jc |= 1u << g[i];
                G.jgate[s] = jc;
            }
            G.vec2 = G.jgate[1] == 1u;
        }
        tc_choose_padding(o, (rng() % 2) == 0);
        padded += o.pad_shift < 31;
        if (o.piece_bits > o.run_bits || (o.pad_shift < 31 && o.piece_bits > o.pad_shift)) ++bad;
        if (o.npieces != (4096u >> o.piece_bits)) ++bad;
        if (o.stage_bytes != 32768u + (o.pad_shift < 31 ? 16u * (4096u >> o.pad_shift) : 0u)) ++bad;
        for (uint32_t b = 0; b < o.nblocks; ++b) {
            const TcBlockGeom& G = o.blk[b];
            // rows and gates cover the tile once; staged offsets follow the padding
            std::vector<char> seen(4096, 0);
            for (uint32_t t = 0; t < 128; ++t) {
                uint32_t xr = 0, rb = 0;
                for (int r = 0; r < 7; ++r)
                    if ((t >> r) & 1) {
                        xr |= G.jrow_bit[r];
                        rb += G.rowoff[r];
                    }
                for (int s = 0; s < 32; ++s) {
                    const uint32_t x = xr | G.jgate[s];
                    if (x >= 4096 || seen[x]) ++bad;
                    else seen[x] = 1;
                    const uint32_t byte = rb + G.gateoff[s];
                    if (byte != staged(x, o.pad_shift) || byte + 8 > o.stage_bytes) ++bad;
                    if (G.vec2 && (s & 1) == 0 && G.gateoff[s + 1] != G.gateoff[s] + 8) ++bad;
                }
            }
        }
    }
    std::printf("trials %d usable %d padded %d bad %d\n", trials, usable, padded, bad);
    return bad != 0;
}
