// Warp-tile layout (warp_tile.h).
#include "warp_tile.h"

#include <cstring>

namespace q1g {

void warp_tile_layout(WarpTile& w, const int* pos, int tb, const uint64_t* offs, int nbits, int tile_bits,
                      int col_bits)
{
    std::memset(&w, 0, sizeof(w));
    if (tile_bits < 9 || tile_bits > 10 || col_bits < 3 || col_bits > 4 || nbits < tile_bits || tb < 1 || tb > 4)
        return;
    uint64_t gmask = 0;
    for (int j = 0; j < tb; ++j) gmask |= uint64_t(1) << pos[j];
    // tile positions L ascending; ng = local slots of the non-gate positions
    int L[10], ng[10];
    int nl = 0, nng = 0;
    for (int p = 0; nl < tile_bits; ++p) {
        if ((gmask >> p) & 1) {
            L[nl++] = p;
        } else if (nng < tile_bits - tb) {
            ng[nng++] = nl;
            L[nl++] = p;
        }
    }
    // row bit -> column mask: the unit-number bits b < col_bits that land in
    // row bits take the column bits of the gate positions among 0..col_bits-1
    const int C = col_bits;
    uint32_t M[10] = {};
    uint32_t used = 0;
    for (int b = 0; b < C; ++b)
        if (ng[b] < C) used |= 1u << ng[b];
    int free_col = 0;
    for (int b = 0; b < C; ++b) {
        if (ng[b] < C) continue;
        while ((used >> free_col) & 1) ++free_col;
        M[ng[b] - C] = 1u << free_col;
        used |= 1u << free_col;
    }
    auto phys = [&](uint32_t idx) {
        uint32_t r = idx;
        for (int q = C; q < tile_bits; ++q)
            if ((idx >> q) & 1) r ^= M[q - C];
        return r;
    };
    auto local = [&](uint64_t amp_offset) {
        uint32_t r = 0;
        for (int k = 0; k < tile_bits; ++k)
            if ((amp_offset >> L[k]) & 1) r |= 1u << k;
        return r;
    };
    w.tiled = 1;
    w.tile_bits = tile_bits;
    w.pairs16 = (C == 4 && !(gmask & 1)) ? 1 : 0;
    for (int b = 0; b < 5; ++b) w.lphys[b] = phys(1u << b);
    w.tile_map.nz = tile_bits;
    for (int k = 0; k < tile_bits; ++k) w.tile_map.zpos[k] = L[k];
    w.tile_map.setmask = 0;
    for (int b = 0; b < tile_bits - 5; ++b) {
        w.gbit[b] = 1u << L[5 + b];
        w.sbit[b] = phys(1u << (5 + b));
    }
    for (int s = 0; s < (1 << tb); ++s) w.gsoff[s] = (uint16_t)phys(local(offs[s]));
    for (int b = 0; b < nng; ++b) w.wbit[b] = (uint16_t)phys(1u << ng[b]);
}

}  // namespace q1g
