// CPU check of the direct two-block tensor-core pass (fused_tc.cu, pair mode
// 3): for random tile geometries, tc_direct_layout's scatter tables send
// every output (row t, gate state g) of the first block, as the kernel
// computes its offset (XOR of scat_row over t's bits, XOR scat_gate[g]), to
// a distinct 4-byte word of the 16 KB operand plane, and that word is where
// a K-major SWIZZLE_128B operand holds (row r2, K index 2 g2) of the second
// block for the same tile coordinate.  Also checks the second block's gate
// order, the staged offsets and the 1024-byte stage alignment.  Then, for
// the four-group kernel, tc_split_map's deal of the first block's tile
// (single-block passes too): every (thread, register) reads a distinct tile
// coordinate at its staged offset and stores it where the first block's A
// operand holds (row, K index 2 g) in the block's new gate order, and the
// scatter follows that order.  For chain layouts whose last block stores
// lane-permuted (TcOffsets::wb_xor), every (row, gate state) lands once at
// its own staged offset, and the brick circuit's pair on the lowest
// positions takes that form at the modelled cost.  Prints how many layouts
// have a conflict-free scatter.  Exit status 1 on any failure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/kernels.h"

using namespace q1g;

static uint32_t staged(uint32_t x, uint32_t pad) { return 8u * x + ((pad < 31 ? (x >> pad) : 0u) << 4); }

static void default_geom(TcBlockGeom& G, const std::vector<int>& gate_bits)
{
    // gate bit k (LSB first) = tile bit gate_bits[k]; rows ascending
    int r = 0;
    for (int j = 0; j < 12; ++j)
        if (std::find(gate_bits.begin(), gate_bits.end(), j) == gate_bits.end()) G.jrow_bit[r++] = 1u << j;
    for (int g = 0; g < 32; ++g) {
        uint32_t jc = 0;
        for (int k = 0; k < 5; ++k)
            if ((g >> k) & 1) jc |= 1u << gate_bits[k];
        G.jgate[g] = jc;
    }
    G.vec2 = G.jgate[1] == 1u ? 1u : 0u;
}

// tc_split_map's deal against the geometry of block 0 (after the map).
static int check_split(const TcOffsets& o)
{
    int bad = 0;
    std::vector<int> inv(40000, -1);
    for (uint32_t x = 0; x < 4096; ++x) inv[staged(x, o.pad_shift)] = (int)x;
    std::vector<int> seen(4096, 0);
    const TcBlockGeom& G = o.blk[0];
    for (int g = 0; g < 32; ++g)
        if (G.gateoff[g] != staged(G.jgate[g], o.pad_shift)) ++bad;
    if (G.vec2 != (G.jgate[1] == 1u ? 1u : 0u) || o.sp_vec2 != G.vec2) ++bad;
    for (uint32_t t = 0; t < 128; ++t) {
        uint32_t tb = 0, ta = 0;
        for (int i = 0; i < 7; ++i)
            if ((t >> i) & 1u) {
                tb += o.sp_thoff[i];
                ta ^= o.sp_athr[i];
            }
        for (int j = 0; j < 32; ++j) {
            const uint32_t off = tb + o.sp_regoff[j];
            if (off >= inv.size() || inv[off] < 0) {
                ++bad;
                continue;
            }
            const uint32_t x = (uint32_t)inv[off];
            if (seen[x]++) ++bad;
            if (o.sp_vec2 && (j & 1) == 0 && o.sp_regoff[j + 1] != o.sp_regoff[j] + 8u) ++bad;
            uint32_t r = 0, gi = 0;
            for (int i = 0; i < 7; ++i)
                if (x & G.jrow_bit[i]) r |= 1u << i;
            for (int k = 0; k < 5; ++k)
                if (x & G.jgate[1 << k]) gi |= 1u << k;
            const uint32_t a = (ta ^ o.sp_achunk[j >> 2]) + 4u * (uint32_t)(j & 3);
            if (a != tc_sw128_offset(r, 2u * gi) || a >= 16384u) ++bad;
        }
    }
    return bad;
}

// Transition k of a direct pass: block k's output (thread t, gate g) lands
// on a distinct word of block k+1's operand plane, where that operand holds
// (row, K = 2 gate) of block k+1 for the same tile coordinate.
static int check_scatter(const TcOffsets& o, int k)
{
    int bad = 0;
    std::vector<int> seen(4096, 0);
    const TcBlockGeom& A = o.blk[k];
    const TcBlockGeom& B = o.blk[k + 1];
    for (uint32_t t = 0; t < 128; ++t) {
        uint32_t rowpart = 0, xrow = 0;
        for (int i = 0; i < 7; ++i)
            if ((t >> i) & 1u) {
                rowpart ^= o.scat_row[k][i];
                xrow |= A.jrow_bit[i];
            }
        for (int g = 0; g < 32; ++g) {
            const uint32_t a = rowpart ^ o.scat_gate[k][g];
            if (a >= 16384u || (a & 3u)) {
                ++bad;
                continue;
            }
            if (seen[a >> 2]++) ++bad;
            const uint32_t x = xrow | A.jgate[g];
            uint32_t r2 = 0, g2 = 0;
            for (int i = 0; i < 7; ++i)
                if (x & B.jrow_bit[i]) r2 |= 1u << i;
            for (int q = 0; q < 5; ++q)
                if (x & B.jgate[1 << q]) g2 |= 1u << q;
            if (a != tc_sw128_offset(r2, 2u * g2)) ++bad;
        }
    }
    return bad;
}

// The last block's lane-permuted write-back (TcOffsets::wb_xor), as the
// kernel computes it: thread t with lane permutation wx stores, at step j of
// half hh, its output gate state 16 hh + (j ^ wx) at staged byte
// (row offset ^ gateoff of wx) ^ gateoff[16 hh + j] (pairs of gate states
// per 16-byte store where vec2).  That must be the state's own staged
// offset, every (row, state) once; the permutation is zero unless the
// layout is unpadded, and keeps 16-byte pairs together.
static int check_wb_xor(const TcOffsets& o, bool* used)
{
    const TcBlockGeom& L = o.blk[o.nblocks - 1];
    uint32_t any = 0;
    for (int r = 0; r < 5; ++r) any |= o.wb_xor[r];
    *used = any != 0;
    if (!any) return 0;
    int bad = 0;
    if (o.pad_shift < 31) ++bad;
    for (int r = 0; r < 5; ++r)
        if (o.wb_xor[r] >= 16u || (L.vec2 && (o.wb_xor[r] & 1u))) ++bad;
    std::vector<int> seen(4096, 0);
    for (uint32_t t = 0; t < 128; ++t) {
        uint32_t rowb = 0, wx = 0;
        for (int i = 0; i < 7; ++i)
            if ((t >> i) & 1u) rowb += L.rowoff[i];
        for (int r = 0; r < 5; ++r)
            if ((t >> r) & 1u) wx ^= o.wb_xor[r];
        uint32_t rowx = rowb;
        for (int k = 0; k < 4; ++k)
            if ((wx >> k) & 1u) rowx ^= L.gateoff[1 << k];
        for (int hh = 0; hh < 2; ++hh)
            for (int j = 0; j < 16; ++j) {
                const uint32_t gs = 16u * hh + ((uint32_t)j ^ wx);   // the state stored at step j
                uint32_t addr;
                if (L.vec2) {
                    // step j / 2 stores the pair (2m, 2m+1), m = j / 2
                    addr = (rowx ^ L.gateoff[16 * hh + (j & ~1)]) + 8u * (uint32_t)(j & 1);
                } else {
                    addr = rowx ^ L.gateoff[16 * hh + j];
                }
                if (addr != rowb + L.gateoff[gs] || (addr & 7u) || addr / 8u >= 4096u) {
                    ++bad;
                    continue;
                }
                if (seen[addr / 8u]++) ++bad;
            }
    }
    return bad;
}

int main()
{
    std::mt19937 rng(7);
    int bad = 0, trials = 0, minimal = 0, padded = 0;
    for (int trial = 0; trial < 1500; ++trial) {
        std::vector<int> all(12);
        for (int j = 0; j < 12; ++j) all[j] = j;
        std::vector<int> g0, g1;
        // block 1 overlaps block 0 on 0..4 tile bits; brick-like pairs
        // (shifted windows) half of the time
        if (trial % 2 == 0) {
            const int lo0 = (int)(rng() % 8), shift = 1 + (int)(rng() % 4);
            const int lo1 = std::max(0, std::min(7, lo0 + ((rng() & 1) ? shift : -shift)));
            for (int k = 0; k < 5; ++k) {
                g0.push_back(lo0 + k);
                g1.push_back(lo1 + k);
            }
        } else {
            std::shuffle(all.begin(), all.end(), rng);
            g0.assign(all.begin(), all.begin() + 5);
            std::shuffle(all.begin(), all.end(), rng);
            g1.assign(all.begin(), all.begin() + 5);
        }
        std::shuffle(g0.begin(), g0.end(), rng);
        std::shuffle(g1.begin(), g1.end(), rng);
        if (g0 == g1) continue;
        TcOffsets o{};
        o.nblocks = 2;
        o.run_bits = (uint32_t)(rng() % 13);
        o.nruns = 1u << (12 - o.run_bits);
        default_geom(o.blk[0], g0);
        default_geom(o.blk[1], g1);
        const uint32_t gate0 = o.blk[0].jgate[31], gate1 = o.blk[1].jgate[31];
        uint32_t jgate0[32];
        for (int g = 0; g < 32; ++g) jgate0[g] = o.blk[0].jgate[g];
        int gbit1[5];
        const bool tma_ok = (rng() % 3) != 0;
        if (!tc_direct_layout(o, tma_ok, 2, gbit1)) {
            ++bad;
            std::printf("layout refused, trial %d\n", trial);
            continue;
        }
        ++trials;
        if (o.pad_shift < 31) ++padded;
        // the direct layout keeps block 0's gate order; block 1 keeps its
        // gate set, in the order gbit1
        for (int g = 0; g < 32; ++g)
            if (o.blk[0].jgate[g] != jgate0[g]) ++bad;
        if (o.blk[1].jgate[31] != gate1 || o.direct != 1 || o.shuffle != 0) ++bad;
        for (int k = 0; k < 5; ++k)
            if (o.blk[1].jgate[1 << k] != (1u << gbit1[k])) ++bad;
        if (o.blk[1].vec2 != (o.blk[1].jgate[1] == 1u ? 1u : 0u)) ++bad;
        // row bits: each block's rows are the tile bits outside its gates
        for (int b = 0; b < 2; ++b) {
            uint32_t rows = 0;
            for (int r = 0; r < 7; ++r) rows |= o.blk[b].jrow_bit[r];
            if (rows != (0xFFFu & ~(b ? gate1 : gate0))) ++bad;
        }
        if (o.stage_bytes % 1024u || o.stage_bytes < 32768u) ++bad;
        // staged offsets: every tile coordinate of each block inside the
        // stage and in its own place
        for (int b = 0; b < 2; ++b) {
            const TcBlockGeom& G = o.blk[b];
            for (int r = 0; r < 7; ++r)
                if (G.rowoff[r] != staged(G.jrow_bit[r], o.pad_shift)) ++bad;
            for (int g = 0; g < 32; ++g)
                if (G.gateoff[g] != staged(G.jgate[g], o.pad_shift)) ++bad;
        }
        // the four-group kernel deals block 0's tile by a split map in a
        // gate order of its own; the checks below use that order
        int gbit0[5];
        tc_split_map(o, gbit0);
        bad += check_split(o);
        for (int k = 0; k < 5; ++k)
            if (o.blk[0].jgate[1 << k] != (1u << gbit0[k])) ++bad;
        if (o.blk[0].jgate[31] != gate0) ++bad;
        // the scatter
        std::vector<int> seen(4096, 0);
        for (uint32_t t = 0; t < 128; ++t) {
            uint32_t rowpart = 0, xrow = 0;
            for (int i = 0; i < 7; ++i)
                if ((t >> i) & 1u) {
                    rowpart ^= o.scat_row[0][i];
                    xrow |= o.blk[0].jrow_bit[i];
                }
            for (int g = 0; g < 32; ++g) {
                const uint32_t a = rowpart ^ o.scat_gate[0][g];
                if (a >= 16384u || (a & 3u)) {
                    ++bad;
                    continue;
                }
                if (seen[a >> 2]++) ++bad;
                const uint32_t x = xrow | o.blk[0].jgate[g];
                uint32_t r2 = 0, g2 = 0;
                for (int i = 0; i < 7; ++i)
                    if (x & o.blk[1].jrow_bit[i]) r2 |= 1u << i;
                for (int k = 0; k < 5; ++k)
                    if (x & o.blk[1].jgate[1 << k]) g2 |= 1u << k;
                if (a != tc_sw128_offset(r2, 2u * g2)) ++bad;
            }
        }
        // predicted wavefronts: the minimum is 64 per warp for each of
        // block 0's reads, the scatter and block 1's stores
        bool at_min = true;
        {
            // scatter: lanes = row bits 0..4 of block 0
            int per_bank[32] = {0}, m = 0;
            for (uint32_t l = 0; l < 32; ++l) {
                uint32_t a = 0;
                for (int i = 0; i < 5; ++i)
                    if ((l >> i) & 1u) a ^= o.scat_row[0][i];
                m = std::max(m, ++per_bank[(a >> 2) & 31u]);
            }
            at_min = m == 1;
        }
        minimal += at_min;
    }
    // single-block passes of the four-group kernel
    int singles = 0;
    for (int trial = 0; trial < 600; ++trial) {
        std::vector<int> all(12);
        for (int j = 0; j < 12; ++j) all[j] = j;
        std::shuffle(all.begin(), all.end(), rng);
        std::vector<int> g0(all.begin(), all.begin() + 5);
        TcOffsets o{};
        o.nblocks = 1;
        o.run_bits = (uint32_t)(rng() % 13);
        o.nruns = 1u << (12 - o.run_bits);
        default_geom(o.blk[0], g0);
        const uint32_t gate0 = o.blk[0].jgate[31];
        tc_choose_padding(o, (rng() % 3) != 0, 2 + (int)(rng() % 3));
        int gbit0[5];
        tc_split_map(o, gbit0);
        bad += check_split(o);
        if (o.blk[0].jgate[31] != gate0) ++bad;
        ++singles;
    }
    // chained layouts of the four-group kernel: pairs and triples
    int chains = 0, chain_free = 0, wb_permuted = 0;
    for (int trial = 0; trial < 900; ++trial) {
        const int nb = 2 + trial % 2;
        std::vector<std::vector<int>> gs(nb);
        if (trial % 3 != 2) {
            // brick-like windows of five, each shifted from the previous
            int lo = (int)(rng() % 4);
            for (int b = 0; b < nb; ++b) {
                for (int k = 0; k < 5; ++k) gs[b].push_back(std::min(11, lo + k) - (lo + 4 > 11 ? lo + 4 - 11 : 0));
                lo = std::max(0, std::min(7, lo + 1 + (int)(rng() % 3)));
            }
        } else {
            for (int b = 0; b < nb; ++b) {
                std::vector<int> all(12);
                for (int j = 0; j < 12; ++j) all[j] = j;
                std::shuffle(all.begin(), all.end(), rng);
                gs[b].assign(all.begin(), all.begin() + 5);
            }
        }
        TcOffsets o{};
        o.nblocks = (uint32_t)nb;
        o.run_bits = (uint32_t)(rng() % 13);
        o.nruns = 1u << (12 - o.run_bits);
        for (int b = 0; b < nb; ++b) {
            std::shuffle(gs[b].begin(), gs[b].end(), rng);
            default_geom(o.blk[b], gs[b]);
        }
        uint32_t gates[3];
        for (int b = 0; b < nb; ++b) gates[b] = o.blk[b].jgate[31];
        int gbits[kTcMaxBlocks][5];
        if (!tc_chain_layout(o, (rng() % 3) != 0, 4, gbits)) {
            ++bad;
            continue;
        }
        int gbit0[5];
        tc_split_map(o, gbit0);
        ++chains;
        if (o.direct != 1 || o.stage_bytes % 1024u) ++bad;
        for (int b = 0; b < nb; ++b) {
            if (o.blk[b].jgate[31] != gates[b]) ++bad;
            uint32_t rows = 0;
            for (int r = 0; r < 7; ++r) rows |= o.blk[b].jrow_bit[r];
            if (rows != (0xFFFu & ~gates[b])) ++bad;
            if (b > 0)
                for (int k = 0; k < 5; ++k)
                    if (o.blk[b].jgate[1 << k] != (1u << gbits[b][k])) ++bad;
            for (int r = 0; r < 7; ++r)
                if (o.blk[b].rowoff[r] != staged(o.blk[b].jrow_bit[r], o.pad_shift)) ++bad;
            for (int g = 0; g < 32; ++g)
                if (o.blk[b].gateoff[g] != staged(o.blk[b].jgate[g], o.pad_shift)) ++bad;
        }
        bad += check_split(o);
        bool permuted = false;
        bad += check_wb_xor(o, &permuted);
        wb_permuted += permuted;
        bool free = true;
        for (int k = 0; k + 1 < nb; ++k) {
            bad += check_scatter(o, k);
            int per_bank[32] = {0}, m = 0;
            for (uint32_t l = 0; l < 32; ++l) {
                uint32_t a = 0;
                for (int i = 0; i < 5; ++i)
                    if ((l >> i) & 1u) a ^= o.scat_row[k][i];
                m = std::max(m, ++per_bank[(a >> 2) & 31u]);
            }
            free = free && m == 1;
        }
        chain_free += free;
    }
    // store boxes: every element of the box, in the box's own order, is the
    // amplitude its tile coordinate denotes, and shared-memory element
    // index = sum of 2^sbit over the coordinate's bits; a chain layout with
    // store boxes puts the last block's offsets in the chosen box's layout
    int boxes = 0, stored = 0;
    for (int trial = 0; trial < 600; ++trial) {
        const int nbits = 12 + (int)(rng() % 18);
        std::vector<int> T;
        const int nb = 2 + trial % 2;
        std::vector<std::vector<int>> gs(nb);
        int lo = (int)(rng() % (nbits - 11));
        for (int b = 0; b < nb; ++b) {
            for (int k = 0; k < 5; ++k) gs[b].push_back(lo + k);
            lo = std::min(nbits - 5, lo + 1 + (int)(rng() % 3));
        }
        for (auto& gb : gs)
            for (int p : gb)
                if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
        if (T.size() > 12) continue;
        for (int p = 0; (int)T.size() < 12; ++p)
            if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
        std::sort(T.begin(), T.end());
        auto tb = [&](int p) { return (int)(std::find(T.begin(), T.end(), p) - T.begin()); };
        uint32_t lastg = 0;
        for (int p : gs[nb - 1]) lastg |= 1u << tb(p);
        const uint64_t ncols = 1;
        const auto cands = tc_store_boxes(T.data(), nbits, ncols, lastg);
        IndexMap tm{};
        tm.nz = 12;
        for (int j = 0; j < 12; ++j) tm.zpos[j] = T[j];
        const uint64_t ntiles = (ncols << nbits) >> 12;
        for (const auto& c : cands) {
            ++boxes;
            std::vector<int> seen(12, 0);
            for (int j = 0; j < 12; ++j)
                if (c.sbit[j] < 0 || c.sbit[j] > 11 || seen[c.sbit[j]]++) ++bad;
            uint64_t elems = 1;
            for (int d = 0; d < 5; ++d) elems *= c.box.box[d];
            if (elems != 4096 || c.box.tmask[0] != 0 || c.box.gstride[0] != 8) ++bad;
            for (int k = 0; k < 3; ++k) {
                const uint64_t t = k == 0 ? 0 : (k == 1 ? ntiles - 1 : rng() % ntiles);
                const uint64_t base = expand_index(t, tm);
                uint64_t e = 0;
                for (uint64_t e4 = 0; e4 < c.box.box[4]; ++e4)
                    for (uint64_t e3 = 0; e3 < c.box.box[3]; ++e3)
                        for (uint64_t e2 = 0; e2 < c.box.box[2]; ++e2)
                            for (uint64_t e1 = 0; e1 < c.box.box[1]; ++e1)
                                for (uint64_t e0 = 0; e0 < c.box.box[0]; ++e0, ++e) {
                                    const uint64_t co[5] = {e0, e1, e2, e3, e4};
                                    uint64_t off = 0;
                                    for (int d = 0; d < 5; ++d) {
                                        const uint64_t cd = ((uint32_t)(t >> c.box.tshift[d]) & c.box.tmask[d]) + co[d];
                                        off += cd * (d ? c.box.gstride[d] / 8 : 1);
                                    }
                                    // tile coordinate of shared-memory element e
                                    uint32_t x = 0;
                                    for (int j = 0; j < 12; ++j)
                                        if ((e >> c.sbit[j]) & 1u) x |= 1u << j;
                                    uint64_t want = base;
                                    for (int j = 0; j < 12; ++j)
                                        if ((x >> j) & 1u) want |= uint64_t(1) << T[j];
                                    if (off != want) ++bad;
                                }
            }
        }
        // a chain layout over these blocks with the store boxes
        TcOffsets o{};
        o.nblocks = (uint32_t)nb;
        int L = 0;
        while (L < 12 && T[L] == L) ++L;
        o.run_bits = (uint32_t)L;
        o.nruns = 1u << (12 - L);
        for (int b = 0; b < nb; ++b) {
            std::vector<int> gbits;
            for (int p : gs[b]) gbits.push_back(tb(p));
            default_geom(o.blk[b], gbits);
        }
        int gbs[kTcMaxBlocks][5], si = -1;
        long cost = 0, ideal = 0;
        if (!tc_chain_layout(o, true, 4, gbs, &cost, &ideal, &cands, &si)) {
            ++bad;
            continue;
        }
        bool permuted = false;
        bad += check_wb_xor(o, &permuted);
        wb_permuted += permuted;
        if (si >= 0 && o.pad_shift >= 31) {
            ++stored;
            const auto& c = cands[(size_t)si];
            const TcBlockGeom& Lb = o.blk[nb - 1];
            for (uint32_t t = 0; t < 128; ++t)
                for (int g = 0; g < 32; ++g) {
                    uint32_t x = Lb.jgate[g], off = Lb.gateoff[g];
                    for (int i = 0; i < 7; ++i)
                        if ((t >> i) & 1u) {
                            x |= Lb.jrow_bit[i];
                            off += Lb.rowoff[i];
                        }
                    uint32_t e = 0;
                    for (int j = 0; j < 12; ++j)
                        if ((x >> j) & 1u) e |= 1u << c.sbit[j];
                    if (off != 8u * e) ++bad;
                }
            if ((si > 0) != (o.st_box != 0)) ++bad;
        }
    }
    // The brick circuit's pair whose last block is the tile's lowest five
    // positions (one contiguous tile: 12 positions from 0): every row of
    // that block starts on the same bank, so row-per-thread 16-byte stores
    // take 4x the minimum wavefronts.  The chain layout stores them
    // lane-permuted instead: the scatter and the write-back at the minimum
    // (64 wavefronts per warp each) plus the three butterflies of 16-byte
    // stores, unpadded.
    {
        TcOffsets o{};
        o.nblocks = 2;
        o.run_bits = 12;
        o.nruns = 1;
        default_geom(o.blk[0], {3, 4, 5, 6, 7});
        default_geom(o.blk[1], {0, 1, 2, 3, 4});
        int gbs[kTcMaxBlocks][5];
        long cost = 0, ideal = 0;
        bool permuted = false;
        if (!tc_chain_layout(o, true, 4, gbs, &cost, &ideal, nullptr, nullptr)) {
            ++bad;
        } else {
            bad += check_wb_xor(o, &permuted);
            if (!permuted || o.pad_shift < 31 || ideal != 128 || cost != 128 + 3 * 12) ++bad;
            std::printf("lowest-positions pair: cost %ld of minimum %ld, permuted %d\n", cost, ideal, (int)permuted);
        }
    }
    std::printf("bad %d trials %d conflict-free scatter %d padded %d singles %d chains %d conflict-free chains %d "
                "store boxes %d chains with a store box %d permuted write-backs %d\n",
                bad, trials, minimal, padded, singles, chains, chain_free, boxes, stored, wb_permuted);
    return bad ? 1 : 0;
}
