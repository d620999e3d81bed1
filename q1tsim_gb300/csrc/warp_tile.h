// Warp tiles of a dense block: the layout shared by the batch executor and
// the single-state tiled dense kernels.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace q1g {

// A warp streams tiles of 2^tile_bits amplitudes.  The tile's positions are
// the block's gate positions plus the lowest other positions, so positions
// 0..4 always belong to it (at most four are gate positions): they are the
// lane bits, and the remaining tile positions are register slots (slot m of
// lane l is amplitude tile_base + goff(m) + l, goff(m) = OR of gbit[b] over the
// set bits b of m).  Every copy and store instruction of a warp therefore
// moves whole runs of 32 contiguous amplitudes whatever the gate positions.
//
// In the warp's stage an amplitude sits at the swizzled offset of its local
// index (local bit k = the tile's k-th position).  A row holds 2^col_bits
// amplitudes (128 bytes); the row bits are XOR-ed into the column bits so
// that the 2^col_bits units a phase of a warp reads for one gate state (16
// lanes of 8-byte reads, 8 lanes of 16-byte reads) land in distinct bank
// groups: a unit's lowest col_bits number bits go to distinct column bits.
// The staged offset is linear (XOR) in the local index, so it is the XOR of
// per-bit offsets: lphys (lane bits), sbit (slot bits), wbit (unit-number
// bits) and gsoff (gate states).
struct WarpTile {
    int tiled;                // 0: the state has fewer than tile_bits qubits (or no block)
    int tile_bits;            // 10 for 8-byte amplitudes, 9 for 16-byte amplitudes
    int pairs16;              // 8-byte amplitudes with position 0 not a gate position: the
                              // swizzle keeps pairs (2i, 2i+1) adjacent and 16-byte aligned
    int pad_;
    uint32_t lphys[5];        // staged offset of lane bit b
    uint32_t gbit[5];         // amplitude offset of slot bit b
    uint32_t sbit[5];         // staged offset of slot bit b
    uint32_t pad2_;
    uint16_t gsoff[16];       // staged offset of gate state s (offs[s] inside the tile)
    uint16_t wbit[10];        // staged offset of bit b of a unit's number in the tile
    uint16_t pad3_[2];
    IndexMap tile_map;        // the tile's positions, zeroed: tile number -> first amplitude
};

// Layout for gate positions pos[0..tb) whose gate state s sits at amplitude
// offset offs[s], on a state of nbits qubits.  tile_bits 10 / col_bits 4 for
// complex64, 9 / 3 for complex128.  w.tiled = 0 when nbits < tile_bits or tb
// is outside 1..4.
void warp_tile_layout(WarpTile& w, const int* pos, int tb, const uint64_t* offs, int nbits, int tile_bits,
                      int col_bits);

}  // namespace q1g
