// Device side of the warp tiles (warp_tile.h): asynchronous copies,
// shared-memory loads kept at their use, and the complex64 tile pass shared
// by the batch executor and the single-state tiled dense kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "warp_tile.h"

namespace q1g {

// 8- and 16-byte asynchronous copies global -> shared, committed in groups;
// the issuing lane's copies of all but the newest N groups are complete
// after cp_async_wait_group<N>
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Shared-memory load of a 32-bit value that the compiler may not hoist out of
// its loop.
__device__ __forceinline__ uint32_t lds_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(v) : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}

// Shared-memory load of one matrix entry (re, im), kept at its use: a plain
// load of the (loop-invariant) matrix would be hoisted out of the tile loop
// into as many registers as the matrix has entries.  All lanes read the same
// entry, so the load is one broadcast wavefront.
__device__ __forceinline__ float2 lds_entry(const float2* p)
{
    float2 v;
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(sa));
    return v;
}

// Complex products on packed FP32x2 FMAs with the matrix entry m = (re, im)
// as one operand: with xa = (x.re, x.re) and xb = (x.im, x.im),
//   a += xa * m = (x.re m.re, x.re m.im),  b += xb * m = (x.im m.re, x.im m.im),
// and sum m x = (a.x - b.y, a.y + b.x).  An entry is read as 8 bytes and
// serves every unit a lane holds; the inputs are duplicated once per unit.
__device__ __forceinline__ float2 cdot_out(float2 a, float2 b) { return make_float2(a.x - b.y, a.y + b.x); }

// Staged offset of lane l: XOR of the lane-bit offsets.
__device__ __forceinline__ uint32_t lane_phys(const WarpTile& w, int lane)
{
    uint32_t p = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b)
        if ((lane >> b) & 1) p ^= w.lphys[b];
    return p;
}

// Complex64 tile pass over tiles t0, t0 + tstride, ... of a state of
// n_amps amplitudes (tile_bits 10: 1024 amplitudes, 8 KB of stage per warp).
// w and mat (row-major 2^TB x 2^TB entries) are in shared memory.  A tile is
// copied asynchronously into the warp's stage: 8 bytes per lane and slot, or,
// where w.pairs16, 16 bytes covering two slots.  The 16-byte form saves
// instructions where the arithmetic is heavy (4-qubit blocks); on one state,
// lighter blocks measured faster with the 8-byte copies, so PAIRS_ANY_TB
// false keeps it to 4-qubit blocks.  Each lane then applies the block
// to 32 / 2^TB units, KB units and RB rows at a time so that one matrix entry
// read serves KB units and 2 KB RB FMA chains are in flight, and the tile is
// stored back.  Warps never synchronise with one another.
template <int TB, bool PAIRS_ANY_TB>
__device__ void tiled_dense_c64(float2* a, uint64_t n_amps, const WarpTile& w, const float2* mat, float2* stage,
                                uint64_t t0, uint64_t tstride)
{
    constexpr int D = 1 << TB;
    constexpr int U = 32 >> TB;
    constexpr int KB = U < 2 ? U : 2;
    constexpr int RB = TB >= 3 ? 2 : 1;
    const int lane = threadIdx.x & 31;
    const uint64_t tiles = n_amps >> 10;
    const uint32_t plane = lane_phys(w, lane);
    // 16-byte form: lane l moves amplitudes 2i, 2i+1 (i = l & 15) of slot 2mm + (l >> 4)
    uint32_t p16 = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b)
        if ((lane >> b) & 1) p16 ^= w.lphys[b + 1];
    uint32_t pl = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b)
        if ((lane >> b) & 1) pl ^= w.wbit[b];

    for (uint64_t t = t0; t < tiles; t += tstride) {
        // slot offsets from the five basis values, read per tile (volatile)
        // so that the 64 derived offsets are not kept in registers across tiles
        uint32_t gb[5], sb[5];
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            gb[b] = lds_u32(&w.gbit[b]);
            sb[b] = lds_u32(&w.sbit[b]);
        }
        float2* amps = a + expand_index(t, w.tile_map);
        if ((PAIRS_ANY_TB || TB == 4) && w.pairs16) {
            const uint32_t gh = (lane & 16) ? gb[0] : 0u, sh = p16 ^ ((lane & 16) ? sb[0] : 0u);
            const float2* src = amps + 2 * (lane & 15) + gh;
#pragma unroll
            for (int mm = 0; mm < 16; ++mm) {
                uint32_t g = 0, so = sh;
#pragma unroll
                for (int b = 1; b < 5; ++b)
                    if ((mm >> (b - 1)) & 1) {
                        g |= gb[b];
                        so ^= sb[b];
                    }
                cp_async16(stage + so, src + g);
            }
        } else {
            const float2* src = amps + lane;
#pragma unroll
            for (int m = 0; m < 32; ++m) {
                uint32_t g = 0, so = plane;
#pragma unroll
                for (int b = 0; b < 5; ++b)
                    if ((m >> b) & 1) {
                        g |= gb[b];
                        so ^= sb[b];
                    }
                cp_async8(stage + so, src + g);
            }
        }
        cp_async_commit();
        cp_async_wait_group<0>();
        __syncwarp();
#pragma unroll 1
        for (int k0 = 0; k0 < U; k0 += KB) {
            uint32_t pw[KB];
            float2 xa[KB][D], xb[KB][D];
#pragma unroll
            for (int k = 0; k < KB; ++k) {
                uint32_t o = pl;
#pragma unroll
                for (int b = 0; b < 5 - TB; ++b)
                    if (((k0 + k) >> b) & 1) o ^= w.wbit[5 + b];
                pw[k] = o;
#pragma unroll
                for (int s = 0; s < D; ++s) {
                    const float2 v = stage[o ^ w.gsoff[s]];
                    xa[k][s] = make_float2(v.x, v.x);
                    xb[k][s] = make_float2(v.y, v.y);
                }
            }
#pragma unroll
            for (int r = 0; r < D; r += RB) {
                float2 ac[RB][KB], bc[RB][KB];
#pragma unroll
                for (int q = 0; q < RB; ++q)
#pragma unroll
                    for (int k = 0; k < KB; ++k) ac[q][k] = bc[q][k] = make_float2(0.f, 0.f);
#pragma unroll
                for (int s = 0; s < D; ++s) {
#pragma unroll
                    for (int q = 0; q < RB; ++q) {
                        const float2 e = lds_entry(mat + (r + q) * D + s);
#pragma unroll
                        for (int k = 0; k < KB; ++k) {
                            ac[q][k] = __ffma2_rn(xa[k][s], e, ac[q][k]);
                            bc[q][k] = __ffma2_rn(xb[k][s], e, bc[q][k]);
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < RB; ++q) {
                    const uint32_t g = w.gsoff[r + q];
#pragma unroll
                    for (int k = 0; k < KB; ++k) stage[pw[k] ^ g] = cdot_out(ac[q][k], bc[q][k]);
                }
            }
        }
        __syncwarp();
        if ((PAIRS_ANY_TB || TB == 4) && w.pairs16) {
            const uint32_t gh = (lane & 16) ? gb[0] : 0u, sh = p16 ^ ((lane & 16) ? sb[0] : 0u);
            float2* dst = amps + 2 * (lane & 15) + gh;
#pragma unroll
            for (int mm = 0; mm < 16; ++mm) {
                uint32_t g = 0, so = sh;
#pragma unroll
                for (int b = 1; b < 5; ++b)
                    if ((mm >> (b - 1)) & 1) {
                        g |= gb[b];
                        so ^= sb[b];
                    }
                *reinterpret_cast<float4*>(dst + g) = *reinterpret_cast<const float4*>(stage + so);
            }
        } else {
            float2* dst = amps + lane;
#pragma unroll
            for (int m = 0; m < 32; ++m) {
                uint32_t g = 0, so = plane;
#pragma unroll
                for (int b = 0; b < 5; ++b)
                    if ((m >> b) & 1) {
                        g |= gb[b];
                        so ^= sb[b];
                    }
                dst[g] = stage[so];
            }
        }
        __syncwarp();
    }
}

}  // namespace q1g
