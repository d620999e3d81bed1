// Runs of swaps on disjoint qubit pairs as one pass (gate_plan.h,
// fuse_runs).  The swaps permute the bit positions: pi, an involution.
// Amplitudes move as out[pi(i)] = in[i], in warp tiles of 1024 amplitudes
// whose 10 positions B are closed under pi: positions 0..4 (the lane bits of
// every copy and store, so that each moves runs of 32 contiguous amplitudes),
// their partners, and the lowest other positions, partners included.  pi then
// maps tile T onto tile pi(T) (the swaps outside B act on the tile bits); a
// warp loads both tiles into its stage and writes each into the other's
// place, reading the stage through the in-tile permutation.  The stage is
// XOR-swizzled (row bits into column bits, chosen per run) so that the
// permuted reads of one phase of a warp hit distinct banks.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "kernels.h"
#include "warp_tile.cuh"

namespace q1g {

namespace {

constexpr int kSwapTileBits = 10;
constexpr size_t kSwapStageBytes = 128 * 1024;   // 2 tiles per warp: 8 warps of 8-byte, 4 of 16-byte amplitudes

template <typename E, int W>
__global__ void __launch_bounds__(W * 32, 1)
k_swap_run(E* a, uint64_t total, const SwapTile* __restrict__ gt)
{
    __shared__ SwapTile t;
    extern __shared__ uint4 swap_stage_raw[];
    {
        const uint32_t* s = reinterpret_cast<const uint32_t*>(gt);
        uint32_t* d = reinterpret_cast<uint32_t*>(&t);
        for (int i = threadIdx.x; i < (int)(sizeof(SwapTile) / 4); i += blockDim.x) d[i] = s[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    E* bufA = reinterpret_cast<E*>(swap_stage_raw) + warp * 2048;
    E* bufB = bufA + 1024;
    const uint64_t tiles = total >> kSwapTileBits;
    for (uint64_t ti = (uint64_t)blockIdx.x * W + warp; ti < tiles; ti += (uint64_t)gridDim.x * W) {
        const uint64_t base = expand_index(ti, t.tile_map);
        uint64_t base2 = base;
        for (int k = 0; k < t.nouter; ++k)
            if (((base >> t.pa[k]) ^ (base >> t.pb[k])) & 1) base2 ^= (uint64_t(1) << t.pa[k]) | (uint64_t(1) << t.pb[k]);
        if (base2 < base) continue;   // the partner tile's warp moves both
        const bool two = base2 != base;
#pragma unroll 4
        for (int m = 0; m < 32; ++m) {
            uint64_t g = 0;
#pragma unroll
            for (int b = 0; b < 5; ++b)
                if ((m >> b) & 1) g |= t.gbit[b];
            const uint32_t so = t.wphys[32 * m + lane];
            if (sizeof(E) == 8) {
                cp_async8(bufA + so, a + base + g + lane);
                if (two) cp_async8(bufB + so, a + base2 + g + lane);
            } else {
                cp_async16(bufA + so, a + base + g + lane);
                if (two) cp_async16(bufB + so, a + base2 + g + lane);
            }
        }
        cp_async_commit();
        cp_async_wait_group<0>();
        __syncwarp();
#pragma unroll 4
        for (int m = 0; m < 32; ++m) {
            uint64_t g = 0;
#pragma unroll
            for (int b = 0; b < 5; ++b)
                if ((m >> b) & 1) g |= t.gbit[b];
            const uint32_t r = t.rphys[32 * m + lane];
            a[base2 + g + lane] = bufA[r];
            if (two) a[base + g + lane] = bufB[r];
        }
        __syncwarp();
    }
}

template <typename K>
cudaError_t swap_opt_in(K kernel)
{
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(reinterpret_cast<const void*>(kernel), dev);
    if (done.count(key)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapStageBytes);
    if (e == cudaSuccess) done.insert(key);
    return e;
}

}  // namespace

bool swap_run_layout(SwapTile& t, const int* pa, const int* pb, int npairs, int nbits, int amp_bytes)
{
    std::memset(&t, 0, sizeof(t));
    if (nbits < kSwapTileBits || npairs < 1 || npairs > 32 || (amp_bytes != 8 && amp_bytes != 16)) return false;
    int perm[64];
    for (int p = 0; p < 64; ++p) perm[p] = p;
    for (int k = 0; k < npairs; ++k) {
        if (pa[k] < 0 || pb[k] < 0 || pa[k] >= nbits || pb[k] >= nbits || pa[k] == pb[k]) return false;
        if (perm[pa[k]] != pa[k] || perm[pb[k]] != pb[k]) return false;   // pairs must be disjoint
        perm[pa[k]] = pb[k];
        perm[pb[k]] = pa[k];
    }
    // tile positions: 0..4 and their partners, then the lowest other positions
    // (with their partners) up to 10
    std::vector<int> B;
    auto has = [&](int p) { return std::find(B.begin(), B.end(), p) != B.end(); };
    for (int p = 0; p < 5; ++p)
        if (!has(p)) B.push_back(p);
    for (int p = 0; p < 5; ++p)
        if (!has(perm[p])) B.push_back(perm[p]);
    for (int p = 5; p < nbits && (int)B.size() < kSwapTileBits; ++p) {
        if (has(p)) continue;
        if (perm[p] == p) B.push_back(p);
        else if ((int)B.size() <= kSwapTileBits - 2) {
            B.push_back(p);
            B.push_back(perm[p]);
        }
    }
    if ((int)B.size() != kSwapTileBits) return false;
    std::sort(B.begin(), B.end());
    int idx[64];
    for (int p = 0; p < 64; ++p) idx[p] = -1;
    for (int k = 0; k < kSwapTileBits; ++k) idx[B[k]] = k;
    // swaps outside the tile permute tile bases
    for (int k = 0; k < npairs; ++k)
        if (idx[pa[k]] < 0) {
            t.pa[t.nouter] = pa[k];
            t.pb[t.nouter] = pb[k];
            ++t.nouter;
        }
    t.tile_map.nz = kSwapTileBits;
    for (int k = 0; k < kSwapTileBits; ++k) t.tile_map.zpos[k] = B[k];
    t.tile_map.setmask = 0;
    for (int b = 0; b < 5; ++b) t.gbit[b] = uint64_t(1) << B[5 + b];
    // in-tile permutation of local indices
    auto pi_local = [&](uint32_t l) {
        uint32_t r = 0;
        for (int k = 0; k < kSwapTileBits; ++k)
            if ((l >> k) & 1) r |= 1u << idx[perm[B[k]]];
        return r;
    };
    // swizzle: one phase of a warp (consecutive lanes) reads the sources of
    // consecutive destinations, whose lane bits k < C sit at local bits
    // idx(pi(k)); row bits among those take the free column bits
    const int C = amp_bytes == 8 ? 4 : 3;
    uint32_t M[kSwapTileBits] = {};
    uint32_t used = 0;
    for (int k = 0; k < C; ++k)
        if (idx[perm[k]] < C) used |= 1u << idx[perm[k]];
    int free_col = 0;
    for (int k = 0; k < C; ++k) {
        const int src = idx[perm[k]];
        if (src < C) continue;
        while ((used >> free_col) & 1) ++free_col;
        M[src] = 1u << free_col;
        used |= 1u << free_col;
    }
    auto phys = [&](uint32_t x) {
        uint32_t r = x;
        for (int q = C; q < kSwapTileBits; ++q)
            if ((x >> q) & 1) r ^= M[q];
        return r;
    };
    for (uint32_t l = 0; l < 1024; ++l) {
        t.wphys[l] = (uint16_t)phys(l);
        t.rphys[l] = (uint16_t)phys(pi_local(l));
    }
    return true;
}

cudaError_t launch_swap_run(void* amps, int amp_bytes, uint64_t total, const void* dtile, int sm_count,
                            cudaStream_t st)
{
    const uint64_t tiles = total >> kSwapTileBits;
    if (tiles == 0) return cudaSuccess;
    const SwapTile* t = static_cast<const SwapTile*>(dtile);
    cudaError_t e;
    if (amp_bytes == 8) {
        constexpr int W = 8;
        e = swap_opt_in(k_swap_run<uint2, W>);
        if (e != cudaSuccess) return e;
        const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sm_count, (tiles + W - 1) / W);
        k_swap_run<uint2, W><<<grid, W * 32, kSwapStageBytes, st>>>((uint2*)amps, total, t);
    } else {
        constexpr int W = 4;
        e = swap_opt_in(k_swap_run<uint4, W>);
        if (e != cudaSuccess) return e;
        const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sm_count, (tiles + W - 1) / W);
        k_swap_run<uint4, W><<<grid, W * 32, kSwapStageBytes, st>>>((uint4*)amps, total, t);
    }
    return cudaGetLastError();
}

}  // namespace q1g
