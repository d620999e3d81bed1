// Dense blocks (t <= 4 targets, no controls) on one state vector in warp
// tiles (warp_tile.h): each warp of a persistent grid (one 16-warp CTA per
// SM) copies a tile asynchronously into its 8 KB stage with every copy
// instruction moving whole runs of 32 contiguous amplitudes, applies the
// block to the tile's units from the stage, and stores the tile back.
//   complex64:  1024-amplitude tiles, packed FP32x2 complex products
//               (tiled_dense_c64, shared with the batch executor).
//   complex128: 512-amplitude tiles of 16-byte amplitudes, double-float
//               products as in the complex128 pair kernel (df64.cuh); a unit
//               with an amplitude outside the split's range is done in FP64.
#include <algorithm>
#include <mutex>
#include <set>
#include <utility>

#include "df64.cuh"
#include "kernels.h"
#include "warp_tile.cuh"

namespace q1g {

namespace {

constexpr int kTiledThreads = 512;
constexpr int kTiledWarps = kTiledThreads / 32;
constexpr size_t kTiledStageBytes = size_t(kTiledWarps) * 8192;

__device__ __forceinline__ void copy_tile_words(WarpTile& dst, const WarpTile& src)
{
    static_assert(sizeof(WarpTile) % 4 == 0, "WarpTile copies as 32-bit words");
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(WarpTile) / 4); i += blockDim.x) d[i] = s[i];
}

template <int TB>
__global__ void __launch_bounds__(kTiledThreads, 1)
k_dense_tiled_c64(float2* a, uint64_t total, const __grid_constant__ WarpTile tile, const float2* __restrict__ gmat)
{
    constexpr int D = 1 << TB;
    __shared__ WarpTile w;
    __shared__ float2 mat[D * D];
    extern __shared__ float2 stage_c64[];
    copy_tile_words(w, tile);
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) mat[e] = gmat[e];
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    tiled_dense_c64<TB, false>(a, total, w, mat, stage_c64 + warp * 1024, (uint64_t)blockIdx.x * kTiledWarps + warp,
                        (uint64_t)gridDim.x * kTiledWarps);
}

// Shared-memory load of one 16-byte term, kept at its use.
__device__ __forceinline__ float4 lds_f4(const float4* p)
{
    float4 v;
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(sa));
    return v;
}

// dot_x2 over N terms whose matrix halves come from shared memory, one term
// at a time: t[k] = (ah.x, ah.y, al.x, al.y).  Lane 0 of the result is the
// real part, lane 1 the imaginary part.
template <int N>
__device__ __forceinline__ void dot_terms(const float4* t, const float2* bh, const float2* bl, float2& h, float2& l)
{
    float2 p[N], lo = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 q = lds_f4(t + k);
        const float2 ah = make_float2(q.x, q.y), al = make_float2(q.z, q.w);
        p[k] = __fmul2_rn(ah, bh[k]);
        const float2 e = __ffma2_rn(ah, bh[k], neg2(p[k]));
        lo = __fadd2_rn(lo, __ffma2_rn(al, bh[k], __ffma2_rn(ah, bl[k], e)));
    }
    float2 s = p[0];
#pragma unroll
    for (int k = 1; k < N; ++k) {
        const float2 tt = __fadd2_rn(s, p[k]);
        const float2 bv = __fadd2_rn(tt, neg2(s));
        const float2 av = __fadd2_rn(tt, neg2(bv));
        lo = __fadd2_rn(lo, __fadd2_rn(__fadd2_rn(s, neg2(av)), __fadd2_rn(p[k], neg2(bv))));
        s = tt;
    }
    h = __fadd2_rn(s, lo);
    const float2 bv = __fadd2_rn(h, neg2(s));
    const float2 av = __fadd2_rn(h, neg2(bv));
    l = __fadd2_rn(__fadd2_rn(s, neg2(av)), __fadd2_rn(lo, neg2(bv)));
}

// Complex128 tiles: terms[r * 2D + 2s] = (m.re, m.re) and
// terms[r * 2D + 2s + 1] = (-m.im, m.im) as (hi, lo) float pairs against the
// inputs (x.re, x.im) and (x.im, x.re); mat is the FP64 matrix for units the
// split cannot take.
template <int TB>
__global__ void __launch_bounds__(kTiledThreads, 1)
k_dense_tiled_c128(double2* a, uint64_t total, const __grid_constant__ WarpTile tile,
                   const float4* __restrict__ gterms, const double2* __restrict__ gmat)
{
    constexpr int D = 1 << TB;
    constexpr int U = 16 >> TB;   // units per lane in a 512-amplitude tile
    __shared__ WarpTile w;
    __shared__ float4 terms[2 * D * D];
    __shared__ double2 mat[D * D];
    extern __shared__ ulonglong2 stage_c128[];
    copy_tile_words(w, tile);
    for (int e = threadIdx.x; e < 2 * D * D; e += blockDim.x) terms[e] = gterms[e];
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) mat[e] = gmat[e];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ulonglong2* stage = stage_c128 + warp * 512;
    ulonglong2* ab = reinterpret_cast<ulonglong2*>(a);
    const uint64_t tiles = total >> 9;
    const uint32_t plane = lane_phys(w, lane);
    uint32_t pl = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b)
        if ((lane >> b) & 1) pl ^= w.wbit[b];
    for (uint64_t t = (uint64_t)blockIdx.x * kTiledWarps + warp; t < tiles; t += (uint64_t)gridDim.x * kTiledWarps) {
        uint32_t gb[4], sb[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            gb[b] = lds_u32(&w.gbit[b]);
            sb[b] = lds_u32(&w.sbit[b]);
        }
        ulonglong2* amps = ab + expand_index(t, w.tile_map) + lane;
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            uint32_t g = 0, so = plane;
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if ((m >> b) & 1) {
                    g |= gb[b];
                    so ^= sb[b];
                }
            cp_async16(stage + so, amps + g);
        }
        cp_async_commit();
        cp_async_wait_group<0>();
        __syncwarp();
#pragma unroll 1
        for (int k = 0; k < U; ++k) {
            uint32_t o = pl;
#pragma unroll
            for (int b = 0; b < 4 - TB; ++b)
                if ((k >> b) & 1) o ^= w.wbit[5 + b];
            ulonglong2 x[D];
            bool fast = true;
#pragma unroll
            for (int s = 0; s < D; ++s) {
                x[s] = stage[o ^ w.gsoff[s]];
                fast = fast & split_fast_ok(x[s].x) & split_fast_ok(x[s].y);
            }
            float2 bh[2 * D], bl[2 * D];
            bool ok = true;
#pragma unroll
            for (int s = 0; s < D; ++s) {
                DF re, im;
                if (fast) {
                    re = split_fast(x[s].x);
                    im = split_fast(x[s].y);
                } else {
                    ok = ok & split_f64(x[s].x, re) & split_f64(x[s].y, im);
                }
                bh[2 * s] = make_float2(re.h, im.h);
                bl[2 * s] = make_float2(re.l, im.l);
                bh[2 * s + 1] = make_float2(im.h, re.h);
                bl[2 * s + 1] = make_float2(im.l, re.l);
            }
            if (ok) {
#pragma unroll 1
                for (int r = 0; r < D; ++r) {
                    float2 h, l;
                    dot_terms<2 * D>(terms + r * 2 * D, bh, bl, h, l);
                    stage[o ^ w.gsoff[r]] = make_ulonglong2(join_f64(DF{h.x, l.x}), join_f64(DF{h.y, l.y}));
                }
            } else {
                double2 y[D];
#pragma unroll
                for (int s = 0; s < D; ++s) y[s] = *reinterpret_cast<const double2*>(&x[s]);
#pragma unroll 1
                for (int r = 0; r < D; ++r) {
                    double re = 0.0, im = 0.0;
#pragma unroll
                    for (int s = 0; s < D; ++s) {
                        const double2 m = mat[r * D + s];
                        re = fma(m.x, y[s].x, fma(-m.y, y[s].y, re));
                        im = fma(m.x, y[s].y, fma(m.y, y[s].x, im));
                    }
                    const double2 out = make_double2(re, im);
                    stage[o ^ w.gsoff[r]] = *reinterpret_cast<const ulonglong2*>(&out);
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            uint32_t g = 0, so = plane;
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if ((m >> b) & 1) {
                    g |= gb[b];
                    so ^= sb[b];
                }
            amps[g] = stage[so];
        }
        __syncwarp();
    }
}

// Opts a kernel in to the 128 KB stage, once per kernel and device.
template <typename K>
cudaError_t opt_in(K kernel)
{
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(reinterpret_cast<const void*>(kernel), dev);
    if (done.count(key)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTiledStageBytes);
    if (e == cudaSuccess) done.insert(key);
    return e;
}

}  // namespace

bool dense_tiled_applies(int prec, int nbits, int t, const IndexMap& map, bool fp64_exact)
{
    if (map.nz != t || map.setmask != 0) return false;   // controls: the per-unit kernel
    if (prec == kC128) return !fp64_exact && t >= 1 && t <= 3 && nbits >= 9;
    // complex64: the per-unit kernel is coalesced, and faster, for 1- and
    // 2-qubit blocks whose gate positions are all >= 2
    return t >= 1 && t <= 4 && nbits >= 10 && (t >= 3 || map.zpos[0] <= 1);
}

size_t dense_tiled_matrix_bytes(int prec, int t)
{
    const size_t d2 = size_t(1) << (2 * t);
    return prec == kC128 ? 2 * d2 * sizeof(float4) + d2 * sizeof(double2) : d2 * sizeof(float2);
}

void dense_tiled_matrix(int prec, int t, const double* m, void* out)
{
    const size_t d = size_t(1) << t;
    if (prec != kC128) {
        float2* f = static_cast<float2*>(out);
        for (size_t e = 0; e < d * d; ++e) f[e] = make_float2((float)m[2 * e], (float)m[2 * e + 1]);
        return;
    }
    float4* terms = static_cast<float4*>(out);
    double2* md = reinterpret_cast<double2*>(terms + 2 * d * d);
    for (size_t r = 0; r < d; ++r)
        for (size_t s = 0; s < d; ++s) {
            const double re = m[2 * (r * d + s)], im = m[2 * (r * d + s) + 1];
            const DF hr = host_split(re), hi = host_split(im);
            terms[r * 2 * d + 2 * s] = make_float4(hr.h, hr.h, hr.l, hr.l);
            terms[r * 2 * d + 2 * s + 1] = make_float4(-hi.h, hi.h, -hi.l, hi.l);
            md[r * d + s] = make_double2(re, im);
        }
}

cudaError_t launch_dense_tiled(void* amps, int prec, uint64_t total, int nbits, const IndexMap& map,
                               const DenseOffsets& offs, int t, const void* dmat, int sm_count, cudaStream_t st)
{
    WarpTile w;
    const bool c128 = prec == kC128;
    warp_tile_layout(w, map.zpos, t, offs.off, nbits, c128 ? 9 : 10, c128 ? 3 : 4);
    if (!w.tiled) return cudaErrorInvalidValue;
    const uint64_t tiles = total >> w.tile_bits;
    const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sm_count, (tiles + kTiledWarps - 1) / kTiledWarps);
    if (grid == 0) return cudaSuccess;
    cudaError_t e = cudaSuccess;
#define Q1G_TILED_C64(TBV)                                                                                    \
    case TBV:                                                                                                 \
        e = opt_in(k_dense_tiled_c64<TBV>);                                                                   \
        if (e == cudaSuccess)                                                                                 \
            k_dense_tiled_c64<TBV><<<grid, kTiledThreads, kTiledStageBytes, st>>>((float2*)amps, total, w,     \
                                                                                  (const float2*)dmat);       \
        break;
#define Q1G_TILED_C128(TBV)                                                                                   \
    case TBV:                                                                                                 \
        e = opt_in(k_dense_tiled_c128<TBV>);                                                                  \
        if (e == cudaSuccess)                                                                                 \
            k_dense_tiled_c128<TBV><<<grid, kTiledThreads, kTiledStageBytes, st>>>(                           \
                (double2*)amps, total, w, (const float4*)dmat,                                                \
                (const double2*)((const float4*)dmat + 2 * (1 << (2 * TBV))));                                \
        break;
    if (c128) {
        switch (t) {
            Q1G_TILED_C128(1)
            Q1G_TILED_C128(2)
            Q1G_TILED_C128(3)
            default:
                return cudaErrorInvalidValue;
        }
    } else {
        switch (t) {
            Q1G_TILED_C64(1)
            Q1G_TILED_C64(2)
            Q1G_TILED_C64(3)
            Q1G_TILED_C64(4)
            default:
                return cudaErrorInvalidValue;
        }
    }
#undef Q1G_TILED_C64
#undef Q1G_TILED_C128
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace q1g
