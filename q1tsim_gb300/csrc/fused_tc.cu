// Fused 5-qubit blocks as tensor-core contractions (complex64 state, 3xTF32).
//
// A fused block is a dense 32x32 complex matrix M on five qubits (gate
// positions p_0 > ... > p_4).  The state is cut into tiles of 2^12
// amplitudes: the 5 gate positions plus the 7 lowest other positions
// ("row" positions); the remaining positions enumerate the tiles.  In a tile,
// row t (0..127) holds the 32 amplitudes of one group, so the update is the
// real GEMM
//     D[t][n] = sum_k A[t][k] * R[n][k],   A[t][2g+c] = component c of amp(t, g),
// with R the 64x64 real embedding of M (R[2g'][2g] = Re M, R[2g'][2g+1] = -Im M,
// R[2g'+1][2g] = Im M, R[2g'+1][2g+1] = Re M).  It runs on tcgen05.mma
// kind::tf32 (M=128, N=64, K=8) with the accumulator in TMEM.  FP32 accuracy
// comes from the 3xTF32 split (Ootomo & Yokota 2022): x = hi + lo with
// hi = tf32(x), lo = tf32(x - hi), and D = A_hi*B_hi + (A_lo*B_hi + A_hi*B_lo).
// The correction products go to a second TMEM accumulator with the lo halves
// pre-scaled by 2^11 (exact), and the epilogue adds D_corr * 2^-11: summed in
// one accumulator with the main products, the correction terms were lost.
//
// One CTA = 4 warps; thread t owns row t: it loads its 32 amplitudes (for a
// fixed g the warp reads 32 consecutive row positions, so loads and stores
// are coalesced), writes the hi/lo halves into the K-major SWIZZLE_128B
// operand tiles in shared memory, and after the MMAs reads its TMEM lane
// back with tcgen05.ld and stores the 32 results in place.  The next tile's
// loads are issued before waiting on the current tile's MMAs.  B (the block's
// hi/lo image, 32 KB) is prepared on the host in the same swizzled layout.
// Every mbarrier wait is bounded: on expiry the kernel records an error and
// releases its TMEM before returning.
#include <cuda_runtime.h>

#include <cstring>

#include "common.cuh"
#include "kernels.h"

namespace q1g {

namespace {

constexpr int kTcThreads = 128;
constexpr uint32_t kTmemCols = 128;   // D_main in columns 0-63, D_corr in 64-127
constexpr float kLoScale = 2048.0f;     // 2^11: lo halves are stored scaled up
constexpr float kLoUnscale = 1.0f / 2048.0f;
constexpr uint32_t kAtomA = 16384;   // 128 rows x 128 B
constexpr uint32_t kAtomB = 8192;    // 64 rows x 128 B
constexpr uint32_t kOffAhi = 0;
constexpr uint32_t kOffAlo = 2 * kAtomA;
constexpr uint32_t kOffBhi = 4 * kAtomA;
constexpr uint32_t kOffBlo = 4 * kAtomA + 2 * kAtomB;
constexpr uint32_t kOffBar = 4 * kAtomA + 4 * kAtomB;   // mbarrier (8 B) + TMEM slot (4 B)
constexpr uint32_t kSmemBytes = kOffBar + 64 + 1024;     // + alignment slack
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// SMEM matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for this layout)
    d |= (uint64_t)(1024u >> 4) << 32;       // stride byte offset
    d |= (uint64_t)1 << 46;                  // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major, N=64, M=128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// Nearest TF32 value (ties away from zero) as an FP32 with the 13 low
// mantissa bits cleared, so that x - to_tf32(x) is the exact remainder.
__device__ __forceinline__ float to_tf32(float x)
{
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// Byte offset of tile coordinate j in the staging buffer: 16-byte chunks
// (two amplitudes) XOR-swizzled by higher chunk bits, so that both the row
// scatter and the linear read-out spread over the banks.
__device__ __forceinline__ uint32_t stage_off(uint32_t j)
{
    const uint32_t c = j >> 1;
    const uint32_t pc = c ^ ((c >> 3) & 7u) ^ ((c >> 6) & 7u);
    return (pc << 4) | ((j & 1u) << 3);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
          "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
          "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
          "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

__global__ void __launch_bounds__(kTcThreads, 2)
k_fused_tc(float2* __restrict__ a, uint64_t ntiles, IndexMap tilemap, TcOffsets offs,
           const uint4* __restrict__ bimage, int* __restrict__ err)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_addr(smem);
    const uint32_t bar = sbase + kOffBar;
    uint32_t* tmem_slot = (uint32_t*)(smem + kOffBar + 8);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;

    // B image (hi and lo, 32 KB) into shared memory.
    {
        uint4* dst = (uint4*)(smem + kOffBhi);
        for (int i = tid; i < (int)(4 * kAtomB / 16); i += kTcThreads) dst[i] = bimage[i];
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // Tile coordinate j (12 bits) <-> tile positions tpos[b]; bit 0 of j is
    // always position 0.  Thread tid moves the amplitude pairs
    // j = 2*(tid + 128*k) + {0,1}, k = 0..15: consecutive threads touch
    // consecutive 16-byte words of global memory.  (row t, gate g) of j is the
    // OR of the contributions of its set bits.
    uint64_t a_tid = 0;
    uint32_t t_tid = 0, g_tid = 0;
#pragma unroll
    for (int b = 1; b < 8; ++b)
        if ((tid >> (b - 1)) & 1) {
            a_tid |= uint64_t(1) << offs.tpos[b];
            t_tid |= offs.rowmask[b];
            g_tid |= offs.gatemask[b];
        }
    const uint32_t t_e = offs.rowmask[0], g_e = offs.gatemask[0];
    // tile coordinate of (row tid, g = 0), for staging the results
    uint32_t jrow = 0;
#pragma unroll
    for (int r = 0; r < 7; ++r)
        if ((tid >> r) & 1) jrow |= offs.row_tbit[r];
    uint8_t* const stage = smem + kOffAlo;   // A_lo is free once the MMAs are done

    float4 x[16];
    uint64_t tile = blockIdx.x;
    uint64_t base = tile < ntiles ? expand_index(tile, tilemap) : 0;
    if (tile < ntiles) {
#pragma unroll
        for (int k = 0; k < 16; ++k) x[k] = *reinterpret_cast<const float4*>(a + (base | a_tid | offs.koff[k]));
    }
    uint32_t phase = 0;
    bool failed = false;
    for (; tile < ntiles; tile += gridDim.x) {
        // operand A: hi and lo' halves, scattered into the swizzled K-major rows
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const uint32_t tk = t_tid | offs.krow[k], gk = g_tid | offs.kgate[k];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const uint32_t t = e ? (tk | t_e) : tk;
                const uint32_t g = e ? (gk | g_e) : gk;
                const float vx = e ? x[k].z : x[k].x, vy = e ? x[k].w : x[k].y;
                const float hx = to_tf32(vx), hy = to_tf32(vy);
                const float2 h = make_float2(hx, hy);
                const float2 l = make_float2(to_tf32((vx - hx) * kLoScale), to_tf32((vy - hy) * kLoScale));
                const uint32_t off = (g >> 4) * kAtomA + (t >> 3) * 1024u + (t & 7u) * 128u +
                                     ((((g & 15u) >> 1) ^ (t & 7u)) << 4) + (g & 1u) * 8u;
                *(float2*)(smem + kOffAhi + off) = h;
                *(float2*)(smem + kOffAlo + off) = l;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // pass 0: D_main = A_hi B_hi; passes 1-2: D_corr = A_lo' B_hi + A_hi B_lo'
            // (lo' = 2^11 lo), kept apart so the small terms never meet the large
            // ones inside one accumulation.
            const uint32_t apass[3] = {sbase + kOffAhi, sbase + kOffAlo, sbase + kOffAhi};
            const uint32_t bpass[3] = {sbase + kOffBhi, sbase + kOffBhi, sbase + kOffBlo};
            const uint32_t dcol[3] = {0u, 64u, 64u};
#pragma unroll
            for (int pss = 0; pss < 3; ++pss)
#pragma unroll
                for (int ks = 0; ks < 8; ++ks) {
                    const uint32_t ka = (uint32_t)(ks >> 2) * kAtomA + (uint32_t)(ks & 3) * 32u;
                    const uint32_t kb = (uint32_t)(ks >> 2) * kAtomB + (uint32_t)(ks & 3) * 32u;
                    const uint32_t acc = (pss == 2 || ks != 0) ? 1u : 0u;
                    mma_tf32(tmem + dcol[pss], desc_sw128(apass[pss] + ka), desc_sw128(bpass[pss] + kb), acc);
                }
            mma_commit(bar);
        }
        // prefetch the next tile while the tensor cores work
        const uint64_t cur = base;
        const uint64_t next = tile + gridDim.x;
        if (next < ntiles) {
            base = expand_index(next, tilemap);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                x[k] = *reinterpret_cast<const float4*>(a + (base | a_tid | offs.koff[k]));
        }
        uint32_t spins = 0;
        bool ok = true;
        while (!mbar_try_wait(bar, phase)) {
            if (++spins > kSpinLimit) {
                ok = false;
                break;
            }
        }
        // one decision for the whole CTA, so every thread leaves together
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(err, 1);
            failed = true;
            break;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // row tid of D = D_main + 2^-11 D_corr, staged in tile-coordinate order
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t dm[32], dc[32];
            tmem_ld32(taddr + 32u * half, dm);
            tmem_ld32(taddr + 64u + 32u * half, dc);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int g = 16 * half + j;
                const float re = __fmaf_rn(__uint_as_float(dc[2 * j]), kLoUnscale, __uint_as_float(dm[2 * j]));
                const float im =
                    __fmaf_rn(__uint_as_float(dc[2 * j + 1]), kLoUnscale, __uint_as_float(dm[2 * j + 1]));
                const uint32_t jc = jrow | offs.jgate[g];
                *(float2*)(stage + stage_off(jc)) = make_float2(re, im);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const uint32_t jc = 2u * (uint32_t)tid + 256u * (uint32_t)k;
            *reinterpret_cast<float4*>(a + (cur | a_tid | offs.koff[k])) =
                *reinterpret_cast<const float4*>(stage + stage_off(jc));
        }
        __syncthreads();   // staging read out before the next split overwrites it
    }
    if (failed) {
        // give the outstanding MMAs a second bounded chance to finish before
        // the accumulator is released
        uint32_t spins = 0;
        while (!mbar_try_wait(bar, phase) && ++spins <= kSpinLimit) {
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

uint32_t fused_tc_smem_bytes() { return kSmemBytes; }

namespace {
// Round to TF32 the way cvt.rna.tf32.f32 does: nearest, ties away from zero.
float host_tf32(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
}  // namespace

void build_tc_image(const double* m, float* image)
{
    // R[n][k]: n = 2g'+c' output component, k = 2g+c input component
    for (int gp = 0; gp < 32; ++gp)
        for (int g = 0; g < 32; ++g) {
            const double re = m[2 * (gp * 32 + g)], im = m[2 * (gp * 32 + g) + 1];
            const double rv[2][2] = {{re, -im}, {im, re}};
            for (int cp = 0; cp < 2; ++cp)
                for (int c = 0; c < 2; ++c) {
                    const int n = 2 * gp + cp, k = 2 * g + c;
                    const float v = (float)rv[cp][c];
                    const float hi = host_tf32(v);
                    const float lo = host_tf32((v - hi) * 2048.0f);
                    const int atom = k >> 5, kc = (k & 31) >> 2, e = k & 3;
                    const size_t off = (size_t)atom * kAtomB + (size_t)(n >> 3) * 1024 + (size_t)(n & 7) * 128 +
                                       (size_t)((kc ^ (n & 7)) << 4) + (size_t)e * 4;
                    image[off / 4] = hi;
                    image[(2 * kAtomB + off) / 4] = lo;
                }
        }
}

cudaError_t launch_fused_tc(float2* amps, uint64_t ntiles, const IndexMap& tilemap, const TcOffsets& offs,
                            const void* d_bimage, int* d_err, int sm_count, cudaStream_t st)
{
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_fused_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmemBytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    uint64_t grid = (uint64_t)sm_count * 2;
    if (grid > ntiles) grid = ntiles;
    if (grid == 0) return cudaSuccess;
    k_fused_tc<<<(unsigned)grid, kTcThreads, kSmemBytes, st>>>(amps, ntiles, tilemap, offs,
                                                               (const uint4*)d_bimage, d_err);
    return cudaGetLastError();
}

}  // namespace q1g
