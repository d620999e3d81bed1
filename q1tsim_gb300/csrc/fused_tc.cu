// Fused 5-qubit blocks as tensor-core contractions (complex64 state, f16
// operand halves, FP32 accuracy).
//
// A fused block is a dense 32x32 complex matrix M on five qubits (gate
// positions p_0 > ... > p_4).  The state is cut into tiles of 2^12
// amplitudes: the 5 gate positions plus 7 other positions ("row"
// positions); the remaining positions enumerate the tiles.  In a tile, row t
// (0..127) holds the 32 amplitudes of one group, so the update is the real
// GEMM
//     D[t][n] = sum_k A[t][k] * R[n][k],   A[t][2g+c] = component c of amp(t, g),
// with R the 64x64 real embedding of M (R[2g'][2g] = Re M, R[2g'][2g+1] = -Im M,
// R[2g'+1][2g] = Im M, R[2g'+1][2g+1] = Re M).  It runs on tcgen05.mma
// kind::f16 (M=128, K=16, FP32 accumulators) with A and the accumulators in
// tensor memory and R in shared memory.  FP32 accuracy comes from splitting
// both operands into two 11-bit halves (the 3-product scheme of Ootomo &
// Yokota 2022): x = hi + lo with hi = x to 11 significant bits and
// lo = x - hi, and D = A_hi*B_hi + (A_lo*B_hi + A_hi*B_lo).  Halves are f16,
// so one 32-bit TMEM column holds one complex amplitude and a row's operands
// take 64 columns.  f16 has a narrow exponent range, so the operands are
// scaled by powers of two: amplitudes by 2^14 / 2^ceil(log2 sqrt(max column
// norm)) (at most 2^14 in magnitude for blocks whose rows have 2-norm <= 1)
// as the first block of a pass reads them; they stay scaled into the second
// block (whose R is not scaled), and the last block's R is scaled by 2^14
// and its epilogue undoes both exactly.  The correction products go to
// a second accumulator with the lo halves pre-scaled by 2^11 (exact), and the
// epilogue adds D_corr * 2^-11: summed in one accumulator with the main
// products, the correction terms were lost.  B is stored as [B_hi; B_lo]
// (128 rows of 64 f16), so A_hi*[B_hi; B_lo] is one N=128 product into
// [D_main | D_corr] and A_lo*B_hi one N=64 product added to D_corr:
// 8 MMAs per block and tile.
//
// One CTA per SM, persistent over tiles, with 11 warps:
//   warp 8   loader: copies a tile into a ring of shared-memory stages,
//            completing on the stage's `full` mbarrier.  An unpadded tile is
//            one box of a rank-5 tensor map over the state (one
//            cp.async.bulk.tensor per tile); a padded one goes in pieces of
//            2^piece_bits amplitudes with cp.async.bulk (many small copies
//            cost bandwidth: 32 x 1 KB reach about 75% of one 32 KB copy);
//   warps 9-10  storers, alternate tiles: when a tile is done, store it back
//            and, once the copy has read the stage, free it on its `empty`
//            mbarrier (two storers keep two stores in flight while each
//            frees its stage without delay);
//   warps 0-3 and 4-7: two consumer groups taking alternate tiles.  Each
//            thread owns one row t (its TMEM lane): it reads the row's 32
//            amplitudes from the stage, writes hi/lo to its group's A columns
//            with tcgen05.st (the MMAs of the first half's K-steps start
//            while the second half converts), one thread issues the MMAs, and after the commit
//            each thread reads its row of D with tcgen05.ld and writes the
//            new amplitudes back into the stage.  While one group waits for
//            its MMAs the other converts or writes back, so the tensor pipe,
//            the ALUs and the copy engine work at the same time.
// TMEM (512 columns): group g uses 256g + [0,64) for A (K-step s: A_hi pairs
// in columns 16s..16s+7, A_lo pairs in 16s+8..16s+15, so that a thread writes
// half a row with one 32-column store), [128,192) D_main, [192,256) D_corr.
// Every wait is bounded (in wall-clock time, %globaltimer); on expiry the CTA
// records an error, lets its copies land and releases its TMEM before
// returning.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "f16_host.h"
#include "kernels.h"

namespace q1g {

namespace {

constexpr int kGroupThreads = 128;              // 4 warps: one per TMEM lane quarter
// The kernel comes in two shapes, by its number of consumer groups NG:
//   NG = 2: each group's A operand (of a pass's first block, and of every
//           block in the staged and shuffled pair modes) in TMEM beside its
//           accumulators, 256 columns per group;
//   NG = 4: every A operand in the group's stage in shared memory (the
//           first block's split writes it there over the tile it has read),
//           only the accumulators in TMEM, 128 columns per group, so that
//           four tiles are in flight per SM.
// Warps 0 .. 4NG-1 are the consumers, then the loader and two storers.
template <int NG>
struct TcShape {
    static constexpr int kLoaderWarp = 4 * NG;
    static constexpr int kStorerWarp0 = 4 * NG + 1;
    static constexpr int kThreads = 32 * (4 * NG + 3);
    static constexpr uint32_t kGroupCols = 512u / NG;
    static constexpr uint32_t kDCol = NG == 2 ? 128u : 0u;   // D_main within the group's columns
    static constexpr bool kSmemA = NG == 4;
};
constexpr uint32_t kTileBytes = 4096 * 8;        // one tile (complex64), without padding
constexpr uint32_t kTmemCols = 512;
constexpr float kLoScale = 2048.0f;     // 2^11: lo halves are stored scaled up
constexpr float kLoUnscale = 1.0f / 2048.0f;
constexpr uint32_t kBImage = 16384;     // one block's [B_hi; B_lo']: 128 rows x 64 f16 (128 B)
constexpr uint32_t kMaxStages = 8;
// shared memory: [0, 1024) barriers, TMEM slot, abort flag, run offsets;
// then nblocks B images; then the stages.
constexpr uint32_t kOffFull = 0;        // 8 B per stage
constexpr uint32_t kOffEmpty = 64;
constexpr uint32_t kOffOut = 128;
constexpr uint32_t kOffMma = 192;       // one per group, up to 4
constexpr uint32_t kOffSlot = 224;
constexpr uint32_t kOffAbort = 228;
constexpr uint32_t kOffRunOff = 256;    // 32 x u64
constexpr uint32_t kOffB = 1024;
constexpr uint32_t kAlignSlack = 1024;
static_assert(kOffEmpty >= kOffFull + 8 * kMaxStages && kOffOut >= kOffEmpty + 8 * kMaxStages &&
                  kOffMma >= kOffOut + 8 * kMaxStages,
              "stage barriers overlap");
static_assert(kOffSlot >= kOffMma + 8 * 4 && kOffAbort >= kOffSlot + 4 && kOffRunOff >= kOffAbort + 4 &&
                  kOffB >= kOffRunOff + 8 * 32,
              "shared-memory header fields overlap");
// Longest any wait may last by default (TcOffsets::wait_ns; the caller may
// shorten it).  Normal waits last microseconds; profiler replays with
// instrumented instructions slow a launch by four orders of magnitude or
// more and must not trip the limit.  A CTA that does give up sets the abort
// flag and every other wait then returns at once.  Before the CTA exits, it
// drains what is still in flight -- issued tile loads, MMAs already
// committed -- each for at most kDrainLimitNs (they complete in
// microseconds), so that no copy lands and no MMA writes after its TMEM is
// released.
constexpr uint64_t kDrainLimitNs = 60000000000ull;

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

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B f16
// (bits 7-9 and 10-12 = 0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t idesc_f16(uint32_t n)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
constexpr uint32_t kIdescN128 = idesc_f16(128);
constexpr uint32_t kIdescN64 = idesc_f16(64);

// x rounded to 11 significant bits (nearest, ties away from zero) as an
// FP32 with the 13 low mantissa bits cleared, so that x - to_tf32(x) is the
// exact remainder.  In the normal range of f16 the result is an f16 value.
__device__ __forceinline__ float to_tf32(float x)
{
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
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

// D (TMEM) (+)= A (TMEM) * B (SMEM descriptor)^T
__device__ __forceinline__ void mma_f16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc));
}

// D (TMEM) (+)= A (SMEM descriptor) * B (SMEM descriptor)^T
__device__ __forceinline__ void mma_f16_ss(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void st_shared_u32(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t* v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]),
        "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]),
        "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst_smem, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst_smem),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst, uint32_t src_smem, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src_smem), "r"(bytes)
                 : "memory");
}

// One box of the tensor map `map` at coordinates c into shared memory,
// completing on `bar`.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, const int* c, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_store_5d(const CUtensorMap* map, const int* c, uint32_t src)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4, %5}], [%6];" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(src)
        : "memory");
}

// Tensor-map coordinates of a tile.
__device__ __forceinline__ void tile_coords(uint64_t tile, const TcOffsets& o, int* c)
{
#pragma unroll
    for (int d = 0; d < 5; ++d) c[d] = (int)((uint32_t)(tile >> o.tshift[d]) & o.tmask[d]);
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_test_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Limits below this are polled with the non-blocking test_wait and the clock
// read on every poll (try_wait may suspend the thread for a while inside one
// poll, longer than such a limit).
constexpr uint64_t kPromptLimitNs = 1000000ull;

// Bounded wait on an mbarrier phase; gives up (returns false) when the CTA's
// abort flag is set or after limit_ns, setting the flag.  The clock is read
// on the first failed poll and every 256th after it.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                           uint64_t limit_ns)
{
    if (limit_ns < kPromptLimitNs) {
        const uint64_t t0 = global_ns();
        while (!mbar_test_wait(bar, parity)) {
            if (*abort_flag) return false;
            if (global_ns() - t0 > limit_ns) {
                *abort_flag = 1;
                return false;
            }
        }
        return true;
    }
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    uint32_t polls = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        ++polls;
        if (polls > 64) __nanosleep(64);   // long waits leave issue slots to the warps waited for
        if ((polls == 1 || (polls & 255u) == 0) && global_ns() - t0 > limit_ns) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

// Wait for a phase regardless of the abort flag, for at most kDrainLimitNs:
// what a CTA that gave up still has in flight.
__device__ __forceinline__ void drain_phase(uint32_t bar, uint32_t parity)
{
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity) && global_ns() - t0 <= kDrainLimitNs) {
    }
}

// Named barrier over one consumer group (ids 1 and 2, 128 threads).
__device__ __forceinline__ void group_sync(uint32_t id)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(kGroupThreads) : "memory");
}

// OR of `fail` over one consumer group: every thread of the group takes the
// same branch, so none can be left waiting at a barrier.
__device__ __forceinline__ bool group_any(bool fail, uint32_t id)
{
    uint32_t any;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(any)
        : "r"((uint32_t)fail), "r"(id), "n"(kGroupThreads)
        : "memory");
    return any != 0;
}

// Two f32 values as an f16 pair: `first` in the low half (the lower K index).
__device__ __forceinline__ uint32_t pack_f16x2(float first, float second)
{
    uint32_t d;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(second), "f"(first));
    return d;
}

// Amplitude v (times sc when SCALE) -> hi = (re, im) to 11 bits and
// lo = 2^11 (v - hi), each an f16 pair with the real part in the low half.
template <bool SCALE>
__device__ __forceinline__ void split_amp(float2 v, float sc, uint32_t& hi, uint32_t& lo)
{
    const float re = SCALE ? v.x * sc : v.x, im = SCALE ? v.y * sc : v.y;
    const float hr = to_tf32(re), hm = to_tf32(im);
    hi = pack_f16x2(hr, hm);
    lo = pack_f16x2((re - hr) * kLoScale, (im - hm) * kLoScale);
}

// The 32 amplitudes of row `rowb`, all loads issued before any is used.
__device__ __forceinline__ void load_row(const uint8_t* raw, uint32_t rowb, const TcBlockGeom& G, float2 (&x)[32])
{
    if (G.vec2) {
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            const float4 p = *(const float4*)(raw + rowb + G.gateoff[2 * m]);
            x[2 * m] = make_float2(p.x, p.y);
            x[2 * m + 1] = make_float2(p.z, p.w);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) x[j] = *(const float2*)(raw + rowb + G.gateoff[j]);
    }
}

// Gates 16*HH .. 16*HH+15 of a loaded row -> f16 operands in TMEM columns
// 32*HH .. 32*HH+31: per K-step of 8 gates (16 f16), 8 columns of hi pairs
// then 8 of lo pairs.  SCALE: the stage holds plain amplitudes (first block
// of a pass), which enter times sc; later blocks find them scaled already.
template <int HH, bool SCALE>
__device__ __forceinline__ void split_store_half(const float2 (&x)[32], float sc, uint32_t tl)
{
    uint32_t v[32];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int c = (j >> 3) * 16 + (j & 7);
        split_amp<SCALE>(x[16 * HH + j], sc, v[c], v[c + 8]);
    }
    tmem_st32(tl + 32u * HH, v);
}

// The whole row's D_main + 2^-11 D_corr back into the stage, half a row per
// TMEM wait.  UNSCALE (last block of a pass): times `unscale`, which undoes
// the operands' powers of two; otherwise the amplitudes stay scaled for the
// next block (whose B is not scaled).
template <bool UNSCALE>
__device__ __forceinline__ void writeback_row(uint8_t* raw, uint32_t rowb, const TcBlockGeom& G, uint32_t td,
                                              float unscale)
{
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        uint32_t dm[32], dc[32];
        tmem_ld32(td + 32u * hh, dm);
        tmem_ld32(td + 64u + 32u * hh, dc);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float d = __fmaf_rn(__uint_as_float(dc[j]), kLoUnscale, __uint_as_float(dm[j]));
            dm[j] = __float_as_uint(UNSCALE ? d * unscale : d);
        }
        if (G.vec2) {
#pragma unroll
            for (int m = 0; m < 8; ++m)
                *(float4*)(raw + rowb + G.gateoff[16 * hh + 2 * m]) =
                    make_float4(__uint_as_float(dm[4 * m]), __uint_as_float(dm[4 * m + 1]),
                                __uint_as_float(dm[4 * m + 2]), __uint_as_float(dm[4 * m + 3]));
        } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                *(float2*)(raw + rowb + G.gateoff[16 * hh + j]) =
                    make_float2(__uint_as_float(dm[2 * j]), __uint_as_float(dm[2 * j + 1]));
        }
    }
}

// The last block's write-back with lane-permuted stores (TcOffsets::wb_xor):
// at step j of half hh the thread stores its output gate state j ^ wx,
// moved into place by register butterflies, at staged byte rowx ^
// gateoff[16 hh + j], rowx = row offset ^ gateoff[wx].  The layout is
// linear (unpadded), so that is the state's own offset.  wx < 16; bit 0
// clear where 16-byte stores keep gate pairs together.  Every butterfly
// runs, selecting by the lane's bit: branches around the unused ones
// measured slower.
__device__ __forceinline__ void writeback_row_xor(uint8_t* raw, uint32_t rowx, const TcBlockGeom& G, uint32_t td,
                                                  float unscale, uint32_t wx)
{
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        // D_corr in two loads of 16 columns: fewer registers live at once
        uint32_t dm[32], dc[16];
        tmem_ld32(td + 32u * hh, dm);
        tmem_ld16(td + 64u + 32u * hh, dc);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j)
            dm[j] = __float_as_uint(__fmaf_rn(__uint_as_float(dc[j]), kLoUnscale, __uint_as_float(dm[j])) * unscale);
        tmem_ld16(td + 80u + 32u * hh, dc);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j)
            dm[16 + j] =
                __float_as_uint(__fmaf_rn(__uint_as_float(dc[j]), kLoUnscale, __uint_as_float(dm[16 + j])) * unscale);
        if (G.vec2) {
            // 8 chunks of two gate states (4 words); chunk m <- chunk m ^ (wx >> 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const bool p = (wx >> (k + 1)) & 1u;
#pragma unroll
                for (int m = 0; m < 8; ++m) {
                    if (m & (1 << k)) continue;
                    const int m1 = m | (1 << k);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const uint32_t v0 = dm[4 * m + e], v1 = dm[4 * m1 + e];
                        dm[4 * m + e] = p ? v1 : v0;
                        dm[4 * m1 + e] = p ? v0 : v1;
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < 8; ++m)
                *(float4*)(raw + (rowx ^ G.gateoff[16 * hh + 2 * m])) =
                    make_float4(__uint_as_float(dm[4 * m]), __uint_as_float(dm[4 * m + 1]),
                                __uint_as_float(dm[4 * m + 2]), __uint_as_float(dm[4 * m + 3]));
        } else {
            // 16 gate states (2 words); state j <- state j ^ wx
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const bool p = (wx >> k) & 1u;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (j & (1 << k)) continue;
                    const int j1 = j | (1 << k);
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const uint32_t v0 = dm[2 * j + e], v1 = dm[2 * j1 + e];
                        dm[2 * j + e] = p ? v1 : v0;
                        dm[2 * j1 + e] = p ? v0 : v1;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < 16; ++j)
                *(float2*)(raw + (rowx ^ G.gateoff[16 * hh + j])) =
                    make_float2(__uint_as_float(dm[2 * j]), __uint_as_float(dm[2 * j + 1]));
        }
    }
}

// A block's results in a direct pass (TcOffsets::direct): each output
// amplitude, still scaled, split into hi/lo f16 pairs and stored as the
// next block's A operand -- hi plane at abase, lo plane 16 KB above -- at
// offset rowpart ^ scat_gate[g].
__device__ __forceinline__ void writeback_scatter(uint32_t abase, uint32_t rowpart, const uint32_t* scat_gate,
                                                  uint32_t td)
{
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        uint32_t dm[32], dc[32];
        tmem_ld32(td + 32u * hh, dm);
        tmem_ld32(td + 64u + 32u * hh, dc);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float2 d = make_float2(__fmaf_rn(__uint_as_float(dc[2 * j]), kLoUnscale, __uint_as_float(dm[2 * j])),
                                         __fmaf_rn(__uint_as_float(dc[2 * j + 1]), kLoUnscale,
                                                   __uint_as_float(dm[2 * j + 1])));
            uint32_t hi, lo;
            split_amp<false>(d, 1.0f, hi, lo);
            const uint32_t a = abase + (rowpart ^ scat_gate[16 * hh + j]);
            st_shared_u32(a, hi);
            st_shared_u32(a + 16384u, lo);
        }
    }
}

// The first block's results of a shuffled pair, kept in registers:
// D_main + 2^-11 D_corr of the row, still scaled for the second block.
__device__ __forceinline__ void writeback_regs(uint32_t td, float2 (&x)[32])
{
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        uint32_t dm[32], dc[32];
        tmem_ld32(td + 32u * hh, dm);
        tmem_ld32(td + 64u + 32u * hh, dc);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j)
            x[16 * hh + j] = make_float2(__fmaf_rn(__uint_as_float(dc[2 * j]), kLoUnscale, __uint_as_float(dm[2 * j])),
                                         __fmaf_rn(__uint_as_float(dc[2 * j + 1]), kLoUnscale,
                                                   __uint_as_float(dm[2 * j + 1])));
    }
}

// Register bit a of every row swaps roles with lane bit swap_lane[a] (when
// >= 0): a lane whose bit is 0 keeps its registers with bit a = 0 and sends
// those with bit a = 1 to its partner lane, which sends back its registers
// with bit a = 0.  Afterwards each thread holds its row of the second block,
// in that block's gate order.
__device__ __forceinline__ void swap_reg_lane_bits(float2 (&x)[32], const int32_t* swap_lane, uint32_t lane)
{
#pragma unroll
    for (int a = 0; a < 5; ++a) {
        const int bl = swap_lane[a];
        if (bl < 0) continue;
        const uint32_t m = 1u << bl;
        const bool up = (lane & m) != 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (j & (1 << a)) continue;
            const int j1 = j | (1 << a);
            const float2 send = up ? x[j] : x[j1];
            float2 got;
            got.x = __shfl_xor_sync(0xffffffffu, send.x, m);
            got.y = __shfl_xor_sync(0xffffffffu, send.y, m);
            if (up) x[j] = got;
            else x[j1] = got;
        }
    }
}

// The MMAs of K-steps k0 and k0+1 (one half of the row's gates):
// [D_main | D_corr] (+)= A_hi [B_hi; B_lo']^T, then D_corr += A_lo' B_hi^T.
__device__ __forceinline__ void issue_mma_ksteps(uint32_t tm, uint32_t bb, int k0)
{
#pragma unroll
    for (int ks = k0; ks < k0 + 2; ++ks)
        mma_f16_ts(tm + 128u, tm + 16u * ks, desc_sw128(bb + (uint32_t)ks * 32u), kIdescN128, ks > 0 ? 1u : 0u);
#pragma unroll
    for (int ks = k0; ks < k0 + 2; ++ks)
        mma_f16_ts(tm + 192u, tm + 16u * ks + 8u, desc_sw128(bb + (uint32_t)ks * 32u), kIdescN64, 1u);
}

// The first block's tile dealt to the group's threads as the split map
// says (TcOffsets::sp_*): 32 amplitudes at tb + sp_regoff[j], every load of
// the group performed (the barrier), then each 16-byte chunk q of hi/lo
// pairs stored at abase + (ta ^ sp_achunk[q]) in both planes.
__device__ __forceinline__ void split_mapped(const uint8_t* raw, uint32_t tb, uint32_t abase, uint32_t ta,
                                             const TcOffsets& o, uint32_t gbar)
{
    float2 x[32];
    if (o.sp_vec2) {
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            const float4 p = *(const float4*)(raw + tb + o.sp_regoff[2 * m]);
            x[2 * m] = make_float2(p.x, p.y);
            x[2 * m + 1] = make_float2(p.z, p.w);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) x[j] = *(const float2*)(raw + tb + o.sp_regoff[j]);
    }
    group_sync(gbar);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split_amp<true>(x[4 * q + e], o.ascale, hi[e], lo[e]);
        const uint32_t a = abase + (ta ^ o.sp_achunk[q]);
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(hi[0]), "r"(hi[1]), "r"(hi[2]),
                     "r"(hi[3])
                     : "memory");
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a + 16384u), "r"(lo[0]), "r"(lo[1]),
                     "r"(lo[2]), "r"(lo[3])
                     : "memory");
    }
}

// The MMAs of K-steps k0 and k0+1 with A in shared memory at abase (hi
// plane, then the lo plane 16 KB above, K-major SWIZZLE_128B): D_main at
// TMEM column td, D_corr at td + 64.
__device__ __forceinline__ void issue_mma_smem_ksteps(uint32_t td, uint32_t abase, uint32_t bb, int k0)
{
#pragma unroll
    for (int ks = k0; ks < k0 + 2; ++ks)
        mma_f16_ss(td, desc_sw128(abase + (uint32_t)ks * 32u), desc_sw128(bb + (uint32_t)ks * 32u), kIdescN128,
                   ks > 0 ? 1u : 0u);
#pragma unroll
    for (int ks = k0; ks < k0 + 2; ++ks)
        mma_f16_ss(td + 64u, desc_sw128(abase + 16384u + (uint32_t)ks * 32u), desc_sw128(bb + (uint32_t)ks * 32u),
                   kIdescN64, 1u);
}

// Half HH of a loaded row (gates 16HH .. 16HH+15) split into hi/lo f16
// pairs and stored as row t of the A operand in shared memory: 16-byte
// chunk c (gates 4c .. 4c+3) of each plane at its SWIZZLE_128B place.
template <int HH, bool SCALE>
__device__ __forceinline__ void split_store_smem(const float2 (&x)[32], float sc, uint32_t arow, uint32_t t)
{
#pragma unroll
    for (int c = 4 * HH; c < 4 * HH + 4; ++c) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split_amp<SCALE>(x[4 * c + e], sc, hi[e], lo[e]);
        const uint32_t a = arow + ((((uint32_t)c ^ t) & 7u) << 4);
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(hi[0]), "r"(hi[1]), "r"(hi[2]),
                     "r"(hi[3])
                     : "memory");
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a + 16384u), "r"(lo[0]), "r"(lo[1]),
                     "r"(lo[2]), "r"(lo[3])
                     : "memory");
    }
}

template <int NG>
__global__ void __launch_bounds__(TcShape<NG>::kThreads, 1)
k_fused_tc(float2* __restrict__ a, uint64_t ntiles, const __grid_constant__ IndexMap tilemap,
           const __grid_constant__ TcOffsets offs, const __grid_constant__ CUtensorMap tmap,
           const __grid_constant__ CUtensorMap tmap_st, const uint4* __restrict__ bimage, int* __restrict__ err)
{
    using Sh = TcShape<NG>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_addr(smem);
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const uint32_t nst = offs.nstages, sbytes = offs.stage_bytes, nblocks = offs.nblocks;
    const uint32_t raw0 = kOffB + nblocks * kBImage;      // stage 0
    uint32_t* tmem_slot = (uint32_t*)(smem + kOffSlot);
    volatile int* abort_flag = (volatile int*)(smem + kOffAbort);
    uint64_t* run_off = (uint64_t*)(smem + kOffRunOff);

    {
        uint4* dst = (uint4*)(smem + kOffB);
        const uint32_t n16 = nblocks * kBImage / 16;
        for (uint32_t i = tid; i < n16; i += Sh::kThreads) dst[i] = bimage[i];
        if (tid < 32) run_off[tid] = offs.run_off[tid];
    }
    if (tid == 0) {
        for (uint32_t s = 0; s < nst; ++s) {
            mbar_init(sbase + kOffFull + 8 * s, 1);
            mbar_init(sbase + kOffEmpty + 8 * s, 1);
            mbar_init(sbase + kOffOut + 8 * s, kGroupThreads);
        }
        for (int g = 0; g < NG; ++g) mbar_init(sbase + kOffMma + 8 * g, 1);
        *abort_flag = 0;
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
    const uint64_t my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t pb = offs.piece_bits, np = offs.npieces, pad = offs.pad_shift, rb = offs.run_bits;
    const uint32_t piece_bytes = 8u << pb;
    const uint64_t run_mask = (uint64_t(1) << rb) - 1u;

    if (warp == Sh::kLoaderWarp) {
        // ---------------------------------------------------------- loader
        uint32_t s = 0, u = 0;
        uint64_t issued = 0;
        for (uint64_t i = 0; i < my_tiles; ++i) {
            // use u of stage s waits until the store of use u-1 has read it
            if (u > 0 && !wait_phase(sbase + kOffEmpty + 8 * s, (u - 1) & 1u, abort_flag, offs.wait_ns)) break;
            const uint64_t tile = blockIdx.x + i * gridDim.x;
            const uint32_t full = sbase + kOffFull + 8 * s;
            const uint32_t st = sbase + raw0 + s * sbytes;
            if (offs.use_tma) {
                if (lane == 0) {
                    int c[5];
                    tile_coords(tile, offs, c);
                    mbar_arrive_tx(full, kTileBytes);
                    tma_load_5d(st, &tmap, c, full);
                }
            } else {
                const uint64_t base = expand_index(tile, tilemap);
                if (lane == 0) mbar_arrive_tx(full, kTileBytes);
                __syncwarp();
                for (uint32_t j = (uint32_t)lane; j < np; j += 32) {
                    const uint32_t x0 = j << pb;
                    bulk_load(st + 8u * x0 + ((x0 >> pad) << 4),
                              a + ((base | run_off[x0 >> rb]) + (x0 & run_mask)), piece_bytes, full);
                }
            }
            __syncwarp();
            issued = i + 1;
            if (++s == nst) {
                s = 0;
                ++u;
            }
        }
        // every load issued has landed before the CTA can exit (the
        // consumers waited for all of them unless the CTA gave up)
        const uint64_t from = issued > nst ? issued - nst : 0;
        for (uint64_t i = from; i < issued; ++i)
            drain_phase(sbase + kOffFull + 8 * (uint32_t)(i % nst), (uint32_t)((i / nst) & 1));
    } else if (warp >= Sh::kStorerWarp0) {
        // --------------------------------------------------------- storers
        // storer w takes tiles w, w+2, ...; after its store has read the
        // stage it frees the stage at once.  A parity wait on the stage's
        // out phase u is only unambiguous once phase u-1 has completed; with
        // an odd number of stages the stage's previous use is the other
        // storer's tile, so first wait until that tile has been stored (the
        // stage's empty phase u-1; it follows its out phase u-1)
        const uint32_t w = (uint32_t)(warp - Sh::kStorerWarp0);
        uint32_t s = w, u = 0;
        for (uint64_t i = w; i < my_tiles; i += 2) {
            if (u > 0 && !wait_phase(sbase + kOffEmpty + 8 * s, (u - 1) & 1u, abort_flag, offs.wait_ns)) break;
            if (!wait_phase(sbase + kOffOut + 8 * s, u & 1u, abort_flag, offs.wait_ns)) break;
            const uint64_t tile = blockIdx.x + i * gridDim.x;
            const uint32_t st = sbase + raw0 + s * sbytes;
            if (offs.use_tma) {
                if (lane == 0) {
                    int c[5];
                    if (offs.st_box) {
                        // the last block wrote the store box's layout
#pragma unroll
                        for (int d = 0; d < 5; ++d)
                            c[d] = (int)((uint32_t)(tile >> offs.st_tshift[d]) & offs.st_tmask[d]);
                        tma_store_5d(&tmap_st, c, st);
                    } else {
                        tile_coords(tile, offs, c);
                        tma_store_5d(&tmap, c, st);
                    }
                }
            } else {
                const uint64_t base = expand_index(tile, tilemap);
                for (uint32_t j = (uint32_t)lane; j < np; j += 32) {
                    const uint32_t x0 = j << pb;
                    bulk_store(a + ((base | run_off[x0 >> rb]) + (x0 & run_mask)),
                               st + 8u * x0 + ((x0 >> pad) << 4), piece_bytes);
                }
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(sbase + kOffEmpty + 8 * s);
            s += 2;
            if (s >= nst) {
                s -= nst;
                ++u;
            }
        }
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    } else {
        // ------------------------------------------------ consumer groups
        // group g = warps 4g..4g+3; warp's lane quarter q (rows 32q..32q+31)
        const uint32_t g = (uint32_t)warp >> 2, q = (uint32_t)warp & 3u;
        const uint32_t t = 32u * q + (uint32_t)lane;       // row = TMEM lane
        const bool issuer = t == 0;
        const uint32_t gbar = 1u + g;
        const uint32_t tm = tmem + Sh::kGroupCols * g;      // the group's columns
        const uint32_t tl = tm + ((32u * q) << 16);         // this warp's lanes
        const uint32_t td = tl + Sh::kDCol;                 // its accumulators
        const uint32_t mbar = sbase + kOffMma + 8u * g;
        // row t of an A operand in shared memory (SWIZZLE_128B, 128 B rows)
        const uint32_t arow = (t >> 3) * 1024u + (t & 7u) * 128u;
        uint32_t rowb0 = 0, rowb1 = 0, rowb2 = 0, rowpart0 = 0, rowpart1 = 0, sp_tb = 0, sp_ta = 0;
#pragma unroll
        for (int r = 0; r < 7; ++r)
            if ((t >> r) & 1u) {
                rowb0 += offs.blk[0].rowoff[r];
                rowb1 += offs.blk[1].rowoff[r];
                rowb2 += offs.blk[2].rowoff[r];
                rowpart0 ^= offs.scat_row[0][r];
                rowpart1 ^= offs.scat_row[1][r];
                sp_tb += offs.sp_thoff[r];
                sp_ta ^= offs.sp_athr[r];
            }
        const bool direct = offs.direct != 0;
        uint32_t s = g, u = 0, mph = 0;     // tile i lives in stage i % nst
        for (uint64_t i = g; i < my_tiles; i += NG) {
            // the stage's full phase u is unambiguous by parity once phase
            // u-1 has completed, which its previous tile's store implies
            // (copies may land out of order); tile i's copy is only issued
            // after that store, so that wait costs nothing
            const bool ready =
                (u == 0 || wait_phase(sbase + kOffEmpty + 8 * s, (u - 1) & 1u, abort_flag, offs.wait_ns)) &&
                wait_phase(sbase + kOffFull + 8 * s, u & 1u, abort_flag, offs.wait_ns);
            if (group_any(!ready, gbar)) break;
            uint8_t* raw = smem + raw0 + s * sbytes;
            const uint32_t abase = smem_addr(raw);
            bool stop = false;
            const bool shuf = !Sh::kSmemA && offs.shuffle != 0;
            float2 x[32];
#pragma unroll
            for (int b = 0; b < kTcMaxBlocks; ++b) {
                if ((uint32_t)b >= nblocks) break;
                const TcBlockGeom& G = offs.blk[b];
                const uint32_t rowb = b == 0 ? rowb0 : (b == 1 ? rowb1 : rowb2);
                // the previous block's results are all staged (or, shuffled,
                // already in this thread's registers)
                if (b > 0 && !shuf && !direct) group_sync(gbar);
                const uint32_t bb = sbase + kOffB + (uint32_t)b * kBImage;
                if (b > 0 && direct) {
                    // the first block's write-back left this block's
                    // operands in the stage: make them visible to the
                    // tensor cores, then the MMAs
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_smem_ksteps(td, abase, bb, 0);
                        issue_mma_smem_ksteps(td, abase, bb, 2);
                        mma_commit(mbar);
                    }
                } else if (Sh::kSmemA && b == 0) {
                    // the tile -> hi/lo operands over it in the stage, dealt
                    // to the threads by the split map; then the 8 MMAs
                    split_mapped(raw, sp_tb, abase, sp_ta, offs, gbar);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_smem_ksteps(td, abase, bb, 0);
                        issue_mma_smem_ksteps(td, abase, bb, 2);
                        mma_commit(mbar);
                    }
                } else if (Sh::kSmemA) {
                    // row t -> hi/lo operands over the tile in the stage:
                    // every load of the group is performed first (the
                    // barrier), then each half is split, stored and its two
                    // K-steps' MMAs issued while the second half converts
                    load_row(raw, rowb, G, x);
                    group_sync(gbar);
                    if (b == 0) split_store_smem<0, true>(x, offs.ascale, abase + arow, t);
                    else split_store_smem<0, false>(x, offs.ascale, abase + arow, t);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_smem_ksteps(td, abase, bb, 0);
                    }
                    if (b == 0) split_store_smem<1, true>(x, offs.ascale, abase + arow, t);
                    else split_store_smem<1, false>(x, offs.ascale, abase + arow, t);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_smem_ksteps(td, abase, bb, 2);
                        mma_commit(mbar);
                    }
                } else {
                    // row t -> hi/lo operands in TMEM: every load of the row is
                    // issued first; after the first half is stored, its two
                    // K-steps' MMAs run while the second half converts
                    if (b == 0 || !shuf) load_row(raw, rowb, G, x);
                    if (b == 0) split_store_half<0, true>(x, offs.ascale, tl);
                    else split_store_half<0, false>(x, offs.ascale, tl);
                    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_ksteps(tm, bb, 0);
                    }
                    if (b == 0) split_store_half<1, true>(x, offs.ascale, tl);
                    else split_store_half<1, false>(x, offs.ascale, tl);
                    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    group_sync(gbar);
                    if (issuer) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        issue_mma_ksteps(tm, bb, 2);
                        mma_commit(mbar);
                    }
                }
                if (group_any(!wait_phase(mbar, mph & 1u, abort_flag, offs.wait_ns), gbar)) {
                    // the MMAs were committed (every thread of the group is
                    // past the issuer's commit): let them finish before the
                    // CTA releases its TMEM
                    drain_phase(mbar, mph & 1u);
                    stop = true;
                    break;
                }
                ++mph;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if ((uint32_t)b + 1 == nblocks) {
                    if ((offs.wb_xor[0] | offs.wb_xor[1] | offs.wb_xor[2] | offs.wb_xor[3] | offs.wb_xor[4]) != 0) {
                        // the store permutation of this lane
                        uint32_t wx = 0;
#pragma unroll
                        for (int r = 0; r < 5; ++r)
                            if ((lane >> r) & 1) wx ^= offs.wb_xor[r];
                        uint32_t rowx = rowb;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if ((wx >> k) & 1u) rowx ^= G.gateoff[1 << k];
                        writeback_row_xor(raw, rowx, G, td, offs.unscale, wx);
                    } else {
                        writeback_row<true>(raw, rowb, G, td, offs.unscale);
                    }
                } else if (shuf) {
                    writeback_regs(td, x);
                    swap_reg_lane_bits(x, offs.swap_lane, (uint32_t)lane);
                } else if (direct) {
                    writeback_scatter(abase, b == 0 ? rowpart0 : rowpart1, offs.scat_gate[b < 1 ? 0 : 1], td);
                } else {
                    writeback_row<false>(raw, rowb, G, td, offs.unscale);
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            }
            if (stop) break;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(sbase + kOffOut + 8 * s);
            s += NG;
            if (s >= nst) {
                s -= nst;
                ++u;
            }
        }
    }
    __syncthreads();
    if (*abort_flag && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

uint32_t staged_offset(uint32_t x, uint32_t pad)
{
    return 8u * x + ((pad < 31 ? (x >> pad) : 0u) << 4);
}

// Shared-memory wavefronts of one warp instruction over its rows (lanes =
// rows 0..31 with row bit r at tile coordinate order[r], all at the same
// gate), `width` bytes per lane.  Shared memory serves 8-byte accesses in
// half-warp phases and 16-byte accesses in quarter-warp phases; a phase takes
// as many wavefronts as the most distinct words any one bank holds.
int warp_wavefronts(const uint32_t* order, uint32_t pad, int width)
{
    const uint32_t lanes_per_phase = width == 16 ? 8 : 16;
    const uint32_t wpl = (uint32_t)width / 4;   // words per lane
    int total = 0;
    for (uint32_t ph = 0; ph < 32 / lanes_per_phase; ++ph) {
        uint32_t words[64];
        uint32_t nw = 0;
        for (uint32_t l = ph * lanes_per_phase; l < (ph + 1) * lanes_per_phase; ++l) {
            uint32_t x = 0;
            for (int r = 0; r < 5; ++r)
                if ((l >> r) & 1u) x |= order[r];
            const uint32_t word0 = staged_offset(x, pad) / 4;
            for (uint32_t w = 0; w < wpl; ++w) words[nw++] = word0 + w;
        }
        std::sort(words, words + nw);
        int per_bank[32] = {0};
        int m = 0;
        for (uint32_t i = 0; i < nw; ++i)
            if (i == 0 || words[i] != words[i - 1]) m = std::max(m, ++per_bank[words[i] % 32]);
        total += m;
    }
    return total;
}

// Wavefronts of one phase of lane addresses a(l) = XOR over the lane's bits
// r < nbits of vec[r] (byte offsets), `width` bytes per lane.
static int phase_wavefronts(const uint32_t* vec, int nbits, int width)
{
    const uint32_t wpl = (uint32_t)width / 4;
    uint32_t words[64];
    uint32_t nw = 0;
    for (uint32_t l = 0; l < (1u << nbits); ++l) {
        uint32_t x = 0;
        for (int r = 0; r < nbits; ++r)
            if ((l >> r) & 1u) x ^= vec[r];
        for (uint32_t w = 0; w < wpl; ++w) words[nw++] = x / 4 + w;
    }
    std::sort(words, words + nw);
    int per_bank[32] = {0};
    int m = 0;
    for (uint32_t i = 0; i < nw; ++i)
        if (i == 0 || words[i] != words[i - 1]) m = std::max(m, ++per_bank[words[i] % 32]);
    return m;
}

// The lane-permuted write-back's register butterflies (4, or 3 with 16-byte
// stores; all run once any lane permutes), each in wavefront units of one
// warp: 64 selects a row, measured at about 12 shared-memory wavefronts'
// worth of pass time (30-qubit brick passes: the four butterflies cost
// 13 % of a conflict-free pass, a 4x conflicted 16-byte write-back 48 %).
constexpr long kWbButterflyCost = 12;

// warp_wavefronts of the last block's write-back in a linear layout (tile
// bit j at element bit sbit[j], or at j when sbit is null) when the stores
// may be permuted per lane (TcOffsets::wb_xor): lane bit r XORs the stored
// gate state by phi[r].  Lane l then stores at its row's offset XOR the
// gate offset of phi(l) (plus the step's, common to all lanes), so each
// phase lane bit r may add any gate offset of gate bits 1-3 (16-byte
// stores) or 0-3 to its row offset.  Lane bits are taken in order, each
// given the first permutation that raises the rank of the phase's bank
// slots (address bits 4-6 for 16-byte, 3-6 for 8-byte stores), none if
// its row offset does already; the result is kept when it beats no
// permutation.  gk[i]: tile bit of gate bit i; phi out (zero: none);
// plain_out: the wavefronts without a permutation.
int warp_wavefronts_xor(const uint32_t* order, const int* sbit, const int* gk, int width, uint32_t* phi,
                        int* plain_out)
{
    auto off = [&](int j) { return 8u << (sbit ? sbit[j] : j); };
    const int nl = width == 16 ? 3 : 4;                 // lane bits of a phase
    const uint32_t lo = width == 16 ? 4u : 3u, slots = width == 16 ? 7u : 15u;
    const uint32_t gmin = width == 16 ? 1u : 0u;        // lowest gate bit permuted
    uint32_t row[5], best[5] = {0, 0, 0, 0, 0};
    for (int r = 0; r < 5; ++r) row[r] = off(__builtin_ctz(order[r]));
    auto gate_off = [&](uint32_t ph) {
        uint32_t a = 0;
        for (int i = 0; i < 4; ++i)
            if ((ph >> i) & 1u) a ^= off(gk[i]);
        return a;
    };
    const int plain = (32 / (1 << nl)) * phase_wavefronts(row, nl, width);
    // greedy rank: basis of the chosen slot vectors, by leading bit
    uint32_t basis[4] = {0, 0, 0, 0};
    auto reduce = [&](uint32_t v) {
        for (int b = 3; b >= 0; --b)
            if (((v >> b) & 1u) && basis[b]) v ^= basis[b];
        return v;
    };
    auto insert = [&](uint32_t v) {
        v = reduce(v);
        if (!v) return false;
        basis[31 - __builtin_clz(v)] = v;
        return true;
    };
    uint32_t vec[5];
    for (int r = 0; r < nl; ++r) {
        uint32_t pick = 0;
        for (uint32_t ph = 0; ph < 16; ++ph) {
            if (ph & ((1u << gmin) - 1u)) continue;
            if (reduce(((row[r] ^ gate_off(ph)) >> lo) & slots)) {
                pick = ph;
                break;
            }
        }
        best[r] = pick;
        vec[r] = row[r] ^ gate_off(pick);
        insert((vec[r] >> lo) & slots);
    }
    const int permuted = (32 / (1 << nl)) * phase_wavefronts(vec, nl, width);
    for (int r = 0; r < 5; ++r) phi[r] = permuted < plain ? best[r] : 0u;
    if (plain_out) *plain_out = plain;
    return std::min(plain, permuted);
}

// The order of a block's 7 row bits (which tile coordinates the low lane
// bits select) with the fewest wavefronts under padding `pad`.  Rows are
// independent in the GEMM, so any order is correct; only the row bits that
// vary inside one phase (3 for 16-byte, 4 for 8-byte accesses) matter.
int best_row_order(const TcBlockGeom& G, uint32_t pad, uint32_t* order)
{
    const bool v2 = G.vec2 != 0;
    const int width = v2 ? 16 : 8, k = v2 ? 3 : 4;
    int best = -1;
    for (uint32_t mask = 0; mask < 128; ++mask) {
        if (__builtin_popcount(mask) != k) continue;
        uint32_t cand[7];
        int c = 0;
        for (int r = 0; r < 7; ++r)
            if ((mask >> r) & 1u) cand[c++] = G.jrow_bit[r];
        for (int r = 0; r < 7; ++r)
            if (!((mask >> r) & 1u)) cand[c++] = G.jrow_bit[r];
        const int wf = warp_wavefronts(cand, pad, width);
        if (best < 0 || wf < best) {
            best = wf;
            std::memcpy(order, cand, sizeof(cand));
            if (best == width / 4) break;     // 32 lanes x width bytes in 128-byte wavefronts
        }
    }
    return best;
}

// Sets the padding fields and both blocks' row orders and staged offsets.
void apply_layout(TcOffsets& o, uint32_t pad, const uint32_t (&order)[kTcMaxBlocks][7])
{
    o.pad_shift = pad;
    o.stage_bytes = kTileBytes + (pad < 31 ? 16u * (4096u >> pad) : 0u);
    o.piece_bits = std::min(pad, o.run_bits);
    o.npieces = 4096u >> o.piece_bits;
    for (uint32_t b = 0; b < o.nblocks; ++b) {
        TcBlockGeom& G = o.blk[b];
        for (int r = 0; r < 7; ++r) {
            G.jrow_bit[r] = order[b][r];
            G.rowoff[r] = staged_offset(G.jrow_bit[r], pad);
        }
        for (int g = 0; g < 32; ++g) G.gateoff[g] = staged_offset(G.jgate[g], pad);
    }
}

// Byte offset, in the second block's A operand (tc_sw128_offset of row r2,
// K index 2 g2), that tile bit j contributes in a direct pass: the offset
// is linear over GF(2) in the bits of r2 and g2, so it is the XOR of its
// tile bits' contributions.  gbit1[k]: tile bit of gate bit k; order1[i]:
// tile bit of row bit i (one-hot coordinates).
uint32_t direct_bit_offset(int j, const int* gbit1, const uint32_t* order1)
{
    for (int k = 0; k < 5; ++k)
        if (gbit1[k] == j) return tc_sw128_offset(0, 2u << k);
    for (int i = 0; i < 7; ++i)
        if (order1[i] == (1u << j)) return tc_sw128_offset(1u << i, 0);
    return 0;
}

// Wavefronts of one warp's 4-byte scattered stores (all 32 lanes in one
// phase): lanes = rows with row bit r at offset pattern pat[r], r < 5.
int scatter_wavefronts(const uint32_t* pat)
{
    int per_bank[32] = {0};
    int m = 0;
    for (uint32_t l = 0; l < 32; ++l) {
        uint32_t a = 0;
        for (int r = 0; r < 5; ++r)
            if ((l >> r) & 1u) a ^= pat[r];
        m = std::max(m, ++per_bank[(a >> 2) & 31u]);
    }
    return m;
}

}  // namespace

bool tc_direct_layout(TcOffsets& o, bool tma_ok, int conflict_slack, int* gbit1)
{
    if (o.nblocks != 2) return false;
    const uint32_t gate0 = o.blk[0].jgate[31], gate1 = o.blk[1].jgate[31];
    if (__builtin_popcount(gate0) != 5 || __builtin_popcount(gate1) != 5) return false;
    std::vector<int> rows0, rows1;
    for (int j = 0; j < 12; ++j) {
        if (!((gate0 >> j) & 1u)) rows0.push_back(j);
        if (!((gate1 >> j) & 1u)) rows1.push_back(j);
    }
    const bool v0 = o.blk[0].vec2 != 0;
    const int width0 = v0 ? 16 : 8, inphase0 = v0 ? 3 : 4;
    // per warp: block 0's row loads, 64 scattered stores, block 1's stores
    const long ideal = 3 * 64;

    struct Best {
        long cost = -1;
        uint32_t pad = 31;
        uint32_t order[kTcMaxBlocks][7] = {};
        int g1[5] = {};
    } best;
    // the choice depends only on the geometry and the slack: remember it
    static std::mutex mu;
    static std::unordered_map<std::string, Best> memo;
    std::string key(1, tma_ok ? 'T' : 'P');
    key.append((const char*)&conflict_slack, sizeof(conflict_slack));
    key.append((const char*)&o.run_bits, sizeof(o.run_bits));
    key.append((const char*)o.blk[0].jgate, sizeof(o.blk[0].jgate));
    key.append((const char*)&gate1, sizeof(gate1));
    bool found = false;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = memo.find(key);
        if (it != memo.end()) {
            best = it->second;
            found = true;
        }
    }
    const uint32_t cands[] = {31, 11, 10, 9, 8, 7, 6, 5};
    for (uint32_t pad : cands) {
        if (found) break;
        if (pad < 31 && tma_ok && best.cost >= 0 && best.cost <= conflict_slack * ideal) break;
        // block 0: which 5 row bits are lanes, and which of them select the
        // access phase (the rest vary inside a phase)
        for (uint32_t lanes = 0; lanes < 128; ++lanes) {
            if (__builtin_popcount(lanes) != 5) continue;
            std::vector<int> S, W;
            for (int r = 0; r < 7; ++r) ((lanes >> r) & 1u ? S : W).push_back(rows0[r]);
            for (uint32_t sel = 0; sel < 32; ++sel) {
                if (__builtin_popcount(sel) != 5 - inphase0) continue;
                uint32_t order0[7];
                int c = 0;
                for (int i = 0; i < 5; ++i)
                    if (!((sel >> i) & 1u)) order0[c++] = 1u << S[i];
                for (int i = 0; i < 5; ++i)
                    if ((sel >> i) & 1u) order0[c++] = 1u << S[i];
                for (int w : W) order0[c++] = 1u << w;
                const long load = (v0 ? 16 : 32) * (long)warp_wavefronts(order0, pad, width0);
                if (best.cost >= 0 && load + 128 >= best.cost) continue;
                // block 1's gate bits: block 0's lane bits first (they then
                // select distinct banks through gate bits 0 and 1)
                std::vector<int> GL, GO, RL, RO;
                for (int i = 0; i < 5; ++i) {
                    const int j = __builtin_ctz(order0[i]);
                    ((gate1 >> j) & 1u ? GL : RL).push_back(j);
                }
                for (int j = 0; j < 12; ++j)
                    if (((gate1 >> j) & 1u) && std::find(GL.begin(), GL.end(), j) == GL.end()) GO.push_back(j);
                for (int j : rows1)
                    if (std::find(RL.begin(), RL.end(), j) == RL.end()) RO.push_back(j);
                int g1[5];
                for (size_t k = 0; k < GL.size(); ++k) g1[k] = GL[k];
                for (size_t k = 0; k < GO.size(); ++k) g1[GL.size() + k] = GO[k];
                // block 1's row bits: block 0's row lanes at rows 0-2 (their
                // bank bits in the operand layout), after the ones gate
                // bits 2-4 already take; the other rows fill the free lane
                // slots in every order for slots 3 and 4
                const int a = (int)GL.size();
                const int first = std::max(0, std::min(a - 2, 3 - (int)RL.size()));
                int slot_of_rl[5];
                for (size_t i = 0; i < RL.size(); ++i) slot_of_rl[i] = first + (int)i;
                std::vector<int> freeslots;
                for (int sl = 0; sl < 7; ++sl) {
                    bool taken = false;
                    for (size_t i = 0; i < RL.size(); ++i) taken = taken || slot_of_rl[i] == sl;
                    if (!taken) freeslots.push_back(sl);
                }
                // RO fills freeslots (same count); try each ordered pair for
                // the first two free slots at or above 3, the rest ascending
                const int nro = (int)RO.size();
                for (int p3 = 0; p3 < nro; ++p3)
                    for (int p4 = 0; p4 < nro; ++p4) {
                        if (p4 == p3) continue;
                        uint32_t order1[7];
                        for (size_t i = 0; i < RL.size(); ++i) order1[slot_of_rl[i]] = 1u << RL[i];
                        std::vector<int> rest;
                        for (int i = 0; i < nro; ++i)
                            if (i != p3 && i != p4) rest.push_back(RO[i]);
                        int ri = 0, hi_used = 0;
                        for (int sl : freeslots) {
                            if (sl >= 3 && hi_used == 0) {
                                order1[sl] = 1u << RO[p3];
                                ++hi_used;
                            } else if (sl >= 3 && hi_used == 1) {
                                order1[sl] = 1u << RO[p4];
                                ++hi_used;
                            } else {
                                order1[sl] = 1u << rest[ri++];
                            }
                        }
                        uint32_t pat[5];
                        for (int i = 0; i < 5; ++i) pat[i] = direct_bit_offset(__builtin_ctz(order0[i]), g1, order1);
                        const long scat = 64 * (long)scatter_wavefronts(pat);
                        const bool v1 = g1[0] == 0;
                        const long store = (v1 ? 16 : 32) * (long)warp_wavefronts(order1, pad, v1 ? 16 : 8);
                        const long cost = load + scat + store;
                        if (best.cost < 0 || cost < best.cost) {
                            best.cost = cost;
                            best.pad = pad;
                            std::memcpy(best.order[0], order0, sizeof(order0));
                            std::memcpy(best.order[1], order1, sizeof(order1));
                            std::memcpy(best.g1, g1, sizeof(g1));
                        }
                    }
            }
        }
        if (best.cost == ideal) break;
    }
    if (best.cost < 0) return false;
    if (!found) {
        std::lock_guard<std::mutex> lock(mu);
        if (memo.size() > 4096) memo.clear();
        memo.emplace(key, best);
    }
    // block 1 in its new gate order
    TcBlockGeom& G1 = o.blk[1];
    for (int g = 0; g < 32; ++g) {
        uint32_t jc = 0;
        for (int k = 0; k < 5; ++k)
            if ((g >> k) & 1) jc |= 1u << best.g1[k];
        G1.jgate[g] = jc;
    }
    G1.vec2 = G1.jgate[1] == 1u ? 1u : 0u;
    apply_layout(o, best.pad, best.order);
    for (int i = 0; i < 7; ++i)
        o.scat_row[0][i] = direct_bit_offset(__builtin_ctz(best.order[0][i]), best.g1, best.order[1]);
    for (int g = 0; g < 32; ++g) {
        uint32_t a = 0;
        for (int j = 0; j < 12; ++j)
            if ((o.blk[0].jgate[g] >> j) & 1u) a ^= direct_bit_offset(j, best.g1, best.order[1]);
        o.scat_gate[0][g] = a;
    }
    // both operand planes (2 x 16 KB) at 1024-byte aligned stage bases
    o.stage_bytes = (o.stage_bytes + 1023u) & ~1023u;
    o.direct = 1;
    o.shuffle = 0;
    std::memcpy(gbit1, best.g1, sizeof(best.g1));
    return true;
}

namespace {

// Offset, in block 0's A operand, of tile bit j: gate bit k (from gate
// order g0) at K index 2 * 2^k, row bit i (one-hot coordinates order0) at
// row 2^i; linear over GF(2) like direct_bit_offset.
uint32_t split_bit_offset(int j, const int* g0, const uint32_t* order0)
{
    for (int k = 0; k < 5; ++k)
        if (g0[k] == j) return tc_sw128_offset(0, 2u << k);
    for (int i = 0; i < 7; ++i)
        if (order0[i] == (1u << j)) return tc_sw128_offset(1u << i, 0);
    return 0;
}

// Wavefronts of one warp's 16-byte stores (quarter-warp phases of 8
// lanes) whose lane bits 0-2 move the address by pat[0..2] (XOR).
int sts128_wavefronts(const uint32_t* pat)
{
    int per_group[8] = {0};
    int m = 0;
    for (uint32_t l = 0; l < 8; ++l) {
        uint32_t a = 0;
        for (int r = 0; r < 3; ++r)
            if ((l >> r) & 1u) a ^= pat[r];
        m = std::max(m, ++per_group[(a >> 4) & 7u]);
    }
    return 4 * m;
}

}  // namespace

void tc_split_map(TcOffsets& o, int* gbit0)
{
    TcBlockGeom& G = o.blk[0];
    const uint32_t pad = o.pad_shift;
    std::vector<int> gates;
    for (int j = 0; j < 12; ++j)
        if ((G.jgate[31] >> j) & 1u) gates.push_back(j);
    // the last block's write-back reads rows (TMEM lanes) with the gate
    // pairs adjacent when gate bit 0 is tile bit 0
    auto wb_cost = [&](bool v2) {
        return o.nblocks == 1 ? (v2 ? 16 : 32) * (long)warp_wavefronts(G.jrow_bit, pad, v2 ? 16 : 8) : 0L;
    };
    long best = -1;
    int best_g[5] = {}, best_bits[12] = {};
    // the choice depends only on the geometry: remember it
    struct Choice {
        int g[5];
        int bits[12];
    };
    static std::mutex mu;
    static std::unordered_map<std::string, Choice> memo;
    std::string key(1, (char)o.nblocks);
    key.append((const char*)&pad, sizeof(pad));
    key.append((const char*)G.jrow_bit, sizeof(G.jrow_bit));
    key.append((const char*)&G.jgate[31], sizeof(uint32_t));
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = memo.find(key);
        if (it != memo.end()) {
            best = 0;
            std::memcpy(best_g, it->second.g, sizeof(best_g));
            std::memcpy(best_bits, it->second.bits, sizeof(best_bits));
        }
    }
    const bool known = best >= 0;
    for (int ia = 0; ia < 5 && !known; ++ia)
        for (int ib = ia + 1; ib < 5; ++ib) {
            int g[5] = {gates[ia], gates[ib], 0, 0, 0};
            int c = 2;
            for (int k = 0; k < 5; ++k)
                if (k != ia && k != ib) g[c++] = gates[k];
            std::vector<int> rest;
            for (int j = 0; j < 12; ++j)
                if (j != g[0] && j != g[1]) rest.push_back(j);
            const bool v2 = g[0] == 0;
            const int width = v2 ? 16 : 8, nld = v2 ? 16 : 32;
            const long wb = wb_cost(v2);
            // lane bits 0-3 from the 10 other bits: which 4, and which of
            // them is lane bit 3 (outside the 16-byte stores' phase)
            for (uint32_t m4 = 0; m4 < 1024; ++m4) {
                if (__builtin_popcount(m4) != 4) continue;
                int P[4], n = 0, l4 = -1;
                for (int r = 0; r < 10; ++r) {
                    if ((m4 >> r) & 1u) P[n++] = rest[r];
                    else if (l4 < 0) l4 = rest[r];
                }
                for (int h = 0; h < 4; ++h) {
                    int lane[5], q = 0;
                    for (int e = 0; e < 4; ++e)
                        if (e != h) lane[q++] = P[e];
                    lane[3] = P[h];
                    lane[4] = l4;
                    uint32_t ord[7];
                    for (int e = 0; e < 5; ++e) ord[e] = 1u << lane[e];
                    ord[5] = ord[6] = 0;
                    const long ld = nld * (long)warp_wavefronts(ord, pad, width);
                    uint32_t pat[3];
                    for (int e = 0; e < 3; ++e) pat[e] = split_bit_offset(lane[e], g, G.jrow_bit);
                    const long cost = ld + 16 * (long)sts128_wavefronts(pat) + wb;
                    if (best < 0 || cost < best) {
                        best = cost;
                        std::memcpy(best_g, g, sizeof(g));
                        // lanes 0-4, warps 5-6, registers 2-4: the rest ascending
                        int bits[12], b = 0;
                        for (int e = 0; e < 5; ++e) bits[b++] = lane[e];
                        for (int j : rest) {
                            bool used = false;
                            for (int e = 0; e < 5; ++e) used = used || lane[e] == j;
                            if (!used) bits[b++] = j;
                        }
                        std::memcpy(best_bits, bits, sizeof(bits));
                    }
                }
            }
        }
    {
        std::lock_guard<std::mutex> lock(mu);
        if (memo.size() > 4096) memo.clear();
        Choice c;
        std::memcpy(c.g, best_g, sizeof(best_g));
        std::memcpy(c.bits, best_bits, sizeof(best_bits));
        memo.emplace(key, c);
    }
    // bits 0-4 lanes, 5-6 warps, 7-9 registers 2-4 (10 of the 12 tile bits;
    // gate bits 0-1 are registers 0-1)
    for (int k = 0; k < 5; ++k) gbit0[k] = best_g[k];
    for (int gi = 0; gi < 32; ++gi) {
        uint32_t jc = 0;
        for (int k = 0; k < 5; ++k)
            if ((gi >> k) & 1) jc |= 1u << best_g[k];
        G.jgate[gi] = jc;
        G.gateoff[gi] = staged_offset(jc, pad);
    }
    G.vec2 = best_g[0] == 0 ? 1u : 0u;
    o.sp_vec2 = G.vec2;
    for (int i = 0; i < 7; ++i) {
        o.sp_thoff[i] = staged_offset(1u << best_bits[i], pad);
        o.sp_athr[i] = split_bit_offset(best_bits[i], best_g, G.jrow_bit);
    }
    const int reg[5] = {best_g[0], best_g[1], best_bits[7], best_bits[8], best_bits[9]};
    for (int j = 0; j < 32; ++j) {
        uint32_t x = 0;
        for (int k = 0; k < 5; ++k)
            if ((j >> k) & 1) x |= 1u << reg[k];
        o.sp_regoff[j] = staged_offset(x, pad);
    }
    for (int q = 0; q < 8; ++q) {
        uint32_t a = 0;
        for (int k = 0; k < 3; ++k)
            if ((q >> k) & 1) a ^= split_bit_offset(reg[2 + k], best_g, G.jrow_bit);
        o.sp_achunk[q] = a;
    }
    if (o.direct) {
        // the scatter table follows block 0's new gate order
        int g1[5];
        for (int k = 0; k < 5; ++k) g1[k] = __builtin_ctz(o.blk[1].jgate[1 << k]);
        for (int gi = 0; gi < 32; ++gi) {
            uint32_t a = 0;
            for (int j = 0; j < 12; ++j)
                if ((G.jgate[gi] >> j) & 1u) a ^= direct_bit_offset(j, g1, o.blk[1].jrow_bit);
            o.scat_gate[0][gi] = a;
        }
    }
}

bool tc_chain_layout(TcOffsets& o, bool tma_ok, int conflict_slack, int (*gbits)[5], long* cost_out,
                     long* ideal_out, const std::vector<TcStoreBox>* stores, int* store_out)
{
    if (stores && stores->empty()) stores = nullptr;
    const int nb = (int)o.nblocks;
    if (nb < 2 || nb > kTcMaxBlocks) return false;
    uint32_t gate[kTcMaxBlocks];
    std::vector<int> rows[kTcMaxBlocks];
    for (int b = 0; b < nb; ++b) {
        gate[b] = o.blk[b].jgate[31];
        if (__builtin_popcount(gate[b]) != 5) return false;
        for (int j = 0; j < 12; ++j)
            if (!((gate[b] >> j) & 1u)) rows[b].push_back(j);
    }
    // per warp: 64 scattered 4-byte stores per transition, the last block's
    // write-back (32 8-byte or 16 16-byte stores)
    const long ideal = 64L * nb;
    struct Best {
        long cost = -1;
        uint32_t pad = 31;
        uint32_t order[kTcMaxBlocks][7] = {};
        int g[kTcMaxBlocks][5] = {};
        int store = -1;
        uint32_t wxor[5] = {};
    } best;
    static std::mutex mu;
    static std::unordered_map<std::string, Best> memo;
    std::string key(1, tma_ok ? 'T' : 'P');
    key.append((const char*)&conflict_slack, sizeof(conflict_slack));
    key.append((const char*)&o.run_bits, sizeof(o.run_bits));
    key.append((const char*)gate, sizeof(uint32_t) * nb);
    if (stores) {
        // the store boxes follow from the tile's runs and the last gates
        for (const auto& sb : *stores) key.append((const char*)sb.sbit, sizeof(sb.sbit));
    }
    bool found = false;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = memo.find(key);
        if (it != memo.end()) {
            best = it->second;
            found = true;
        }
    }
    uint32_t order[kTcMaxBlocks][7];
    int g[kTcMaxBlocks][5];
    uint32_t pad = 31;
    // transition k -> k+1 from block k's lanes (order[k][0..4]); cost so far
    std::function<void(int, long)> step = [&](int k, long cost) {
        int lanes[5];
        for (int i = 0; i < 5; ++i) lanes[i] = __builtin_ctz(order[k][i]);
        const uint32_t gn = gate[k + 1];
        std::vector<int> GL, RL, GO, RO;
        for (int i = 0; i < 5; ++i) ((gn >> lanes[i]) & 1u ? GL : RL).push_back(lanes[i]);
        std::sort(GL.begin(), GL.end());
        std::sort(RL.begin(), RL.end());
        for (int j = 0; j < 12; ++j)
            if (((gn >> j) & 1u) && std::find(GL.begin(), GL.end(), j) == GL.end()) GO.push_back(j);
        for (int j : rows[k + 1])
            if (std::find(RL.begin(), RL.end(), j) == RL.end()) RO.push_back(j);
        int* gk = g[k + 1];
        for (size_t i = 0; i < GL.size(); ++i) gk[i] = GL[i];
        for (size_t i = 0; i < GO.size(); ++i) gk[GL.size() + i] = GO[i];
        // the lanes that are rows of block k+1 take its row bits (a-2)..2,
        // after the ones its gate bits 2-4 already take (a conflict-free
        // scatter when a >= 2)
        const int a = (int)GL.size();
        const int first = std::max(0, std::min(a - 2, 3 - (int)RL.size()));
        bool taken[7] = {};
        for (size_t i = 0; i < RL.size(); ++i) taken[first + i] = true;
        std::vector<int> FL, FW;
        for (int sl = 0; sl < 7; ++sl)
            if (!taken[sl]) (sl < 5 ? FL : FW).push_back(sl);
        const bool last = k + 2 == nb;
        const int nro = (int)RO.size(), nfl = (int)FL.size();
        auto fill = [&](const std::vector<int>& lane_bits, int at4) {
            // lane_bits into the free lane slots (at4: the one for slot 4,
            // -1 if none), the rest of RO into the warp slots, ascending
            uint32_t* ok1 = order[k + 1];
            for (size_t i = 0; i < RL.size(); ++i) ok1[first + i] = 1u << RL[i];
            size_t li = 0;
            for (int sl : FL) {
                if (sl == 4 && at4 >= 0) ok1[sl] = 1u << at4;
                else {
                    while (li < lane_bits.size() && lane_bits[li] == at4) ++li;
                    ok1[sl] = 1u << lane_bits[li++];
                }
            }
            size_t wi = 0;
            for (int j : RO)
                if (std::find(lane_bits.begin(), lane_bits.end(), j) == lane_bits.end()) ok1[FW[wi++]] = 1u << j;
        };
        auto scatter_cost = [&]() {
            uint32_t pat[5];
            for (int i = 0; i < 5; ++i) pat[i] = direct_bit_offset(lanes[i], gk, order[k + 1]);
            return 64L * scatter_wavefronts(pat);
        };
        if (last) {
            // every choice of the lane rows, and of the one in slot 4 (it
            // selects the write-back's phase)
            const bool v2 = gk[0] == 0;
            const int width = v2 ? 16 : 8, nwb = v2 ? 16 : 32;
            const bool slot4_free = std::find(FL.begin(), FL.end(), 4) != FL.end();
            for (uint32_t m = 0; m < (1u << nro); ++m) {
                if (__builtin_popcount(m) != nfl) continue;
                std::vector<int> lb;
                for (int i = 0; i < nro; ++i)
                    if ((m >> i) & 1u) lb.push_back(RO[i]);
                const size_t n4 = slot4_free ? lb.size() : 1;
                for (size_t c4 = 0; c4 < n4; ++c4) {
                    fill(lb, slot4_free ? lb[c4] : -1);
                    // the write-back in the load layout, or (unpadded) in
                    // the best store box
                    // (lane-permuted stores where the layout is linear)
                    long wb = -1;
                    int si = -1;
                    uint32_t wx[5] = {0, 0, 0, 0, 0};
                    auto permuted = [&](const int* sbit, uint32_t* ph) {
                        int plain = 0;
                        const long w = nwb * (long)warp_wavefronts_xor(order[k + 1], sbit, gk, width, ph, &plain) +
                                       kWbButterflyCost * (width == 16 ? 3 : 4);
                        if (w < nwb * (long)plain) return w;
                        for (int r = 0; r < 5; ++r) ph[r] = 0;
                        return nwb * (long)plain;
                    };
                    if (stores && pad >= 31) {
                        for (size_t c = 0; c < stores->size(); ++c) {
                            uint32_t ph[5];
                            const long w = permuted((*stores)[c].sbit, ph);
                            if (wb < 0 || w < wb) {
                                wb = w;
                                si = (int)c;
                                std::memcpy(wx, ph, sizeof(wx));
                            }
                        }
                    } else if (pad >= 31) {
                        wb = permuted(nullptr, wx);
                    } else {
                        wb = nwb * (long)warp_wavefronts(order[k + 1], pad, width);
                    }
                    const long total = cost + scatter_cost() + wb;
                    if (best.cost < 0 || total < best.cost) {
                        best.cost = total;
                        best.pad = pad;
                        std::memcpy(best.order, order, sizeof(order));
                        std::memcpy(best.g, g, sizeof(g));
                        best.store = si;
                        std::memcpy(best.wxor, wx, sizeof(wx));
                    }
                }
            }
        } else {
            // a middle block's lane rows: the next block's gate bits first
            // (its scatter then has gate lanes), or simply the lowest
            std::vector<int> pref = RO;
            std::stable_sort(pref.begin(), pref.end(), [&](int x, int y) {
                return ((gate[k + 2] >> x) & 1u) > ((gate[k + 2] >> y) & 1u);
            });
            for (int variant = 0; variant < 2; ++variant) {
                std::vector<int> lb(variant == 0 ? pref.begin() : RO.begin(),
                                    (variant == 0 ? pref.begin() : RO.begin()) + nfl);
                std::sort(lb.begin(), lb.end());
                fill(lb, -1);
                const long c = cost + scatter_cost();
                if (best.cost >= 0 && c + 64L * (nb - k - 1) >= best.cost) continue;
                step(k + 1, c);
            }
        }
    };
    const uint32_t cands[] = {31, 11, 10, 9, 8, 7, 6, 5};
    for (uint32_t pc : cands) {
        if (found) break;
        if (pc < 31 && tma_ok && best.cost >= 0 && best.cost <= conflict_slack * ideal) break;
        pad = pc;
        for (uint32_t lm = 0; lm < 128; ++lm) {
            if (__builtin_popcount(lm) != 5) continue;
            int c = 0;
            for (int r = 0; r < 7; ++r)
                if ((lm >> r) & 1u) order[0][c++] = 1u << rows[0][r];
            for (int r = 0; r < 7; ++r)
                if (!((lm >> r) & 1u)) order[0][c++] = 1u << rows[0][r];
            step(0, 0);
            if (best.cost == ideal) break;
        }
        if (best.cost == ideal) break;
    }
    if (best.cost < 0) return false;
    if (!found) {
        std::lock_guard<std::mutex> lock(mu);
        if (memo.size() > 4096) memo.clear();
        memo.emplace(key, best);
    }
    if (cost_out) *cost_out = best.cost;
    if (ideal_out) *ideal_out = ideal;
    // later blocks in their new gate orders
    for (int b = 1; b < nb; ++b) {
        TcBlockGeom& G = o.blk[b];
        for (int gi = 0; gi < 32; ++gi) {
            uint32_t jc = 0;
            for (int k = 0; k < 5; ++k)
                if ((gi >> k) & 1) jc |= 1u << best.g[b][k];
            G.jgate[gi] = jc;
        }
        G.vec2 = G.jgate[1] == 1u ? 1u : 0u;
        for (int k = 0; k < 5; ++k) gbits[b][k] = best.g[b][k];
    }
    apply_layout(o, best.pad, best.order);
    for (int k = 0; k + 1 < nb; ++k) {
        for (int i = 0; i < 7; ++i)
            o.scat_row[k][i] = direct_bit_offset(__builtin_ctz(best.order[k][i]), best.g[k + 1], best.order[k + 1]);
        for (int gi = 0; gi < 32; ++gi) {
            uint32_t a = 0;
            for (int j = 0; j < 12; ++j)
                if ((o.blk[k].jgate[gi] >> j) & 1u) a ^= direct_bit_offset(j, best.g[k + 1], best.order[k + 1]);
            o.scat_gate[k][gi] = a;
        }
    }
    o.stage_bytes = (o.stage_bytes + 1023u) & ~1023u;
    o.direct = 1;
    o.shuffle = 0;
    o.st_box = 0;
    for (int r = 0; r < 5; ++r) o.wb_xor[r] = best.wxor[r];
    if (store_out) *store_out = best.store;
    if (stores && best.store >= 0) {
        // the last block writes the chosen store box's layout
        const TcStoreBox& sb = (*stores)[best.store];
        TcBlockGeom& L = o.blk[nb - 1];
        auto off = [&](uint32_t x) {
            uint32_t a = 0;
            for (int j = 0; j < 12; ++j)
                if ((x >> j) & 1u) a += 8u << sb.sbit[j];
            return a;
        };
        for (int r = 0; r < 7; ++r) L.rowoff[r] = off(L.jrow_bit[r]);
        for (int gi = 0; gi < 32; ++gi) L.gateoff[gi] = off(L.jgate[gi]);
        if (best.store > 0) {
            o.st_box = 1;
            for (int d = 0; d < 5; ++d) {
                o.st_tshift[d] = sb.box.tshift[d];
                o.st_tmask[d] = sb.box.tmask[d];
            }
        }
    }
    return true;
}

void tc_choose_padding(TcOffsets& o, bool tma_ok, int conflict_slack)
{
    // The choice depends only on the tile geometry (and the slack), which
    // repeats from run to run of a plan: remember it.
    struct Choice {
        uint32_t pad;
        uint32_t order[kTcMaxBlocks][7];
    };
    static std::mutex mu;
    static std::unordered_map<std::string, Choice> memo;
    std::string key(1, tma_ok ? 'T' : 'P');
    key.append(1, o.shuffle ? 'S' : 'N');
    key.append((const char*)&conflict_slack, sizeof(conflict_slack));
    key.append((const char*)&o.nblocks, sizeof(o.nblocks));
    key.append((const char*)&o.run_bits, sizeof(o.run_bits));
    for (uint32_t b = 0; b < o.nblocks; ++b) {
        key.append((const char*)o.blk[b].jrow_bit, sizeof(o.blk[b].jrow_bit));
        key.append((const char*)o.blk[b].jgate, sizeof(o.blk[b].jgate));
    }
    Choice ch{};
    bool found = false;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = memo.find(key);
        if (it != memo.end()) {
            ch = it->second;
            found = true;
        }
    }
    if (!found) {
        // candidates: unpadded, then 16 B every 2^pad amplitudes (fewest
        // pieces first); per block the row order that suits the padding best
        // (a shuffled pass keeps its row layout: only block 0 reads the stage
        // and only block 1 writes it)
        const uint32_t cands[] = {31, 11, 10, 9, 8, 7, 6, 5};
        long best = -1, ideal = 0;
        for (uint32_t b = 0; b < o.nblocks; ++b) ideal += o.blk[b].vec2 ? 16 * 4 : 32 * 2;
        for (uint32_t pad : cands) {
            if (pad < 31 && tma_ok && best >= 0 && best <= conflict_slack * ideal) break;   // keep the tensor-map copy
            long cost = 0;
            uint32_t order[kTcMaxBlocks][7] = {};
            for (uint32_t b = 0; b < o.nblocks; ++b) {
                if (o.shuffle) {
                    std::memcpy(order[b], o.blk[b].jrow_bit, sizeof(order[b]));
                    cost += (o.blk[b].vec2 ? 16 : 32) * warp_wavefronts(order[b], pad, o.blk[b].vec2 ? 16 : 8);
                } else {
                    cost += (o.blk[b].vec2 ? 16 : 32) * best_row_order(o.blk[b], pad, order[b]);
                }
            }
            if (best < 0 || cost < best) {
                best = cost;
                ch.pad = pad;
                std::memcpy(ch.order, order, sizeof(order));
                if (best == ideal) break;
            }
        }
        std::lock_guard<std::mutex> lock(mu);
        if (memo.size() > 4096) memo.clear();
        memo.emplace(key, ch);
    }
    apply_layout(o, ch.pad, ch.order);
}

bool tc_shuffle_layout(TcBlockGeom& b0, TcBlockGeom& b1, int32_t* swap_lane, int* reg1)
{
    // register bit k of block 0 holds tile bit r0[k]; block 1's gates are the
    // tile bits set in its jgate table
    int r0[5];
    uint32_t gates0 = 0, gates1 = 0;
    for (int k = 0; k < 5; ++k) {
        r0[k] = __builtin_ctz(b0.jgate[1 << k]);
        gates0 |= 1u << r0[k];
        gates1 |= b1.jgate[1 << k];
    }
    if (__builtin_popcount(gates0) != 5 || __builtin_popcount(gates1) != 5) return false;
    std::vector<int> s1, s2, common;   // leaving the gates, entering them, rows of both
    for (int j = 0; j < 12; ++j) {
        const bool in0 = (gates0 >> j) & 1u, in1 = (gates1 >> j) & 1u;
        if (in0 && !in1) s1.push_back(j);
        if (in1 && !in0) s2.push_back(j);
        if (!in0 && !in1) common.push_back(j);
    }
    const int s = (int)s1.size();
    if ((int)s2.size() != s || (int)common.size() != 7 - s) return false;
    // lanes: the lowest common rows first (one warp phase reads them as
    // contiguous amplitudes), the bits that swap at the top; the two other
    // common rows select the warp
    int lane0[5], lane1[5];
    for (int b = 0; b < 5 - s; ++b) lane0[b] = lane1[b] = common[b];
    for (int i = 0; i < s; ++i) {
        lane0[5 - s + i] = s2[i];
        lane1[5 - s + i] = s1[i];
    }
    for (int k = 0; k < 5; ++k) {
        swap_lane[k] = -1;
        reg1[k] = r0[k];
    }
    for (int i = 0; i < s; ++i)
        for (int k = 0; k < 5; ++k)
            if (r0[k] == s1[i]) {
                swap_lane[k] = 5 - s + i;
                reg1[k] = s2[i];
            }
    for (int b = 0; b < 5; ++b) {
        b0.jrow_bit[b] = 1u << lane0[b];
        b1.jrow_bit[b] = 1u << lane1[b];
    }
    for (int w = 0; w < 2; ++w) b0.jrow_bit[5 + w] = b1.jrow_bit[5 + w] = 1u << common[5 - s + w];
    for (int g = 0; g < 32; ++g) {
        uint32_t jc = 0;
        for (int k = 0; k < 5; ++k)
            if ((g >> k) & 1) jc |= 1u << reg1[k];
        b1.jgate[g] = jc;
    }
    b1.vec2 = b1.jgate[1] == 1u ? 1u : 0u;
    return true;
}

void build_tc_image(const double* m, uint16_t* image, int scale_log2)
{
    // R[n][k]: n = 2g'+c' output component, k = 2g+c input component, times
    // 2^scale_log2.  Rows n of B_hi and 64+n of B_lo' (= 2^11 lo) as f16,
    // K-major, SWIZZLE_128B: 8-row groups of 1024 B, 16-byte chunk j of row r
    // at chunk position j ^ (r & 7).  Entries below f16's normal range keep
    // their remainder in B_lo' (scaled by 2^11), to 2^-35 absolute.
    const double bs = std::ldexp(1.0, scale_log2);
    for (int gp = 0; gp < 32; ++gp)
        for (int g = 0; g < 32; ++g) {
            const double re = m[2 * (gp * 32 + g)], im = m[2 * (gp * 32 + g) + 1];
            const double rv[2][2] = {{re, -im}, {im, re}};
            for (int cp = 0; cp < 2; ++cp)
                for (int c = 0; c < 2; ++c) {
                    const int n = 2 * gp + cp, k = 2 * g + c;
                    const double v = rv[cp][c] * bs;
                    double hi = 0.0, lo = 0.0;
                    const uint16_t hb = host_f16_bits(v, &hi);
                    const uint16_t lb = host_f16_bits((v - hi) * 2048.0, &lo);
                    for (int half = 0; half < 2; ++half) {
                        const int row = n + 64 * half;
                        const size_t off = (size_t)(row >> 3) * 1024 + (size_t)(row & 7) * 128 +
                                           (size_t)(((k >> 3) ^ (row & 7)) << 4) + (size_t)(k & 7) * 2;
                        image[off / 2] = half ? lb : hb;
                    }
                }
        }
}

void tc_operand_scales(double max_norm, TcOffsets& offs)
{
    // |amplitude| <= sqrt(column norm) <= 2^e: amplitudes enter the tensor
    // cores times 2^(14-e), at most 2^14 (f16 holds up to 65504), so that
    // those above 2^(-28+e) are normal f16 numbers.  They stay scaled from
    // block to block; the last block's B carries 2^kTcLastBScaleLog2 and its
    // epilogue multiplies by `unscale`.
    int e = 0;
    if (max_norm > 0.0 && std::isfinite(max_norm)) e = (int)std::ceil(0.5 * std::log2(max_norm));
    e = std::max(-60, std::min(60, e));
    offs.ascale = std::ldexp(1.0f, 14 - e);
    offs.unscale = std::ldexp(1.0f, -(14 - e) - kTcLastBScaleLog2);
}

bool tc_block_bounded(const std::complex<double>* m, int dim)
{
    // every output amplitude is a row of m times the input: with row
    // 2-norms <= 1 it stays within the column norm (true of unitary blocks)
    for (int r = 0; r < dim; ++r) {
        double s = 0.0;
        for (int c = 0; c < dim; ++c) s += std::norm(m[(size_t)r * dim + c]);
        if (!(s <= 1.0 + 1e-6)) return false;
    }
    return true;
}

TcTileBox tc_tile_box(const int* tile_pos, int nbits, uint64_t ncols)
{
    TcTileBox b{};
    std::vector<char> in_tile(nbits, 0);
    for (int j = 0; j < 12; ++j) in_tile[tile_pos[j]] = 1;
    int nd = 0;
    uint32_t below = 0;      // tile-index bits used by the dimensions so far
    bool top_outside = false;
    auto add = [&](int first, int len, bool tile) {
        if (nd == 5) {
            nd = 6;
            return;
        }
        b.gdim[nd] = uint64_t(1) << len;
        b.gstride[nd] = uint64_t(8) << first;
        b.box[nd] = tile ? (1u << len) : 1u;
        b.tshift[nd] = tile ? 0u : below;
        b.tmask[nd] = tile ? 0u : (uint32_t)((uint64_t(1) << len) - 1);
        if (!tile) below += (uint32_t)len;
        ++nd;
    };
    for (int p = 0; p < nbits && nd <= 5;) {
        int q = p;
        while (q < nbits && in_tile[q] == in_tile[p]) ++q;
        if (in_tile[p]) {
            for (int f = p; f < q; f += 8) add(f, std::min(8, q - f), true);   // box dims <= 256
        } else {
            add(p, q - p, false);
        }
        top_outside = !in_tile[p];
        p = q;
    }
    if (nd <= 5 && ncols > 1) {
        if (top_outside) {
            // the column index continues the top dimension
            b.gdim[nd - 1] *= ncols;
            b.tmask[nd - 1] = 0xFFFFFFFFu;
        } else {
            add(nbits, 0, false);
            if (nd <= 5) {
                b.gdim[nd - 1] = ncols;
                b.tmask[nd - 1] = 0xFFFFFFFFu;
            }
        }
    }
    // dimension 0 must be a tile dimension (its coordinate, the innermost
    // one, is then always 0) and the box must be the whole tile
    b.usable = nd >= 1 && nd <= 5 && b.tmask[0] == 0;
    uint64_t elems = 1;
    for (int d = 0; d < nd && b.usable; ++d) {
        if (b.gdim[d] > (uint64_t(1) << 32)) b.usable = 0;
        elems *= b.box[d];
    }
    if (elems != 4096) b.usable = 0;
    if (!b.usable) return b;
    for (int d = nd; d < 5; ++d) {
        b.gdim[d] = 1;
        b.gstride[d] = b.gstride[d - 1] * b.gdim[d - 1];
        b.box[d] = 1;
        b.tshift[d] = 0;
        b.tmask[d] = 0;
    }
    return b;
}

std::vector<TcStoreBox> tc_store_boxes(const int* tile_pos, int nbits, uint64_t ncols, uint32_t gates)
{
    std::vector<TcStoreBox> out;
    {
        TcStoreBox id{};
        id.box = tc_tile_box(tile_pos, nbits, ncols);
        if (!id.box.usable) return out;
        for (int j = 0; j < 12; ++j) id.sbit[j] = j;
        out.push_back(id);
    }
    // runs of consecutive tile positions, as tile-bit ranges
    std::vector<std::pair<int, int>> runs;   // (first tile bit, length)
    for (int j = 0; j < 12;) {
        int k = j + 1;
        while (k < 12 && tile_pos[k] == tile_pos[k - 1] + 1) ++k;
        runs.push_back({j, k - j});
        j = k;
    }
    // the gap dimensions (box 1) in position order, as tc_tile_box makes them
    std::vector<char> in_tile(nbits, 0);
    for (int j = 0; j < 12; ++j) in_tile[tile_pos[j]] = 1;
    struct Dim {
        uint64_t gdim, gstride;
        uint32_t box, tshift, tmask;
    };
    std::vector<Dim> gaps;
    {
        uint32_t below = 0;
        bool top_outside = false;
        for (int p = 0; p < nbits;) {
            int q = p;
            while (q < nbits && in_tile[q] == in_tile[p]) ++q;
            if (!in_tile[p]) {
                gaps.push_back({uint64_t(1) << (q - p), uint64_t(8) << p, 1u, below,
                                (uint32_t)((uint64_t(1) << (q - p)) - 1)});
                below += (uint32_t)(q - p);
            }
            top_outside = !in_tile[p];
            p = q;
        }
        if (ncols > 1) {
            if (top_outside) {
                gaps.back().gdim *= ncols;
                gaps.back().tmask = 0xFFFFFFFFu;
            } else {
                gaps.push_back({ncols, uint64_t(8) << nbits, 1u, below, 0xFFFFFFFFu});
            }
        }
    }
    // dimension 0 is the stores' contiguous run in memory: at least 8
    // amplitudes (64 bytes) or the whole first run, so that no store box
    // writes shorter runs than the tile has
    const int s_max = std::min(8, runs[0].second);
    for (int s0 = std::min(3, runs[0].second); s0 <= s_max; ++s0) {
        // the other tile bits cut into pieces of one role (row or gate of
        // the last block), within a run, of at most 8 bits; rows first
        std::vector<std::pair<int, int>> rowp, gatep;
        for (size_t r = 0; r < runs.size(); ++r) {
            int j = r == 0 ? s0 : runs[r].first;
            const int end = runs[r].first + runs[r].second;
            while (j < end) {
                const bool g = (gates >> j) & 1u;
                int k = j + 1;
                while (k < end && (((gates >> k) & 1u) != 0) == g && k - j < 8) ++k;
                (g ? gatep : rowp).push_back({j, k - j});
                j = k;
            }
        }
        std::vector<std::pair<int, int>> pieces = {{0, s0}};
        pieces.insert(pieces.end(), rowp.begin(), rowp.end());
        pieces.insert(pieces.end(), gatep.begin(), gatep.end());
        if (pieces.size() + gaps.size() > 5) continue;
        TcStoreBox c{};
        int nd = 0, acc = 0;
        for (auto& pc : pieces) {
            c.box.gdim[nd] = c.box.box[nd] = 1u << pc.second;
            c.box.gstride[nd] = uint64_t(8) << tile_pos[pc.first];
            c.box.tshift[nd] = 0;
            c.box.tmask[nd] = 0;
            for (int e = 0; e < pc.second; ++e) c.sbit[pc.first + e] = acc + e;
            acc += pc.second;
            ++nd;
        }
        for (auto& g : gaps) {
            c.box.gdim[nd] = g.gdim;
            c.box.gstride[nd] = g.gstride;
            c.box.box[nd] = g.box;
            c.box.tshift[nd] = g.tshift;
            c.box.tmask[nd] = g.tmask;
            ++nd;
        }
        bool ok = true;
        for (int d = 0; d < nd; ++d) ok = ok && c.box.gdim[d] <= (uint64_t(1) << 32);
        if (!ok) continue;
        for (int d = nd; d < 5; ++d) {
            c.box.gdim[d] = 1;
            c.box.gstride[d] = c.box.gstride[d - 1] * c.box.gdim[d - 1];
            c.box.box[d] = 1;
            c.box.tshift[d] = 0;
            c.box.tmask[d] = 0;
        }
        c.box.usable = 1;
        bool same = true;
        for (int j = 0; j < 12; ++j) same = same && c.sbit[j] == j;
        if (!same) out.push_back(c);
    }
    return out;
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}
}  // namespace

cudaError_t launch_fused_tc(float2* amps, uint64_t ntiles, const IndexMap& tilemap, const TcOffsets& offs_in,
                            const TcTileBox& box, const void* d_bimage, int* d_err, int sm_count,
                            cudaStream_t st, uint64_t wait_ns, const TcTileBox* store_box)
{
    static std::mutex mu;
    static int optin[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!optin[dev]) {
            int v = 0;
            e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            if (e != cudaSuccess) return e;
            e = cudaFuncSetAttribute(k_fused_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
            if (e != cudaSuccess) return e;
            e = cudaFuncSetAttribute(k_fused_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
            if (e != cudaSuccess) return e;
            optin[dev] = v;
        }
    }
    TcOffsets offs = offs_in;
    offs.wait_ns = wait_ns ? wait_ns : kTcDefaultWaitNs;
    const uint32_t ng = offs.groups == 4 ? 4u : 2u;
    const uint32_t fixed = kAlignSlack + kOffB + offs.nblocks * kBImage;
    // four groups hold four stages: at least one more for the copies;
    // operands in shared memory need 1024-byte aligned stages
    const uint32_t min_stages = ng == 4 ? 5u : 3u;
    // three blocks only as a direct chain of the four-group kernel
    if (offs.nblocks < 1 || offs.nblocks > (ng == 4 && offs.direct ? 3u : 2u) || offs.stage_bytes < kTileBytes ||
        ((ng == 4 || offs.direct) && offs.stage_bytes % 1024u) ||
        (uint32_t)optin[dev] < fixed + min_stages * offs.stage_bytes)
        return cudaErrorInvalidConfiguration;
    offs.nstages = std::min(kMaxStages, ((uint32_t)optin[dev] - fixed) / offs.stage_bytes);
    const uint32_t smem = fixed + offs.nstages * offs.stage_bytes;
    // unpadded tiles: one tensor-map box per tile
    CUtensorMap tmap, tmap_st;
    std::memset(&tmap, 0, sizeof(tmap));
    std::memset(&tmap_st, 0, sizeof(tmap_st));
    offs.use_tma = 0;
    EncodeTiledFn enc = encode_tiled();
    auto encode = [&](CUtensorMap* m, const TcTileBox& b) {
        cuuint64_t gdim[5], gstride[4];
        cuuint32_t bdim[5], estride[5] = {1, 1, 1, 1, 1};
        for (int d = 0; d < 5; ++d) {
            gdim[d] = b.gdim[d];
            bdim[d] = b.box[d];
            if (d > 0) gstride[d - 1] = b.gstride[d];
        }
        return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, amps, gdim, gstride, bdim, estride,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    if (offs.pad_shift >= 31 && box.usable && enc && encode(&tmap, box)) {
        offs.use_tma = 1;
        for (int d = 0; d < 5; ++d) {
            offs.tshift[d] = box.tshift[d];
            offs.tmask[d] = box.tmask[d];
        }
    }
    // the last block's write-back follows the store box: without it (or
    // its map) the pass cannot run
    if (offs.st_box && (!offs.use_tma || !store_box || !store_box->usable || !encode(&tmap_st, *store_box)))
        return cudaErrorInvalidConfiguration;
    // the piece path has a table of 32 runs: a tile of more runs must go as
    // one tensor-map box
    if (!offs.use_tma && (offs.nruns > 32 || offs.npieces > 4096u >> 5)) return cudaErrorInvalidConfiguration;
    uint64_t grid = (uint64_t)sm_count;
    if (grid > ntiles) grid = ntiles;
    if (grid == 0) return cudaSuccess;
    if (ng == 4)
        k_fused_tc<4><<<(unsigned)grid, TcShape<4>::kThreads, smem, st>>>(amps, ntiles, tilemap, offs, tmap, tmap_st,
                                                                          (const uint4*)d_bimage, d_err);
    else
        k_fused_tc<2><<<(unsigned)grid, TcShape<2>::kThreads, smem, st>>>(amps, ntiles, tilemap, offs, tmap, tmap_st,
                                                                          (const uint4*)d_bimage, d_err);
    return cudaGetLastError();
}

}  // namespace q1g
