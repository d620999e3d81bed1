// Measurement kernels: |amp|^2 reductions, FP64 prefix sums, sorted-uniform
// generation and binary-search shot sampling.
//
// They replace the reference's per-column `WeightedIndex::new(|a|^2)` +
// `sample_iter` (src/vectorstate.rs:119-133) and the w0 block sums of
// measure_into / peek_into (src/vectorstate.rs:252-261, 361-370).  All sums
// are FP64 with a fixed reduction order, so repeated runs give identical
// results.
#include "common.cuh"
#include <algorithm>

#include "kernels.h"
#include "sampling.cuh"

namespace q1g {

namespace {

template <typename T>
__device__ __forceinline__ double norm_sqr(T v)
{
    const double x = (double)v.x, y = (double)v.y;
    return x * x + y * y;
}

// Sum of v over the block (blockDim.x a multiple of 32, <= 1024); result in
// thread 0.  Fixed order: lanes by xor-butterfly, then warps in index order.
__device__ double block_sum(double v, double* red)
{
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    __syncthreads();
    return s;
}

// --------------------------------------------------------- chunk sums

template <typename T>
__global__ void __launch_bounds__(256)
k_chunk_sums(const T* __restrict__ a, uint64_t units, uint64_t chunk, IndexMap map, double* out)
{
    __shared__ double red[32];
    const uint64_t nchunks = units / chunk;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        double acc = 0.0;
        const uint64_t j0 = c * chunk;
        for (uint64_t j = threadIdx.x; j < chunk; j += blockDim.x)
            acc += norm_sqr(a[expand_index(j0 + j, map)]);
        const double s = block_sum(acc, red);
        if (threadIdx.x == 0) out[c] = s;
    }
}

__global__ void __launch_bounds__(256)
k_segment_sums(const double* __restrict__ in, uint64_t len, double* out)
{
    __shared__ double red[32];
    const uint64_t s0 = uint64_t(blockIdx.x) * len;
    double acc = 0.0;
    for (uint64_t j = threadIdx.x; j < len; j += blockDim.x) acc += in[s0 + j];
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// First level of a long segment reduction: block b sums part b % parts of
// segment b / parts (kSegPart values, the last part shorter).
constexpr uint64_t kSegPart = 8192;

__global__ void __launch_bounds__(256)
k_segment_parts(const double* __restrict__ in, uint64_t len, uint64_t parts, double* __restrict__ tmp)
{
    __shared__ double red[32];
    const uint64_t seg = blockIdx.x / parts, part = blockIdx.x % parts;
    const uint64_t p0 = part * kSegPart;
    const uint64_t n = len - p0 < kSegPart ? len - p0 : kSegPart;
    const double* src = in + seg * len + p0;
    double acc = 0.0;
    for (uint64_t j = threadIdx.x; j < n; j += blockDim.x) acc += src[j];
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) tmp[blockIdx.x] = s;
}

// ------------------------------------------------------------- scans

constexpr int kScanThreads = 512;
constexpr int kScanPerThread = 4;
constexpr uint64_t kScanTile = kScanThreads * kScanPerThread;

// Exclusive scan of one tile in place (offset added); tile_total optional.
__device__ void tile_scan(double* data, uint64_t n, uint64_t t0, double offset, double* tile_total)
{
    __shared__ double wsum[kScanThreads / 32];
    double v[kScanPerThread];
    double local = 0.0;
    const uint64_t base = t0 + uint64_t(threadIdx.x) * kScanPerThread;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) {
        v[k] = base + k < n ? data[base + k] : 0.0;
        local += v[k];
    }
    // warp inclusive scan of thread totals
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    double incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += y;
    }
    if (l == 31) wsum[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        double run = 0.0;
        for (int k = 0; k < kScanThreads / 32; ++k) {
            const double t = wsum[k];
            wsum[k] = run;
            run += t;
        }
        if (tile_total) *tile_total = run;
    }
    __syncthreads();
    double run = offset + wsum[w] + (incl - local);
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kScanThreads)
k_tile_sums(const double* __restrict__ data, uint64_t n, double* sums)
{
    __shared__ double red[32];
    const uint64_t t0 = uint64_t(blockIdx.x) * kScanTile;
    double acc = 0.0;
    for (uint64_t j = threadIdx.x; j < kScanTile; j += blockDim.x)
        if (t0 + j < n) acc += data[t0 + j];
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_single(double* data, uint64_t n, double* total_out)
{
    __shared__ double tot;
    tile_scan(data, n, 0, 0.0, &tot);
    if (threadIdx.x == 0 && total_out) *total_out = tot;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_tiles(double* data, uint64_t n, const double* offsets)
{
    const uint64_t t0 = uint64_t(blockIdx.x) * kScanTile;
    tile_scan(data, n, t0, offsets[blockIdx.x], nullptr);
}

// ------------------------------------------------- sorted uniforms

__global__ void k_exp_spacings(uint64_t seed, uint64_t counter0, uint64_t n, double* e, double* copy)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const double v = -log1p(-stream_uniform(seed, counter0 + k));
        e[k] = v;
        copy[k] = v;
    }
}

__global__ void k_normalise_spacings(const double* excl, const double* e, const double* total,
                                     uint64_t m, double* out)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const double t = *total;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < m; j += stride)
        out[j] = (excl[j] + e[j]) / t;
}

// ----------------------------------------------------------- sampling
//
// Outcome probabilities are summed hierarchically, with the same arithmetic
// in the reduction and in the search so the two agree: p_i = |a_i|^2 in the
// state's precision, groups of 8 consecutive p_i summed sequentially in that
// precision, chunks of 32 groups (256 amplitudes) summed in FP64, and the
// FP64 exclusive prefix over chunks.  A shot finds its chunk by a 32-ary warp
// search on that prefix, its group by an FP64 warp scan of the chunk's 32
// group sums, and its amplitude by a sequential scan of the group.

// One warp per chunk of `chunk` (<= 256) amplitudes.
template <typename T>
__global__ void __launch_bounds__(256)
k_chunk_sums_dense(const T* __restrict__ a, uint64_t nchunks, uint64_t chunk, double* out)
{
    using R = typename ProbT<T>::R;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t c = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += warps) {
        R p[8];
        group_probs(a, c * chunk, chunk, lane, p);
        const double s = chunk_total(group_sum(p), lane);
        if (lane == 0) out[c] = s;
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_sample(SampleArgs s)
{
    // one warp per shot, warps looping over the shots (a few blocks per SM
    // rather than one short-lived block per eight shots)
    const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t r = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < s.nruns; r += nwarps) {
        uint64_t idx;
        if (sample_one((const T*)s.amps, s.chunk, s.excl, s.nchunks, *s.total, s.u[r], threadIdx.x & 31, &idx)) {
            s.outcome[r] = idx;
            s.word[r] = outcome_word(idx, s.nbits, s.d_cbit_of_pos);
        }
    }
}

// The chunk of every shot of a column: the largest c with excl[c] <=
// target(u[r]), for sorted u, found by one merge of the targets with the
// chunk prefix (excl first on ties).  The merge is cut into spans of
// kMergeSpan steps (merge path): thread t finds where its span starts by a
// binary search on its diagonal and walks it, so that every thread does the
// same work whatever the distribution of the shots over the chunks.
constexpr uint64_t kMergeSpan = 32;

__global__ void k_locate_chunks(const double* __restrict__ excl, uint64_t nchunks, const double* __restrict__ u,
                                const double* total_p, uint64_t nruns, uint32_t* __restrict__ chunk_of)
{
    const uint64_t d0 = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kMergeSpan;
    const uint64_t len = nchunks + nruns;
    if (d0 >= len) return;
    const double total = *total_p;
    // largest i in [max(0, d0 - nruns), min(d0, nchunks)] whose first i
    // prefixes all precede the first d0 - i targets
    uint64_t lo = d0 > nruns ? d0 - nruns : 0, hi = d0 < nchunks ? d0 : nchunks;
    while (lo < hi) {
        const uint64_t i = (lo + hi + 1) >> 1;     // candidate: excl[i-1] precedes target[d0-i]
        const uint64_t j = d0 - i;
        if (j >= nruns || excl[i - 1] <= shot_target(u[j], total)) lo = i;
        else hi = i - 1;
    }
    uint64_t i = lo, j = d0 - lo;
    const uint64_t end = d0 + kMergeSpan < len ? d0 + kMergeSpan : len;
    double tj = j < nruns ? shot_target(u[j], total) : 0.0;
    for (uint64_t d = d0; d < end; ++d) {
        if (j < nruns && (i >= nchunks || excl[i] > tj)) {
            chunk_of[j] = (uint32_t)(i - 1);   // excl[0] = 0 precedes every target
            ++j;
            if (j < nruns) tj = shot_target(u[j], total);
        } else {
            ++i;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_sample_located(SampleArgs s, const uint32_t* __restrict__ chunk_of)
{
    const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    const double total = *s.total;
    for (uint64_t r = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < s.nruns; r += nwarps) {
        uint64_t idx;
        const double target = shot_target(s.u[r], total);
        if (sample_in_chunk((const T*)s.amps, s.chunk, s.excl, chunk_of[r], target, threadIdx.x & 31, &idx)) {
            s.outcome[r] = idx;
            s.word[r] = outcome_word(idx, s.nbits, s.d_cbit_of_pos);
        }
    }
}

// Per-block FP64 partials for comparing two states a, b of n amplitudes:
// [sum|a|^2, sum|b|^2, Re<a|b>, Im<a|b>, sum|wa|a|^2 - wb|b|^2|, max|a-b|]
// (wa, wb: 1/norms for the total variation of the outcome distributions).
template <typename TA, typename TB>
__global__ void __launch_bounds__(256)
k_compare(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t n, double wa, double wb, double* part)
{
    __shared__ double red[32];
    double s[6] = {0, 0, 0, 0, 0, 0};
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double ar = a[i].x, ai = a[i].y, br = b[i].x, bi = b[i].y;
        const double pa = ar * ar + ai * ai, pb = br * br + bi * bi;
        s[0] += pa;
        s[1] += pb;
        s[2] += ar * br + ai * bi;
        s[3] += ar * bi - ai * br;
        s[4] += fabs(pa * wa - pb * wb);
        const double dr = ar - br, di = ai - bi;
        s[5] = fmax(s[5], sqrt(dr * dr + di * di));
    }
    for (int k = 0; k < 5; ++k) {
        const double t = block_sum(s[k], red);
        if (threadIdx.x == 0) part[uint64_t(blockIdx.x) * 6 + k] = t;
    }
    double m = s[5];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mm = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) mm = fmax(mm, red[k]);
        part[uint64_t(blockIdx.x) * 6 + 5] = mm;
    }
}

// Column c times scales[c]; col_len is a power of two (shift, no division),
// and complex64 columns are scaled in FP32 with 16-byte accesses.
__global__ void k_scale_columns_c64(float4* a, uint64_t n4, int col_shift4, const double* scales)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float f = (float)scales[i >> col_shift4];
        float4 v = a[i];
        v.x *= f;
        v.y *= f;
        v.z *= f;
        v.w *= f;
        a[i] = v;
    }
}

__global__ void k_scale_columns_c128(double2* a, uint64_t n, int col_shift, const double* scales)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double f = scales[i >> col_shift];
        double2 v = a[i];
        v.x *= f;
        v.y *= f;
        a[i] = v;
    }
}

inline unsigned cap_grid(uint64_t g)
{
    if (g == 0) return 1;
    return g > 152ull * 128 ? 152u * 128 : (unsigned)g;
}

}  // namespace

cudaError_t launch_chunk_sums(const void* amps, int prec, uint64_t units, uint64_t chunk,
                              const IndexMap& map, double* out, cudaStream_t st)
{
    const uint64_t nchunks = units / chunk;
    const unsigned grid = cap_grid(nchunks);
    if (prec == kC128)
        k_chunk_sums<double2><<<grid, 256, 0, st>>>((const double2*)amps, units, chunk, map, out);
    else
        k_chunk_sums<float2><<<grid, 256, 0, st>>>((const float2*)amps, units, chunk, map, out);
    return cudaGetLastError();
}

cudaError_t launch_chunk_sums_dense(const void* amps, int prec, uint64_t total, uint64_t chunk, double* out,
                                    cudaStream_t st)
{
    const uint64_t nchunks = total / chunk;
    const unsigned grid = cap_grid((nchunks * 32 + 255) / 256);
    if (prec == kC128)
        k_chunk_sums_dense<double2><<<grid, 256, 0, st>>>((const double2*)amps, nchunks, chunk, out);
    else
        k_chunk_sums_dense<float2><<<grid, 256, 0, st>>>((const float2*)amps, nchunks, chunk, out);
    return cudaGetLastError();
}

uint64_t segment_sums_tmp_doubles(uint64_t nseg, uint64_t len)
{
    return len > kSegPart ? nseg * ((len + kSegPart - 1) / kSegPart) : 0;
}

cudaError_t launch_segment_sums(const double* in, uint64_t nseg, uint64_t len, double* out, double* tmp,
                                cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    if (len <= kSegPart) {
        k_segment_sums<<<(unsigned)nseg, 256, 0, st>>>(in, len, out);
        return cudaGetLastError();
    }
    // two levels, each in a fixed order: parts of kSegPart values, then the
    // parts of each segment
    const uint64_t parts = (len + kSegPart - 1) / kSegPart;
    k_segment_parts<<<(unsigned)(nseg * parts), 256, 0, st>>>(in, len, parts, tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_segment_sums<<<(unsigned)nseg, 256, 0, st>>>(tmp, parts, out);
    return cudaGetLastError();
}

uint64_t scan_tmp_doubles(uint64_t n)
{
    uint64_t need = 0;
    while (n > kScanTile) {
        n = (n + kScanTile - 1) / kScanTile;
        need += n;
    }
    return need + 1;
}

cudaError_t launch_exclusive_scan(double* data, uint64_t n, double* tmp, double* total_out,
                                  cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (n <= kScanTile) {
        k_scan_single<<<1, kScanThreads, 0, st>>>(data, n, total_out);
        return cudaGetLastError();
    }
    const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, st>>>(data, n, tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = launch_exclusive_scan(tmp, tiles, tmp + tiles, total_out, st);
    if (e != cudaSuccess) return e;
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(data, n, tmp);
    return cudaGetLastError();
}

cudaError_t launch_sorted_uniforms(uint64_t seed, uint64_t counter0, uint64_t m, double* out,
                                   double* tmp, cudaStream_t st)
{
    if (m == 0) return cudaSuccess;
    const uint64_t n = m + 1;
    double* e = tmp;                 // n doubles: the spacings
    double* work = tmp + n;          // n doubles: scanned copy
    double* stmp = tmp + 2 * n;      // scan scratch, last slot = total
    const unsigned grid = cap_grid((n + 255) / 256);
    k_exp_spacings<<<grid, 256, 0, st>>>(seed, counter0, n, e, work);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    double* total = stmp + scan_tmp_doubles(n);
    err = launch_exclusive_scan(work, n, stmp, total, st);
    if (err != cudaSuccess) return err;
    k_normalise_spacings<<<cap_grid((m + 255) / 256), 256, 0, st>>>(work, e, total, m, out);
    return cudaGetLastError();
}

cudaError_t launch_compare(const void* a, int prec_a, const void* b, int prec_b, uint64_t n, double wa, double wb,
                           double* part, unsigned blocks, cudaStream_t st)
{
    if (prec_a == kC128 && prec_b == kC128)
        k_compare<double2, double2><<<blocks, 256, 0, st>>>((const double2*)a, (const double2*)b, n, wa, wb, part);
    else if (prec_a == kC128)
        k_compare<double2, float2><<<blocks, 256, 0, st>>>((const double2*)a, (const float2*)b, n, wa, wb, part);
    else if (prec_b == kC128)
        k_compare<float2, double2><<<blocks, 256, 0, st>>>((const float2*)a, (const double2*)b, n, wa, wb, part);
    else
        k_compare<float2, float2><<<blocks, 256, 0, st>>>((const float2*)a, (const float2*)b, n, wa, wb, part);
    return cudaGetLastError();
}

cudaError_t launch_scale_columns(void* amps, int prec, uint64_t col_len, uint64_t ncols, const double* d_scales,
                                 cudaStream_t st)
{
    int shift = 0;
    while ((uint64_t(1) << shift) < col_len) ++shift;
    if (prec == kC128) {
        const uint64_t n = col_len * ncols;
        k_scale_columns_c128<<<cap_grid((n + 255) / 256), 256, 0, st>>>((double2*)amps, n, shift, d_scales);
    } else {
        if (col_len < 2) return cudaErrorInvalidValue;   // pairs of amplitudes per float4
        const uint64_t n4 = col_len * ncols / 2;
        k_scale_columns_c64<<<cap_grid((n4 + 255) / 256), 256, 0, st>>>((float4*)amps, n4, shift - 1, d_scales);
    }
    return cudaGetLastError();
}

cudaError_t launch_sample(const SampleArgs& a, cudaStream_t st)
{
    if (a.nruns == 0) return cudaSuccess;
    // 8 warps per block, 8 blocks per SM (64 warps): every SM full, each
    // warp taking every nwarps-th shot
    const uint64_t blocks = (a.nruns + 7) / 8;
    const unsigned grid = (unsigned)std::min<uint64_t>(blocks, 152ull * 8);
    if (a.chunk_of && a.nchunks < (uint64_t(1) << 32)) {
        const uint64_t spans = (a.nchunks + a.nruns + kMergeSpan - 1) / kMergeSpan;
        k_locate_chunks<<<(unsigned)((spans + 255) / 256), 256, 0, st>>>(a.excl, a.nchunks, a.u, a.total, a.nruns,
                                                                          a.chunk_of);
        if (a.prec == kC128)
            k_sample_located<double2><<<grid, 256, 0, st>>>(a, a.chunk_of);
        else
            k_sample_located<float2><<<grid, 256, 0, st>>>(a, a.chunk_of);
        return cudaGetLastError();
    }
    if (a.prec == kC128)
        k_sample<double2><<<grid, 256, 0, st>>>(a);
    else
        k_sample<float2><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace q1g
