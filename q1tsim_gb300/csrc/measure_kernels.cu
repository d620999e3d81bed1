// Measurement kernels: |amp|^2 reductions, FP64 prefix sums, sorted-uniform
// generation and binary-search shot sampling.
//
// They replace the reference's per-column `WeightedIndex::new(|a|^2)` +
// `sample_iter` (src/vectorstate.rs:119-133) and the w0 block sums of
// measure_into / peek_into (src/vectorstate.rs:252-261, 361-370).  All sums
// are FP64 with a fixed reduction order, so repeated runs give identical
// results.
#include "common.cuh"
#include "kernels.h"

namespace q1g {

namespace {

template <typename T>
__device__ __forceinline__ double norm_sqr(T v)
{
    const double x = (double)v.x, y = (double)v.y;
    return x * x + y * y;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
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

__device__ __forceinline__ uint64_t splitmix_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double stream_uniform(uint64_t seed, uint64_t counter)
{
    const uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    return (double)(splitmix_mix(z) >> 11) * (1.0 / 9007199254740992.0);
}

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

template <typename T>
__global__ void __launch_bounds__(256)
k_sample(SampleArgs s)
{
    const uint64_t r = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= s.nruns) return;
    const T* a = (const T*)s.amps;
    const double total = *s.total;
    double target = s.u[r] * total;
    // u < 1, but keep the target strictly inside the mass if rounding pushed
    // it onto the total: the sample then lands on the last nonzero amplitude.
    if (!(target < total)) target = nextafter(total, 0.0);
    // largest chunk c with excl[c] <= target
    uint64_t lo = 0, hi = s.nchunks - 1;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (s.excl[mid] <= target) lo = mid; else hi = mid - 1;
    }
    const uint64_t c = lo;
    const double tl = target - s.excl[c];
    const uint64_t i0 = c * s.chunk;
    double base = 0.0;
    int64_t found = -1, last_nz = -1;
    for (uint64_t st = 0; st < s.chunk; st += 32) {
        const uint64_t i = st + lane;
        const double w = i < s.chunk ? norm_sqr(a[i0 + i]) : 0.0;
        double incl = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        incl += base;
        const unsigned hit = __ballot_sync(0xffffffffu, w > 0.0 && incl > tl);
        const unsigned nz = __ballot_sync(0xffffffffu, w > 0.0);
        if (nz) last_nz = (int64_t)(st + 31 - __clz(nz));
        if (hit) {
            found = (int64_t)(st + __ffs(hit) - 1);
            break;
        }
        base = __shfl_sync(0xffffffffu, incl, 31);
    }
    if (found < 0) found = last_nz >= 0 ? last_nz : 0;
    if (lane == 0) {
        const uint64_t idx = i0 + (uint64_t)found;
        uint64_t word = 0;
        for (int p = 0; p < s.nbits; ++p)
            if ((idx >> p) & 1) word |= s.d_cbit_of_pos[p];
        s.outcome[r] = idx;
        s.word[r] = word;
    }
}

// Per-block FP64 partials for comparing two states a, b of n amplitudes:
// [sum|a|^2, sum|b|^2, Re<a|b>, Im<a|b>, sum||a|^2-|b|^2|, max|a-b|].
template <typename TA, typename TB>
__global__ void __launch_bounds__(256)
k_compare(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t n, double* part)
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
        s[4] += fabs(pa - pb);
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

cudaError_t launch_segment_sums(const double* in, uint64_t nseg, uint64_t len, double* out,
                                cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    k_segment_sums<<<(unsigned)nseg, 256, 0, st>>>(in, len, out);
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

cudaError_t launch_compare(const void* a, int prec_a, const void* b, int prec_b, uint64_t n,
                           double* part, unsigned blocks, cudaStream_t st)
{
    if (prec_a == kC128 && prec_b == kC128)
        k_compare<double2, double2><<<blocks, 256, 0, st>>>((const double2*)a, (const double2*)b, n, part);
    else if (prec_a == kC128)
        k_compare<double2, float2><<<blocks, 256, 0, st>>>((const double2*)a, (const float2*)b, n, part);
    else if (prec_b == kC128)
        k_compare<float2, double2><<<blocks, 256, 0, st>>>((const float2*)a, (const double2*)b, n, part);
    else
        k_compare<float2, float2><<<blocks, 256, 0, st>>>((const float2*)a, (const float2*)b, n, part);
    return cudaGetLastError();
}

cudaError_t launch_sample(const SampleArgs& a, cudaStream_t st)
{
    if (a.nruns == 0) return cudaSuccess;
    const uint64_t threads = a.nruns * 32;
    const unsigned grid = (unsigned)((threads + 255) / 256);
    if (a.prec == kC128)
        k_sample<double2><<<grid, 256, 0, st>>>(a);
    else
        k_sample<float2><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace q1g
