// State construction, precision conversion and measurement collapse kernels.
#include "common.cuh"
#include "kernels.h"
#include "sampling.cuh"

namespace q1g {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(uint64_t n, int per_block)
{
    uint64_t g = (n + per_block - 1) / per_block;
    if (g > 0x7fffffffULL) g = 0x7fffffffULL;
    return (unsigned)(g ? g : 1);
}

template <typename T>
__global__ void k_set_basis(T* a, const uint64_t* col_index, uint64_t ncols, uint64_t col_len)
{
    uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < ncols) a[c * col_len + col_index[c]] = cmake<T>(1.0, 0.0);
}

// amp(i) = c_0[b_0] * c_1[b_1] * ... multiplied left to right, b_q the bit of
// qubit q (position n-1-q) -- the kron chain of src/vectorstate.rs:68-74.
template <typename T>
__global__ void k_product_state(T* a, int nbits, const double* coefs)
{
    const uint64_t n = uint64_t(1) << nbits;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double re = 1.0, im = 0.0;
        for (int q = 0; q < nbits; ++q) {
            const int b = (i >> (nbits - 1 - q)) & 1;
            const double cr = coefs[4 * q + 2 * b], ci = coefs[4 * q + 2 * b + 1];
            const double nr = cr * re - ci * im;
            const double ni = cr * im + ci * re;
            re = nr;
            im = ni;
        }
        a[i] = cmake<T>(re, im);
    }
}

// Amplitude i gets re, im i.i.d. N(0,1) by the Box-Muller transform of
// uniforms 2i and 2i+1 of the SplitMix64 stream `seed`:
// r = sqrt(-2 ln(1 - u1)), (re, im) = r (cos 2 pi u2, sin 2 pi u2).
// complex128 in FP64, complex64 in FP32 (1 - u1 formed in FP64 first, so it
// is never 0).
__global__ void k_random_normal_c128(double2* a, uint64_t total, uint64_t seed)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += stride) {
        const double u1 = stream_uniform(seed, 2 * i), u2 = stream_uniform(seed, 2 * i + 1);
        const double r = sqrt(-2.0 * log1p(-u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        a[i] = make_double2(r * cs, r * sn);
    }
}

__global__ void k_random_normal_c64(float2* a, uint64_t total, uint64_t seed)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += stride) {
        const double u1 = stream_uniform(seed, 2 * i), u2 = stream_uniform(seed, 2 * i + 1);
        const float r = sqrtf(-2.0f * logf((float)(1.0 - u1)));
        float sn, cs;
        sincospif(2.0f * (float)u2, &sn, &cs);
        a[i] = make_float2(r * cs, r * sn);
    }
}

__global__ void k_c128_to_c64(float2* dst, const double2* src, uint64_t n)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 v = src[i];
        dst[i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_c64_to_c128(double2* dst, const float2* src, uint64_t n)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        float2 v = src[i];
        dst[i] = make_double2(v.x, v.y);
    }
}

template <typename T, typename R>
__global__ void k_collapse_copy(T* dst, const T* src, uint64_t col_len,
                                int pos, const CollapseCol* __restrict__ cols, uint64_t ncols)
{
    const uint64_t total = col_len * ncols;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < total; g += stride) {
        const uint64_t j = g / col_len;
        const uint64_t i = g - j * col_len;
        const CollapseCol c = cols[j];
        T v = src[c.src_col * col_len + i];
        if (c.keep >= 0) {
            if ((int)((i >> pos) & 1) != c.keep) {
                v.x = R(0);
                v.y = R(0);
            } else {
                v.x = v.x * R(c.scale);
                v.y = v.y * R(c.scale);
            }
        }
        dst[g] = v;
    }
}

// full[deposit(c) | fixed] = compact[c]: bit k of c goes to position pos[k]
template <typename T>
__global__ void k_scatter_subspace(T* full, const T* compact, uint64_t count, SubspacePositions sp, uint64_t fixed)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < count; c += stride) {
        uint64_t idx = fixed;
#pragma unroll 8
        for (int k = 0; k < sp.n; ++k)
            if ((c >> k) & 1) idx |= uint64_t(1) << sp.pos[k];
        full[idx] = compact[c];
    }
}

// Every amplitude of the full state in one coalesced pass: full[i] is
// compact[i with the excluded positions removed] where i's excluded bits
// equal `fixed`, zero elsewhere.  ex holds the excluded positions, highest
// first, so that removing one leaves the lower ones in place.
struct Excluded {
    int n;
    int pos[kFillMaxExcluded];
};

template <typename T>
__device__ __forceinline__ T fill_value(const T* compact, uint64_t i, uint64_t exmask, uint64_t fixed,
                                        const Excluded& ex)
{
    T v{};
    if ((i & exmask) == fixed) {
        uint64_t c = i;
#pragma unroll
        for (int k = 0; k < kFillMaxExcluded; ++k)
            if (k < ex.n) {
                const int p = ex.pos[k];
                c = ((c >> (p + 1)) << p) | (c & ((uint64_t(1) << p) - 1));
            }
        v = compact[c];
    }
    return v;
}

// One 16-byte unit per thread and iteration (two complex64 amplitudes or
// one complex128), so that each store instruction of a warp writes 512
// contiguous bytes (n even).
template <typename T>
__global__ void k_fill_subspace(T* full, const T* compact, uint64_t n, uint64_t exmask, uint64_t fixed, Excluded ex)
{
    constexpr int kPer = 16 / (int)sizeof(T);
    const uint64_t units = n / kPer;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
        const uint64_t i = u * kPer;
        if constexpr (kPer == 2) {
            const T a = fill_value(compact, i, exmask, fixed, ex);
            const T b = fill_value(compact, i + 1, exmask, fixed, ex);
            reinterpret_cast<float4*>(full)[u] = make_float4(a.x, a.y, b.x, b.y);
        } else {
            full[i] = fill_value(compact, i, exmask, fixed, ex);
        }
    }
}

}  // namespace

cudaError_t launch_scatter_subspace(void* full, const void* compact, int prec, int nbits_full, int nbits_compact,
                                   const SubspacePositions& sp, uint64_t fixed, cudaStream_t st)
{
    const uint64_t n = uint64_t(1) << nbits_full;
    const int nex = nbits_full - nbits_compact;
    if (nex >= 0 && nex <= kFillMaxExcluded && nbits_full >= 2) {
        Excluded ex{};
        uint64_t in = 0;
        for (int k = 0; k < sp.n; ++k) in |= uint64_t(1) << sp.pos[k];
        for (int p = nbits_full - 1; p >= 0; --p)
            if (!((in >> p) & 1)) ex.pos[ex.n++] = p;
        const uint64_t exmask = (n - 1) & ~in;
        const uint64_t units = prec == kC128 ? n : n / 2;
        const unsigned grid = blocks_for(units, kThreads) > 152 * 32 ? 152 * 32 : blocks_for(units, kThreads);
        if (prec == kC128)
            k_fill_subspace<double2><<<grid, kThreads, 0, st>>>((double2*)full, (const double2*)compact, n, exmask,
                                                               fixed & exmask, ex);
        else
            k_fill_subspace<float2><<<grid, kThreads, 0, st>>>((float2*)full, (const float2*)compact, n, exmask,
                                                              fixed & exmask, ex);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(full, 0, n * (prec == kC128 ? 16 : 8), st);
    if (e != cudaSuccess) return e;
    const uint64_t count = uint64_t(1) << nbits_compact;
    const unsigned grid = blocks_for(count, kThreads) > 152 * 32 ? 152 * 32 : blocks_for(count, kThreads);
    if (prec == kC128)
        k_scatter_subspace<double2><<<grid, kThreads, 0, st>>>((double2*)full, (const double2*)compact, count, sp,
                                                               fixed);
    else
        k_scatter_subspace<float2><<<grid, kThreads, 0, st>>>((float2*)full, (const float2*)compact, count, sp, fixed);
    return cudaGetLastError();
}

cudaError_t launch_fill_basis(void* amps, int prec, uint64_t n_amps, const uint64_t* d_col_index,
                              uint64_t ncols, uint64_t col_len, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(amps, 0, n_amps * amp_bytes(prec), st);
    if (e != cudaSuccess) return e;
    if (ncols == 0) return cudaSuccess;
    if (prec == kC128)
        k_set_basis<double2><<<blocks_for(ncols, kThreads), kThreads, 0, st>>>(
            (double2*)amps, d_col_index, ncols, col_len);
    else
        k_set_basis<float2><<<blocks_for(ncols, kThreads), kThreads, 0, st>>>(
            (float2*)amps, d_col_index, ncols, col_len);
    return cudaGetLastError();
}

cudaError_t launch_product_state(void* amps, int prec, int nbits, const double* d_coefs,
                                 cudaStream_t st)
{
    const uint64_t n = uint64_t(1) << nbits;
    const unsigned grid = blocks_for(n, kThreads) > 152 * 64 ? 152 * 64 : blocks_for(n, kThreads);
    if (prec == kC128)
        k_product_state<double2><<<grid, kThreads, 0, st>>>((double2*)amps, nbits, d_coefs);
    else
        k_product_state<float2><<<grid, kThreads, 0, st>>>((float2*)amps, nbits, d_coefs);
    return cudaGetLastError();
}

cudaError_t launch_random_normal(void* amps, int prec, uint64_t total, uint64_t seed, cudaStream_t st)
{
    const unsigned grid = blocks_for(total, kThreads) > 152 * 64 ? 152 * 64 : blocks_for(total, kThreads);
    if (prec == kC128)
        k_random_normal_c128<<<grid, kThreads, 0, st>>>((double2*)amps, total, seed);
    else
        k_random_normal_c64<<<grid, kThreads, 0, st>>>((float2*)amps, total, seed);
    return cudaGetLastError();
}

cudaError_t launch_convert_c128_to_c64(float2* dst, const double2* src, uint64_t n, cudaStream_t st)
{
    const unsigned grid = blocks_for(n, kThreads) > 152 * 64 ? 152 * 64 : blocks_for(n, kThreads);
    k_c128_to_c64<<<grid, kThreads, 0, st>>>(dst, src, n);
    return cudaGetLastError();
}

cudaError_t launch_convert_c64_to_c128(double2* dst, const float2* src, uint64_t n, cudaStream_t st)
{
    const unsigned grid = blocks_for(n, kThreads) > 152 * 64 ? 152 * 64 : blocks_for(n, kThreads);
    k_c64_to_c128<<<grid, kThreads, 0, st>>>(dst, src, n);
    return cudaGetLastError();
}

cudaError_t launch_collapse_copy(void* dst, const void* src, int prec, uint64_t col_len, int pos,
                                 const CollapseCol* d_cols, uint64_t ncols, cudaStream_t st)
{
    const uint64_t total = col_len * ncols;
    if (total == 0) return cudaSuccess;
    const unsigned grid = blocks_for(total, kThreads) > 152 * 64 ? 152 * 64 : blocks_for(total, kThreads);
    if (prec == kC128)
        k_collapse_copy<double2, double><<<grid, kThreads, 0, st>>>(
            (double2*)dst, (const double2*)src, col_len, pos, d_cols, ncols);
    else
        k_collapse_copy<float2, float><<<grid, kThreads, 0, st>>>(
            (float2*)dst, (const float2*)src, col_len, pos, d_cols, ncols);
    return cudaGetLastError();
}

}  // namespace q1g
