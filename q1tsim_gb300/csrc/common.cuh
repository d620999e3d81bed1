// Shared device/host helpers of the q1tsim GB300 statevector engine.
//
// Amplitude index convention (src/gates.rs:133-141, src/vectorstate.rs:249-250):
// qubit q of an n-qubit state is bit position n-1-q of the row index, so
// qubit 0 is the most significant bit.  Kernels work on bit POSITIONS.
//
// Device layout: a state with ncols columns (src/vectorstate.rs:24-35) holds
// column c at amps[c * 2^n .. (c+1) * 2^n), i.e. column-contiguous, so the
// column is just the bits above n of a flat index and every gate kernel runs
// over all columns in one launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace q1g {

// Largest number of bit positions an index map can clear (gate qubits).
constexpr int kMaxMapBits = 12;

// Maps a dense counter j onto an amplitude index by inserting zero bits at
// the (ascending) positions zpos[] and then OR-ing setmask.  Enumerating j
// over [0, total >> nz) visits every index whose gate bits are zero exactly
// once; setmask selects the control=1 / target basis state to touch.
struct IndexMap {
    int nz;
    int zpos[kMaxMapBits];
    uint64_t setmask;
};

// Fully unrolled over kMaxMapBits with a predicate, so every zpos[] access
// has a constant index and the map stays in the kernel-parameter bank
// instead of being copied to local memory.
__host__ __device__ __forceinline__ uint64_t expand_index(uint64_t j, const IndexMap& m)
{
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int q = 0; q < kMaxMapBits; ++q) {
        if (q < m.nz) {
            const int p = m.zpos[q];
            const uint64_t low = j & ((uint64_t(1) << p) - 1);
            j = ((j >> p) << (p + 1)) | low;
        }
    }
    return j | m.setmask;
}

// expand_index for a map of exactly NZ zero positions, unrolled without
// predicates (NZ = 0: any count up to kMaxMapBits, as expand_index).  A
// predicated iteration still issues, so small maps use the exact form.
template <int NZ>
__host__ __device__ __forceinline__ uint64_t expand_nz(uint64_t j, const IndexMap& m)
{
    if constexpr (NZ == 0) {
        return expand_index(j, m);
    } else {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
        for (int q = 0; q < NZ; ++q) {
            const int p = m.zpos[q];
            const uint64_t low = j & ((uint64_t(1) << p) - 1);
            j = ((j >> p) << (p + 1)) | low;
        }
        return j | m.setmask;
    }
}

template <typename R> struct Cplx;
template <> struct Cplx<double> { using T = double2; };
template <> struct Cplx<float> { using T = float2; };

template <typename T> __host__ __device__ __forceinline__ T cmake(double re, double im);
template <> __host__ __device__ __forceinline__ double2 cmake<double2>(double re, double im) { return make_double2(re, im); }
template <> __host__ __device__ __forceinline__ float2 cmake<float2>(double re, double im) { return make_float2(float(re), float(im)); }

// a*x + b*y with complex a, b, x, y (FMA-contracted in R).
template <typename T>
__device__ __forceinline__ T cmuladd2(T a, T x, T b, T y)
{
    T r;
    r.x = a.x * x.x - a.y * x.y + b.x * y.x - b.y * y.y;
    r.y = a.x * x.y + a.y * x.x + b.x * y.y + b.y * y.x;
    return r;
}

template <typename T>
__device__ __forceinline__ T cmul(T a, T x)
{
    T r;
    r.x = a.x * x.x - a.y * x.y;
    r.y = a.x * x.y + a.y * x.x;
    return r;
}

// Host-side error string of the current thread (the C-ABI's q1g_last_error).
void set_last_error(const std::string& msg);

}  // namespace q1g
