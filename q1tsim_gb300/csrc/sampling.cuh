// Device helpers shared by the shot samplers (measure_kernels.cu and the
// batched executor): the SplitMix64 uniform stream, |a|^2 group sums, and the
// per-shot search.
//
// Outcome probabilities are summed hierarchically, with the same arithmetic
// in the reduction and in the search so the two agree: p_i = |a_i|^2 in the
// state's precision, groups of 8 consecutive p_i summed sequentially in that
// precision, chunks of 32 groups (256 amplitudes) summed in the state's
// precision too (FP64 for complex128), and an FP64 exclusive prefix over
// chunks.  A shot finds its chunk by a 32-ary warp
// search on that prefix, its group by an FP64 warp scan of the chunk's 32
// group sums, and its amplitude by a sequential scan of the group.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace q1g {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// SplitMix64 (Steele, Lea & Flood 2014): draw k of stream `seed` is
// mix(seed + (k+1) * golden_gamma) as a 53-bit uniform in [0, 1).
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

template <typename T> struct ProbT;
template <> struct ProbT<float2> { using R = float; };
template <> struct ProbT<double2> { using R = double; };

__device__ __forceinline__ float psq(float2 v) { return __fmaf_rn(v.x, v.x, __fmul_rn(v.y, v.y)); }
__device__ __forceinline__ double psq(double2 v) { return __fma_rn(v.x, v.x, __dmul_rn(v.y, v.y)); }
__device__ __forceinline__ float padd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double padd(double a, double b) { return __dadd_rn(a, b); }

// p of the 8 amplitudes [8*lane, 8*lane+8) of the chunk at i0.
__device__ __forceinline__ void group_probs(const float2* a, uint64_t i0, uint64_t chunk, int lane, float p[8])
{
    const uint64_t g0 = (uint64_t)lane * 8;
    if (chunk >= 256) {
        const float4* v = reinterpret_cast<const float4*>(a + i0 + g0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 w = v[q];
            p[2 * q] = psq(make_float2(w.x, w.y));
            p[2 * q + 1] = psq(make_float2(w.z, w.w));
        }
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) p[e] = g0 + e < chunk ? psq(a[i0 + g0 + e]) : 0.0f;
    }
}

__device__ __forceinline__ void group_probs(const double2* a, uint64_t i0, uint64_t chunk, int lane, double p[8])
{
    const uint64_t g0 = (uint64_t)lane * 8;
#pragma unroll
    for (int e = 0; e < 8; ++e) p[e] = g0 + e < chunk ? psq(a[i0 + g0 + e]) : 0.0;
}

template <typename R>
__device__ __forceinline__ R group_sum(const R p[8])
{
    R s = p[0];
#pragma unroll
    for (int e = 1; e < 8; ++e) s = padd(s, p[e]);
    return s;
}

// Inclusive prefix of v over the warp's lanes, in v's precision: the order
// in which the sampler adds a chunk's 32 group sums.
template <typename R>
__device__ __forceinline__ R warp_incl_scan(R v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const R y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// A chunk's total from its lanes' group sums (all lanes get it).
// complex64: in FP32, in the sampler's scan order, so that the total is the
// value the sampler's scan reaches at lane 31 (an FP64 warp reduction costs
// 16 cycles of an SM's FP64 pipe per instruction; a chunk holds about 2^-22
// of the mass at 30 qubits, so FP32 leaves it good to about 1e-14).
// complex128: in FP64.
__device__ __forceinline__ double chunk_total(float gs, int lane)
{
    return (double)__shfl_sync(0xffffffffu, warp_incl_scan(gs, lane), 31);
}
__device__ __forceinline__ double chunk_total(double gs, int) { return warp_sum(gs); }

// Chunk sum of one warp's chunk (all lanes get it).
template <typename T>
__device__ __forceinline__ double chunk_sum(const T* a, uint64_t i0, uint64_t chunk, int lane)
{
    typename ProbT<T>::R p[8];
    group_probs(a, i0, chunk, lane, p);
    return chunk_total(group_sum(p), lane);
}

// One shot, executed by a whole warp: the basis index whose inclusive
// probability prefix first exceeds u * total.  Returns true on the lane that
// holds the result in *idx.
// The shot's target u * total, kept strictly inside the mass if rounding
// pushed it onto the total (u < 1): the shot then lands on the last nonzero
// amplitude.
__device__ __forceinline__ double shot_target(double u, double total)
{
    const double target = u * total;
    return target < total ? target : nextafter(total, 0.0);
}

// One shot whose chunk lo is known (the largest chunk c with excl[c] <=
// target), executed by a whole warp.  Returns true on the lane that holds
// the result in *idx.
template <typename T>
__device__ bool sample_in_chunk(const T* a, uint64_t chunk, const double* excl, uint64_t lo, double target,
                                int lane, uint64_t* idx);

template <typename T>
__device__ bool sample_one(const T* a, uint64_t chunk, const double* excl, uint64_t nchunks, double total,
                           double u, int lane, uint64_t* idx)
{
    const double target = shot_target(u, total);
    // Largest chunk c with excl[c] <= target (excl is non-decreasing and
    // excl[0] = 0).  The warp searches 32-ary: lane j probes lo + j * step,
    // and the last lane whose prefix is <= target narrows [lo, hi) to one
    // step: 5 dependent rounds over 2^22 chunks instead of 22 for a binary
    // search.
    uint64_t lo = 0, hi = nchunks;
    while (hi - lo > 1) {
        const uint64_t step = (hi - lo + 31) >> 5;
        const uint64_t pj = lo + (uint64_t)lane * step;
        const unsigned ok = __ballot_sync(0xffffffffu, pj < hi && excl[pj] <= target);
        lo += (uint64_t)(31 - __clz(ok)) * step;    // lane 0 always qualifies
        hi = min(hi, lo + step);
    }
    return sample_in_chunk(a, chunk, excl, lo, target, lane, idx);
}

template <typename T>
__device__ bool sample_in_chunk(const T* a, uint64_t chunk, const double* excl, uint64_t lo, double target,
                                int lane, uint64_t* idx)
{
    using R = typename ProbT<T>::R;
    const uint64_t i0 = lo * chunk;
    const double tl = target - excl[lo];
    R p[8];
    group_probs(a, i0, chunk, lane, p);
    // the chunk's group sums scanned in the state's precision (the chunk
    // sums add them in the same order, chunk_total)
    // and the target's offset into the chunk compared in that precision too
    // (it is at most the chunk's mass)
    const R gs = group_sum(p);
    const R incl = warp_incl_scan(gs, lane);
    const R tlr = (R)tl;
    const unsigned hit = __ballot_sync(0xffffffffu, gs > R(0) && incl > tlr);
    const unsigned nz = __ballot_sync(0xffffffffu, gs > R(0));
    int owner;
    R local;
    if (hit) {
        owner = __ffs(hit) - 1;
        local = tlr - (incl - gs);
    } else {
        owner = nz ? 31 - __clz(nz) : 0;
        local = R(INFINITY);   // past the end: take the group's last nonzero amplitude
    }
    if (lane != owner) return false;
    int e_pick = -1, e_last = 0;
    R run = R(0);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        run = padd(run, p[e]);
        if (p[e] > R(0)) {
            e_last = e;
            if (e_pick < 0 && run > local) e_pick = e;
        }
    }
    if (e_pick < 0) e_pick = e_last;
    *idx = i0 + (uint64_t)lane * 8 + (uint64_t)e_pick;
    return true;
}

// Classical word of outcome idx: bit position p of idx goes to the mask
// cbit_of_pos[p] (qubit q = position n-1-q lands on cbits[q]).
__device__ __forceinline__ uint64_t outcome_word(uint64_t idx, int nbits, const uint64_t* cbit_of_pos)
{
    uint64_t word = 0;
    for (int q = 0; q < nbits; ++q)
        if ((idx >> q) & 1) word |= cbit_of_pos[q];
    return word;
}

}  // namespace q1g
