// Plain gate-application kernels (one gate per HBM pass).
//
// These replace Gate::apply_mat_slice / apply_gate_mat_slice
// (src/gates.rs:121-152, 210-326) and the specialised overrides of
// src/gates/*.rs.  The host classifies each gate matrix (gate_plan.cpp) into
//   PAIR  - a 2x2 update of the amplitude pair (i|o0, i|o1), which covers
//           every dense 1-qubit gate, every controlled 1-qubit gate (controls
//           folded into the index map) and Swap;
//   PHASE - a diagonal phase on one basis state of the gate qubits (Z, S, T,
//           U1, CZ, CU1, CCZ ...), touching only the amplitudes it changes;
//   DENSE - a dense 2^t x 2^t update on t <= 5 target qubits (Kron, Composite,
//           fused blocks), controls again folded into the index map.
// All are streaming kernels: each thread owns U independent units whose
// loads are issued before any store, consecutive threads own consecutive
// units (coalesced), and complex64 states use 16-byte vector accesses.
#include "common.cuh"
#include "kernels.h"

namespace q1g {

namespace {

constexpr int kThreads = 256;

template <typename T>
struct Mat2 {
    T m00, m01, m10, m11;
};

template <typename T>
__host__ Mat2<T> make_mat2(const double* m)
{
    Mat2<T> r;
    r.m00 = cmake<T>(m[0], m[1]);
    r.m01 = cmake<T>(m[2], m[3]);
    r.m10 = cmake<T>(m[4], m[5]);
    r.m11 = cmake<T>(m[6], m[7]);
    return r;
}

// ---------------------------------------------------------------- PAIR

// Scalar form: one pair per unit (complex128, or complex64 when the pair
// members are not 16-byte neighbours).
template <typename T, int U>
__global__ void __launch_bounds__(kThreads)
k_pair(T* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, Mat2<T> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x0[U], x1[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_index(u, map) : ~uint64_t(0);
        if (u < units) {
            x0[k] = a[idx[k] | o0];
            x1[k] = a[idx[k] | o1];
        }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] != ~uint64_t(0)) {
            a[idx[k] | o0] = cmuladd2(m.m00, x0[k], m.m01, x1[k]);
            a[idx[k] | o1] = cmuladd2(m.m10, x0[k], m.m11, x1[k]);
        }
    }
}

// complex64, no gate bit at position 0: unit = two neighbouring pairs, so
// both members are loaded as float4 (two amplitudes each).
template <int U>
__global__ void __launch_bounds__(kThreads)
k_pair_vec2(float2* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, Mat2<float2> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x0[U], x1[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_index(u * 2, map) : ~uint64_t(0);
        if (u < units) {
            x0[k] = *reinterpret_cast<const float4*>(a + (idx[k] | o0));
            x1[k] = *reinterpret_cast<const float4*>(a + (idx[k] | o1));
        }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] != ~uint64_t(0)) {
            float2 p0 = make_float2(x0[k].x, x0[k].y), q0 = make_float2(x0[k].z, x0[k].w);
            float2 p1 = make_float2(x1[k].x, x1[k].y), q1 = make_float2(x1[k].z, x1[k].w);
            float2 r0 = cmuladd2(m.m00, p0, m.m01, p1), s0 = cmuladd2(m.m00, q0, m.m01, q1);
            float2 r1 = cmuladd2(m.m10, p0, m.m11, p1), s1 = cmuladd2(m.m10, q0, m.m11, q1);
            *reinterpret_cast<float4*>(a + (idx[k] | o0)) = make_float4(r0.x, r0.y, s0.x, s0.y);
            *reinterpret_cast<float4*>(a + (idx[k] | o1)) = make_float4(r1.x, r1.y, s1.x, s1.y);
        }
    }
}

// complex64, pair members are the neighbours (i, i+1): one float4 per unit.
template <int U>
__global__ void __launch_bounds__(kThreads)
k_pair_adj(float2* __restrict__ a, uint64_t units, IndexMap map, Mat2<float2> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_index(u, map) : ~uint64_t(0);
        if (u < units) x[k] = *reinterpret_cast<const float4*>(a + idx[k]);
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] != ~uint64_t(0)) {
            float2 p = make_float2(x[k].x, x[k].y), q = make_float2(x[k].z, x[k].w);
            float2 r = cmuladd2(m.m00, p, m.m01, q), s = cmuladd2(m.m10, p, m.m11, q);
            *reinterpret_cast<float4*>(a + idx[k]) = make_float4(r.x, r.y, s.x, s.y);
        }
    }
}

// --------------------------------------------------------------- PHASE

template <typename T, int U>
__global__ void __launch_bounds__(kThreads)
k_phase(T* __restrict__ a, uint64_t units, IndexMap map, T ph)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_index(u, map) : ~uint64_t(0);
        if (u < units) x[k] = a[idx[k]];
    }
#pragma unroll
    for (int k = 0; k < U; ++k)
        if (idx[k] != ~uint64_t(0)) a[idx[k]] = cmul(ph, x[k]);
}

template <int U>
__global__ void __launch_bounds__(kThreads)
k_phase_vec2(float2* __restrict__ a, uint64_t units, IndexMap map, float2 ph)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_index(u * 2, map) : ~uint64_t(0);
        if (u < units) x[k] = *reinterpret_cast<const float4*>(a + idx[k]);
    }
#pragma unroll
    for (int k = 0; k < U; ++k)
        if (idx[k] != ~uint64_t(0)) {
            float2 p = cmul(ph, make_float2(x[k].x, x[k].y));
            float2 q = cmul(ph, make_float2(x[k].z, x[k].w));
            *reinterpret_cast<float4*>(a + idx[k]) = make_float4(p.x, p.y, q.x, q.y);
        }
}

// --------------------------------------------------------------- DENSE

// One thread per group of 2^TB amplitudes at i | off[s]; the matrix sits in
// shared memory (row-major, complex R).
template <typename T, int TB>
__global__ void __launch_bounds__(128)
k_dense(T* __restrict__ a, uint64_t units, IndexMap map, DenseOffsets offs, const T* __restrict__ gmat)
{
    constexpr int D = 1 << TB;
    __shared__ T mat[D * D];
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) mat[e] = gmat[e];
    __syncthreads();
    const uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (u >= units) return;
    const uint64_t i = expand_index(u, map);
    T x[D];
#pragma unroll
    for (int s = 0; s < D; ++s) x[s] = a[i | offs.off[s]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        T acc = cmul(mat[r * D], x[0]);
#pragma unroll
        for (int s = 1; s < D; ++s) {
            const T mm = mat[r * D + s];
            acc.x += mm.x * x[s].x - mm.y * x[s].y;
            acc.y += mm.x * x[s].y + mm.y * x[s].x;
        }
        a[i | offs.off[r]] = acc;
    }
}

constexpr int kUnroll = 4;

inline unsigned grid_for(uint64_t units, int per_block)
{
    uint64_t g = (units + per_block - 1) / per_block;
    return (unsigned)(g ? g : 1);
}

}  // namespace

cudaError_t launch_pair(void* amps, int prec, uint64_t total, const IndexMap& map,
                        uint64_t o0, uint64_t o1, const double* m, cudaStream_t st)
{
    const uint64_t pairs = total >> map.nz;
    if (pairs == 0) return cudaSuccess;
    if (prec == kC128) {
        auto mm = make_mat2<double2>(m);
        k_pair<double2, kUnroll><<<grid_for(pairs, kThreads * kUnroll), kThreads, 0, st>>>(
            (double2*)amps, pairs, map, o0, o1, mm);
    } else {
        auto mm = make_mat2<float2>(m);
        const bool pos0_free = map.nz == 0 || map.zpos[0] > 0;
        if (pos0_free && (map.setmask & 1) == 0 && ((o0 | o1) & 1) == 0 && pairs >= 2) {
            const uint64_t units = pairs / 2;
            k_pair_vec2<kUnroll><<<grid_for(units, kThreads * kUnroll), kThreads, 0, st>>>(
                (float2*)amps, units, map, o0, o1, mm);
        } else if (o0 == 0 && o1 == 1 && (map.setmask & 1) == 0) {
            k_pair_adj<kUnroll><<<grid_for(pairs, kThreads * kUnroll), kThreads, 0, st>>>(
                (float2*)amps, pairs, map, mm);
        } else {
            k_pair<float2, kUnroll><<<grid_for(pairs, kThreads * kUnroll), kThreads, 0, st>>>(
                (float2*)amps, pairs, map, o0, o1, mm);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_phase(void* amps, int prec, uint64_t total, const IndexMap& map,
                         double ph_re, double ph_im, cudaStream_t st)
{
    const uint64_t units = total >> map.nz;
    if (units == 0) return cudaSuccess;
    if (prec == kC128) {
        k_phase<double2, kUnroll><<<grid_for(units, kThreads * kUnroll), kThreads, 0, st>>>(
            (double2*)amps, units, map, make_double2(ph_re, ph_im));
    } else {
        const bool pos0_free = map.nz == 0 || map.zpos[0] > 0;
        if (pos0_free && (map.setmask & 1) == 0 && units >= 2) {
            k_phase_vec2<kUnroll><<<grid_for(units / 2, kThreads * kUnroll), kThreads, 0, st>>>(
                (float2*)amps, units / 2, map, make_float2((float)ph_re, (float)ph_im));
        } else {
            k_phase<float2, kUnroll><<<grid_for(units, kThreads * kUnroll), kThreads, 0, st>>>(
                (float2*)amps, units, map, make_float2((float)ph_re, (float)ph_im));
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_dense(void* amps, int prec, uint64_t total, const IndexMap& map,
                         const DenseOffsets& offs, int tb, const void* dmat, cudaStream_t st)
{
    const uint64_t units = total >> map.nz;
    if (units == 0) return cudaSuccess;
    const unsigned grid = grid_for(units, 128);
#define Q1G_DENSE_CASE(TBV)                                                                  \
    case TBV:                                                                                \
        if (prec == kC128)                                                                   \
            k_dense<double2, TBV><<<grid, 128, 0, st>>>((double2*)amps, units, map, offs,    \
                                                        (const double2*)dmat);               \
        else                                                                                 \
            k_dense<float2, TBV><<<grid, 128, 0, st>>>((float2*)amps, units, map, offs,      \
                                                       (const float2*)dmat);                 \
        break;
    switch (tb) {
        Q1G_DENSE_CASE(1)
        Q1G_DENSE_CASE(2)
        Q1G_DENSE_CASE(3)
        Q1G_DENSE_CASE(4)
        Q1G_DENSE_CASE(5)
        default:
            return cudaErrorInvalidValue;
    }
#undef Q1G_DENSE_CASE
    return cudaGetLastError();
}

}  // namespace q1g
