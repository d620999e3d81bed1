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
#include <type_traits>

#include "common.cuh"
#include "df64.cuh"
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
template <typename T, int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_pair(T* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, Mat2<T> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x0[U], x1[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
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
template <int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_pair_vec2(float2* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, Mat2<float2> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x0[U], x1[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u * 2, map) : ~uint64_t(0);
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
template <int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_pair_adj(float2* __restrict__ a, uint64_t units, IndexMap map, Mat2<float2> m)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
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

// ------------------------------------------------- exact unit shuffles
//
// A 2x2 matrix with one entry of 0, +-1 or +-i per row and column (X, Y,
// CX, CY, CCX, Swap ...) moves and re-signs amplitudes; no arithmetic.
// Unit code u: 0 -> x, 1 -> i x, 2 -> -x, 3 -> -i x.
template <typename T>
__device__ __forceinline__ T unit_times(int u, T x)
{
    switch (u) {
        case 1: return T{-x.y, x.x};
        case 2: return T{-x.x, -x.y};
        case 3: return T{x.y, -x.x};
        default: return x;
    }
}

// out0 = u0 * x[s0], out1 = u1 * x[s1] (s0 != s1)
template <typename T, int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_pair_mono(T* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, int swap, int u0, int u1)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x0[U], x1[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
        if (u < units) {
            x0[k] = a[idx[k] | o0];
            x1[k] = a[idx[k] | o1];
        }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] != ~uint64_t(0)) {
            a[idx[k] | o0] = unit_times(u0, swap ? x1[k] : x0[k]);
            a[idx[k] | o1] = unit_times(u1, swap ? x0[k] : x1[k]);
        }
    }
}

// ------------------------------------- complex128 without the FP64 pipe

// Coefficients of out_j = m_j0 x0 + m_j1 x1 for the packed dot products:
// lane 0 is Re out_j, lane 1 Im out_j, with terms
//   k=0: (m_j0r, m_j0r) * (x0r, x0i)    k=1: (m_j1r, m_j1r) * (x1r, x1i)
//   k=2: (-m_j0i, m_j0i) * (x0i, x0r)   k=3: (-m_j1i, m_j1i) * (x1i, x1r)
struct Mat2DF {
    float2 h[2][4], l[2][4];
};


// Warps 0 and 2 of each 8-warp block do their pairs in FP64.  The
// double-float path is issue-bound and leaves GB300's FP64 pipe idle; with a
// quarter of the warps on it both pipes work (0.93 against 0.82 of measured
// HBM at 28 qubits; more FP64 warps make that pipe the bottleneck).  Both
// paths are within the complex128 contract, and which pairs take which is
// fixed by the launch shape, so results are reproducible.
constexpr unsigned kPairFp64Warps = 0x05;
static_assert(kThreads == 256, "kPairFp64Warps assumes 8 warps per block");

// out0 = m00 x0 + m01 x1, out1 = m10 x0 + m11 x1 on double-float pairs; a
// unit with an amplitude outside the split's range, and every unit of the
// warps in kPairFp64Warps, is done in FP64 (md).
template <int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_pair_c128x(double2* __restrict__ a, uint64_t units, IndexMap map, uint64_t o0, uint64_t o1, Mat2DF m,
             Mat2<double2> md)
{
    const bool fp64_warp = ((kPairFp64Warps >> (threadIdx.x >> 5)) & 1u) != 0;
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    ulonglong2 x0[U], x1[U];
    uint64_t idx[U];
    ulonglong2* ab = reinterpret_cast<ulonglong2*>(a);
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
        if (u < units) {
            x0[k] = ab[idx[k] | o0];
            x1[k] = ab[idx[k] | o1];
        }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] == ~uint64_t(0)) continue;
        DF v[4];   // x0.re, x0.im, x1.re, x1.im
        bool ok;
        if (fp64_warp) {
            ok = false;
        } else if (split_fast_ok(x0[k].x) & split_fast_ok(x0[k].y) & split_fast_ok(x1[k].x) & split_fast_ok(x1[k].y)) {
            v[0] = split_fast(x0[k].x);
            v[1] = split_fast(x0[k].y);
            v[2] = split_fast(x1[k].x);
            v[3] = split_fast(x1[k].y);
            ok = true;
        } else {
            ok = split_f64(x0[k].x, v[0]) & split_f64(x0[k].y, v[1]) & split_f64(x1[k].x, v[2]) &
                 split_f64(x1[k].y, v[3]);
        }
        if (ok) {
            const float2 bh[4] = {make_float2(v[0].h, v[1].h), make_float2(v[2].h, v[3].h),
                                  make_float2(v[1].h, v[0].h), make_float2(v[3].h, v[2].h)};
            const float2 bl[4] = {make_float2(v[0].l, v[1].l), make_float2(v[2].l, v[3].l),
                                  make_float2(v[1].l, v[0].l), make_float2(v[3].l, v[2].l)};
            float2 h0, l0, h1, l1;
            dot_x2<4>(m.h[0], m.l[0], bh, bl, h0, l0);
            dot_x2<4>(m.h[1], m.l[1], bh, bl, h1, l1);
            ab[idx[k] | o0] = make_ulonglong2(join_f64(DF{h0.x, l0.x}), join_f64(DF{h0.y, l0.y}));
            ab[idx[k] | o1] = make_ulonglong2(join_f64(DF{h1.x, l1.x}), join_f64(DF{h1.y, l1.y}));
        } else {
            const double2 y0 = *reinterpret_cast<const double2*>(&x0[k]);
            const double2 y1 = *reinterpret_cast<const double2*>(&x1[k]);
            a[idx[k] | o0] = cmuladd2(md.m00, y0, md.m01, y1);
            a[idx[k] | o1] = cmuladd2(md.m10, y0, md.m11, y1);
        }
    }
}

// --------------------------------------------------------------- PHASE

template <typename T, int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_phase(T* __restrict__ a, uint64_t units, IndexMap map, T ph)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
        if (u < units) x[k] = a[idx[k]];
    }
#pragma unroll
    for (int k = 0; k < U; ++k)
        if (idx[k] != ~uint64_t(0)) a[idx[k]] = cmul(ph, x[k]);
}

template <int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_phase_vec2(float2* __restrict__ a, uint64_t units, IndexMap map, float2 ph)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    float4 x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u * 2, map) : ~uint64_t(0);
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

// x -> u x for a unit u in {1, i, -1, -i} (code as unit_times)
template <typename T, int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_phase_mono(T* __restrict__ a, uint64_t units, IndexMap map, int code)
{
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    T x[U];
    uint64_t idx[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
        if (u < units) x[k] = a[idx[k]];
    }
#pragma unroll
    for (int k = 0; k < U; ++k)
        if (idx[k] != ~uint64_t(0)) a[idx[k]] = unit_times(code, x[k]);
}

// complex128 phase on double-float pairs (FP64 for out-of-range amplitudes
// and for the warps in kPairFp64Warps: 0.84 against 0.80 of measured HBM)
template <int U, int NZ>
__global__ void __launch_bounds__(kThreads)
k_phase_c128x(double2* __restrict__ a, uint64_t units, IndexMap map, DF pr, DF pi, double2 pd)
{
    const bool fp64_warp = ((kPairFp64Warps >> (threadIdx.x >> 5)) & 1u) != 0;   // as k_pair_c128x
    uint64_t base = (uint64_t(blockIdx.x) * U) * blockDim.x + threadIdx.x;
    ulonglong2 x[U];
    uint64_t idx[U];
    ulonglong2* ab = reinterpret_cast<ulonglong2*>(a);
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const uint64_t u = base + uint64_t(k) * blockDim.x;
        idx[k] = u < units ? expand_nz<NZ>(u, map) : ~uint64_t(0);
        if (u < units) x[k] = ab[idx[k]];
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
        if (idx[k] == ~uint64_t(0)) continue;
        DF v[2];
        bool ok;
        if (fp64_warp) {
            ok = false;
        } else if (split_fast_ok(x[k].x) & split_fast_ok(x[k].y)) {
            v[0] = split_fast(x[k].x);
            v[1] = split_fast(x[k].y);
            ok = true;
        } else {
            ok = split_f64(x[k].x, v[0]) & split_f64(x[k].y, v[1]);
        }
        if (ok) {
            // lane 0: pr xr - pi xi, lane 1: pr xi + pi xr
            const float2 ah[2] = {make_float2(pr.h, pr.h), make_float2(-pi.h, pi.h)};
            const float2 al[2] = {make_float2(pr.l, pr.l), make_float2(-pi.l, pi.l)};
            const float2 bh[2] = {make_float2(v[0].h, v[1].h), make_float2(v[1].h, v[0].h)};
            const float2 bl[2] = {make_float2(v[0].l, v[1].l), make_float2(v[1].l, v[0].l)};
            float2 h, l;
            dot_x2<2>(ah, al, bh, bl, h, l);
            ab[idx[k]] = make_ulonglong2(join_f64(DF{h.x, l.x}), join_f64(DF{h.y, l.y}));
        } else {
            a[idx[k]] = cmul(pd, *reinterpret_cast<const double2*>(&x[k]));
        }
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

// Calls f with a compile-time map size: the exact count for 1-3 zero
// positions, 0 (generic) otherwise.
template <typename F>
void with_nz(int nz, F&& f)
{
    switch (nz) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        default: f(std::integral_constant<int, 0>{}); break;
    }
}

inline unsigned grid_for(uint64_t units, int per_block)
{
    uint64_t g = (units + per_block - 1) / per_block;
    return (unsigned)(g ? g : 1);
}

}  // namespace

namespace {
// Unit code of (re, im) if it is 1, i, -1 or -i (as unit_times), -1 for 0,
// -2 otherwise.
int unit_code(double re, double im)
{
    if (re == 0.0 && im == 0.0) return -1;
    if (re == 1.0 && im == 0.0) return 0;
    if (re == 0.0 && im == 1.0) return 1;
    if (re == -1.0 && im == 0.0) return 2;
    if (re == 0.0 && im == -1.0) return 3;
    return -2;
}

// A 2x2 matrix with one unit entry per row and column: (swap, u0, u1).
bool mono_pair(const double* m, int& swap, int& u0, int& u1)
{
    const int c00 = unit_code(m[0], m[1]), c01 = unit_code(m[2], m[3]);
    const int c10 = unit_code(m[4], m[5]), c11 = unit_code(m[6], m[7]);
    if (c00 >= 0 && c11 >= 0 && c01 == -1 && c10 == -1) {
        swap = 0, u0 = c00, u1 = c11;
        return true;
    }
    if (c01 >= 0 && c10 >= 0 && c00 == -1 && c11 == -1) {
        swap = 1, u0 = c01, u1 = c10;
        return true;
    }
    return false;
}
}  // namespace

cudaError_t launch_pair(void* amps, int prec, uint64_t total, const IndexMap& map,
                        uint64_t o0, uint64_t o1, const double* m, cudaStream_t st, bool fp64_exact)
{
    const uint64_t pairs = total >> map.nz;
    if (pairs == 0) return cudaSuccess;
    const unsigned grid = grid_for(pairs, kThreads * kUnroll);
    int swap = 0, u0 = 0, u1 = 0;
    const bool mono = mono_pair(m, swap, u0, u1);
    Mat2DF mx{};
    if (!mono && prec == kC128 && !fp64_exact)
        for (int j = 0; j < 2; ++j) {
            const DF r0 = host_split(m[4 * j]), i0 = host_split(m[4 * j + 1]);
            const DF r1 = host_split(m[4 * j + 2]), i1 = host_split(m[4 * j + 3]);
            const DF c[4][2] = {{r0, r0}, {r1, r1}, {DF{-i0.h, -i0.l}, i0}, {DF{-i1.h, -i1.l}, i1}};
            for (int k = 0; k < 4; ++k) {
                mx.h[j][k] = make_float2(c[k][0].h, c[k][1].h);
                mx.l[j][k] = make_float2(c[k][0].l, c[k][1].l);
            }
        }
    with_nz(map.nz, [&](auto nzc) {
        constexpr int NZ = decltype(nzc)::value;
        if (mono) {
            if (prec == kC128)
                k_pair_mono<double2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, pairs, map, o0, o1,
                                                                            swap, u0, u1);
            else
                k_pair_mono<float2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((float2*)amps, pairs, map, o0, o1, swap,
                                                                           u0, u1);
        } else if (prec == kC128 && fp64_exact) {
            k_pair<double2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, pairs, map, o0, o1,
                                                                   make_mat2<double2>(m));
        } else if (prec == kC128) {
            k_pair_c128x<kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, pairs, map, o0, o1, mx,
                                                                make_mat2<double2>(m));
        } else {
            auto mm = make_mat2<float2>(m);
            const bool pos0_free = map.nz == 0 || map.zpos[0] > 0;
            if (pos0_free && (map.setmask & 1) == 0 && ((o0 | o1) & 1) == 0 && pairs >= 2) {
                const uint64_t units = pairs / 2;
                k_pair_vec2<kUnroll, NZ><<<grid_for(units, kThreads * kUnroll), kThreads, 0, st>>>(
                    (float2*)amps, units, map, o0, o1, mm);
            } else if (o0 == 0 && o1 == 1 && (map.setmask & 1) == 0) {
                k_pair_adj<kUnroll, NZ><<<grid, kThreads, 0, st>>>((float2*)amps, pairs, map, mm);
            } else {
                k_pair<float2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((float2*)amps, pairs, map, o0, o1, mm);
            }
        }
    });
    return cudaGetLastError();
}

cudaError_t launch_phase(void* amps, int prec, uint64_t total, const IndexMap& map,
                         double ph_re, double ph_im, cudaStream_t st, bool fp64_exact)
{
    const uint64_t units = total >> map.nz;
    if (units == 0) return cudaSuccess;
    const unsigned grid = grid_for(units, kThreads * kUnroll);
    const int code = unit_code(ph_re, ph_im);
    with_nz(map.nz, [&](auto nzc) {
        constexpr int NZ = decltype(nzc)::value;
        if (code >= 0) {
            if (prec == kC128)
                k_phase_mono<double2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, units, map, code);
            else
                k_phase_mono<float2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((float2*)amps, units, map, code);
        } else if (prec == kC128 && fp64_exact) {
            k_phase<double2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, units, map,
                                                                    make_double2(ph_re, ph_im));
        } else if (prec == kC128) {
            k_phase_c128x<kUnroll, NZ><<<grid, kThreads, 0, st>>>((double2*)amps, units, map, host_split(ph_re),
                                                                 host_split(ph_im), make_double2(ph_re, ph_im));
        } else {
            const bool pos0_free = map.nz == 0 || map.zpos[0] > 0;
            if (pos0_free && (map.setmask & 1) == 0 && units >= 2) {
                k_phase_vec2<kUnroll, NZ><<<grid_for(units / 2, kThreads * kUnroll), kThreads, 0, st>>>(
                    (float2*)amps, units / 2, map, make_float2((float)ph_re, (float)ph_im));
            } else {
                k_phase<float2, kUnroll, NZ><<<grid, kThreads, 0, st>>>((float2*)amps, units, map,
                                                                       make_float2((float)ph_re, (float)ph_im));
            }
        }
    });
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
