// Runs of diagonal gates as one pass (gate_plan.h, fuse_runs).  Every
// amplitude i is multiplied by e^{i phi(x)}, x = i mod 2^n its basis bits and
//   phi(x) = c + L0(x) + x_p L1(x),   L0, L1 linear in the bits,
// from per-byte tables of complex factors (computed in double on the host):
//   T0[b][v] = e^{i L0(v << 8b)}  (T0[0] also carries e^{ic}),
//   T1[b][v] = e^{i L1(v << 8b)}.
// With a trailing 1-qubit gate on position q, its 2x2 matrix is then applied
// to each pair (i, i | 2^q) in the same pass.  complex64, states of up to 32
// qubits; a persistent grid, so that each CTA loads the 16 KB of tables into
// shared memory once.
#include <algorithm>
#include <cmath>
#include <complex>

#include "kernels.h"

namespace q1g {

namespace {

constexpr int kPhaseThreads = 256;
constexpr int kPhaseTable = 2048;   // T0 then T1, 4 bytes x 256 values each

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 phase_of(uint64_t i, uint64_t nmask, int pivot, const float2* T)
{
    const uint32_t x = (uint32_t)(i & nmask);
    float2 f = cmulf(cmulf(T[x & 255u], T[256 + ((x >> 8) & 255u)]),
                     cmulf(T[512 + ((x >> 16) & 255u)], T[768 + (x >> 24)]));
    if (pivot >= 0 && ((x >> pivot) & 1u)) {
        const float2* T1 = T + 1024;
        f = cmulf(f, cmulf(cmulf(T1[x & 255u], T1[256 + ((x >> 8) & 255u)]),
                           cmulf(T1[512 + ((x >> 16) & 255u)], T1[768 + (x >> 24)])));
    }
    return f;
}

__device__ __forceinline__ void load_tables(float2* T, const float2* __restrict__ gtab)
{
    for (int e = threadIdx.x; e < kPhaseTable; e += blockDim.x) T[e] = gtab[e];
    __syncthreads();
}

// Phases only: two amplitudes per 16-byte access (total is even).
__global__ void __launch_bounds__(kPhaseThreads)
k_phase_run(float2* a, uint64_t total, uint64_t nmask, int pivot, const float2* __restrict__ gtab)
{
    __shared__ float2 T[kPhaseTable];
    load_tables(T, gtab);
    float4* a4 = reinterpret_cast<float4*>(a);
    const uint64_t n2 = total / 2;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n2; v += (uint64_t)gridDim.x * blockDim.x) {
        const float4 q = a4[v];
        const float2 y0 = cmulf(phase_of(2 * v, nmask, pivot, T), make_float2(q.x, q.y));
        const float2 y1 = cmulf(phase_of(2 * v + 1, nmask, pivot, T), make_float2(q.z, q.w));
        a4[v] = make_float4(y0.x, y0.y, y1.x, y1.y);
    }
}

struct Mat2f {
    float2 m00, m01, m10, m11;
};

// Phases, then the 2x2 matrix on the pairs (i, i | bit); map zeroes position q.
__global__ void __launch_bounds__(kPhaseThreads)
k_phase_pair(float2* a, uint64_t pairs, IndexMap map, uint64_t bit, uint64_t nmask, int pivot,
             const float2* __restrict__ gtab, Mat2f m)
{
    __shared__ float2 T[kPhaseTable];
    load_tables(T, gtab);
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < pairs;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = expand_nz<1>(u, map), i1 = i0 | bit;
        const float2 y0 = cmulf(phase_of(i0, nmask, pivot, T), a[i0]);
        const float2 y1 = cmulf(phase_of(i1, nmask, pivot, T), a[i1]);
        const float2 p0 = cmulf(m.m00, y0), q0 = cmulf(m.m01, y1);
        const float2 p1 = cmulf(m.m10, y0), q1 = cmulf(m.m11, y1);
        a[i0] = make_float2(p0.x + q0.x, p0.y + q0.y);
        a[i1] = make_float2(p1.x + q1.x, p1.y + q1.y);
    }
}

}  // namespace

void phase_run_tables(int nbits, double c, const double* lin0, const double* lin1, float2* out)
{
    for (int t = 0; t < 2; ++t) {
        const double* coef = t == 0 ? lin0 : lin1;
        for (int b = 0; b < 4; ++b)
            for (int v = 0; v < 256; ++v) {
                double ph = (t == 0 && b == 0) ? c : 0.0;
                for (int k = 0; k < 8; ++k) {
                    const int pos = 8 * b + k;
                    if (pos < nbits && ((v >> k) & 1)) ph += coef[pos];
                }
                out[t * 1024 + b * 256 + v] = make_float2((float)std::cos(ph), (float)std::sin(ph));
            }
    }
}

cudaError_t launch_phase_run(float2* amps, uint64_t total, int nbits, int pivot_pos, const void* dtab, int q_pos,
                             const double* m2, int sm_count, cudaStream_t st)
{
    if (nbits < 1 || nbits > 32) return cudaErrorInvalidValue;
    const uint64_t nmask = nbits == 32 ? 0xFFFFFFFFull : ((uint64_t(1) << nbits) - 1);
    const uint64_t units = total / 2;   // amplitude pairs, or pairs of adjacent amplitudes
    const unsigned want = (unsigned)std::max<uint64_t>(1, (units + kPhaseThreads - 1) / kPhaseThreads);
    const unsigned grid = std::min<unsigned>(want, (unsigned)std::max(1, sm_count) * 8u);
    const float2* tab = static_cast<const float2*>(dtab);
    if (q_pos < 0) {
        k_phase_run<<<grid, kPhaseThreads, 0, st>>>(amps, total, nmask, pivot_pos, tab);
    } else {
        IndexMap map{};
        map.nz = 1;
        map.zpos[0] = q_pos;
        map.setmask = 0;
        Mat2f m{make_float2((float)m2[0], (float)m2[1]), make_float2((float)m2[2], (float)m2[3]),
                make_float2((float)m2[4], (float)m2[5]), make_float2((float)m2[6], (float)m2[7])};
        k_phase_pair<<<grid, kPhaseThreads, 0, st>>>(amps, total / 2, map, uint64_t(1) << q_pos, nmask, pivot_pos,
                                                     tab, m);
    }
    return cudaGetLastError();
}

}  // namespace q1g
