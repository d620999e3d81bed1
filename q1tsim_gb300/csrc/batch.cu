// Batched execution of many independent circuits in one persistent launch.
//
// Each circuit is a short program over its own complex64 state of up to two
// run columns (src/vectorstate.rs:24-35): fused gate blocks, at most one
// mid-circuit measurement (src/vectorstate.rs:237-329), gates conditioned on
// that measured bit (src/vectorstate.rs:193-227) and a final measure_all
// (src/vectorstate.rs:106-161).  The kernel keeps one CTA per SM slot; a CTA
// takes the next circuit from an atomic queue (largest circuits first) and
// runs its whole program: the gate passes stream the circuit's columns
// through registers, the measurement reduces and splits the column, and the
// shots are sampled from the final columns with the same search as the
// single-state sampler.  No CTA ever waits on another, so the launch needs no
// inter-CTA synchronisation.  The host replays the launch from a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "engine.h"
#include "sampling.cuh"

namespace q1g {

namespace {

constexpr int kBatchThreads = 512;
constexpr int kBatchWarps = kBatchThreads / 32;

__device__ __forceinline__ double block_reduce(double v, double* red)
{
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < kBatchWarps; ++k) s += red[k];
    return s;
}

// In-place exclusive FP64 scan of n values by the whole CTA; returns the sum.
__device__ double block_scan_excl(double* data, uint64_t n, double* wsum)
{
    double carry = 0.0;
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint64_t t0 = 0; t0 < n; t0 += 4 * kBatchThreads) {
        const uint64_t base = t0 + 4 * (uint64_t)threadIdx.x;
        double v[4], local = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = base + k < n ? data[base + k] : 0.0;
            local += v[k];
        }
        double incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (l >= o) incl += y;
        }
        __syncthreads();
        if (l == 31) wsum[w] = incl;
        __syncthreads();
        double before = carry, tile = 0.0;
        for (int k = 0; k < kBatchWarps; ++k) {
            if (k < w) before += wsum[k];
            tile += wsum[k];
        }
        double run = before + (incl - local);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (base + k < n) data[base + k] = run;
            run += v[k];
        }
        carry += tile;
    }
    __syncthreads();
    return carry;
}

// Smallest k with Binomial(n, p) CDF(k) > u; the host's binomial_inv.
__device__ uint64_t binomial_inv_dev(uint64_t n, double p, double u)
{
    if (n == 0 || p <= 0.0) return 0;
    if (p >= 1.0) return n;
    const double nn = (double)n;
    const double mean = nn * p;
    const double sd = sqrt(nn * p * (1.0 - p));
    const double lo_d = floor(mean - 40.0 * sd - 40.0);
    const double hi_d = ceil(mean + 40.0 * sd + 40.0);
    const uint64_t lo = lo_d < 0.0 ? 0 : (uint64_t)lo_d;
    const uint64_t hi = hi_d > nn ? n : (uint64_t)hi_d;
    const double lp = log(p), lq = log1p(-p);
    const double lnf = lgamma(nn + 1.0);
    double cdf = 0.0;
    for (uint64_t k = lo; k <= hi; ++k) {
        const double kk = (double)k;
        cdf += exp(lnf - lgamma(kk + 1.0) - lgamma(nn - kk + 1.0) + kk * lp + (nn - kk) * lq);
        if (u < cdf) return k;
    }
    return hi;
}

template <int TB>
__device__ void dense_pass(float2* a, uint64_t n_amps, const BatchOp& op, const float2* mat)
{
    constexpr int D = 1 << TB;
    const uint64_t units = n_amps >> op.map.nz;
    for (uint64_t u = threadIdx.x; u < units; u += kBatchThreads) {
        const uint64_t i = expand_index(u, op.map);
        float2 x[D];
#pragma unroll
        for (int s = 0; s < D; ++s) x[s] = a[i | op.offs[s]];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            float2 acc = cmul(mat[r * D], x[0]);
#pragma unroll
            for (int s = 1; s < D; ++s) {
                const float2 m = mat[r * D + s];
                acc.x += m.x * x[s].x - m.y * x[s].y;
                acc.y += m.x * x[s].y + m.y * x[s].x;
            }
            a[i | op.offs[r]] = acc;
        }
    }
}

__global__ void __launch_bounds__(kBatchThreads, 1)
k_batch(BatchArgs args)
{
    __shared__ float2 smat[256];
    __shared__ BatchOp sop;
    __shared__ double red[kBatchWarps];
    __shared__ int s_circ;
    __shared__ int s_ncols, s_colbit[2];
    __shared__ uint64_t s_counts[2];
    __shared__ double s_scale[2];
    __shared__ int s_keep[2];
    double* scratch = args.scratch + (uint64_t)blockIdx.x * args.scratch_per_cta;

    for (;;) {
        if (threadIdx.x == 0) s_circ = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int c = s_circ;
        __syncthreads();
        if (c >= args.ncircuits) break;
        const BatchCircuit C = args.circuits[c];
        const uint64_t N = uint64_t(1) << C.nbits;
        float2* col[2] = {args.arena + C.state_off, args.arena + C.state_off + N};
        uint64_t* res = args.results + C.res_off;
        for (uint64_t i = threadIdx.x; i < N; i += kBatchThreads) col[0][i] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
        if (threadIdx.x == 0) {
            s_ncols = 1;
            s_counts[0] = C.nshots;
            s_counts[1] = 0;
            s_colbit[0] = s_colbit[1] = -1;
        }
        uint64_t ctr = 0;   // position in the circuit's uniform stream
        __syncthreads();
        for (uint32_t oi = C.op_begin; oi < C.op_end; ++oi) {
            if (threadIdx.x == 0) sop = args.ops[oi];
            __syncthreads();
            const int kind = sop.kind;
            if (kind == kBatchDense) {
                const int D = 1 << sop.t;
                for (int e = threadIdx.x; e < D * D; e += kBatchThreads) smat[e] = args.mats[sop.mat + e];
                __syncthreads();
                for (int k = 0; k < s_ncols; ++k) {
                    if (sop.cond >= 0 && s_colbit[k] != sop.cond) continue;
                    switch (sop.t) {
                        case 1: dense_pass<1>(col[k], N, sop, smat); break;
                        case 2: dense_pass<2>(col[k], N, sop, smat); break;
                        case 3: dense_pass<3>(col[k], N, sop, smat); break;
                        default: dense_pass<4>(col[k], N, sop, smat); break;
                    }
                }
                __syncthreads();
            } else if (kind == kBatchMeasure) {
                // P(bit = 0) of the single column (src/vectorstate.rs:252-261)
                const uint64_t bit = uint64_t(1) << sop.pos;
                double acc = 0.0;
                for (uint64_t i = threadIdx.x; i < N; i += kBatchThreads)
                    if (!(i & bit)) acc += (double)psq(col[0][i]);
                const double w0 = block_reduce(acc, red);
                if (threadIdx.x == 0) {
                    const double u = stream_uniform(C.seed, ctr);
                    const uint64_t n0 = binomial_inv_dev(C.nshots, fmin(w0, 1.0), u);
                    const uint64_t one = uint64_t(1) << sop.cbit;
                    for (uint64_t r = 0; r < C.nshots; ++r) res[r] = r < n0 ? (res[r] & ~one) : (res[r] | one);
                    if (n0 == C.nshots || n0 == 0) {
                        s_ncols = 1;
                        s_keep[0] = n0 == 0 ? 1 : 0;
                        s_scale[0] = 1.0 / sqrt(n0 == 0 ? 1.0 - w0 : w0);
                        s_colbit[0] = s_keep[0];
                        s_counts[0] = C.nshots;
                    } else {
                        s_ncols = 2;
                        s_keep[0] = 0;
                        s_keep[1] = 1;
                        s_scale[0] = 1.0 / sqrt(w0);
                        s_scale[1] = 1.0 / sqrt(1.0 - w0);
                        s_colbit[0] = 0;
                        s_colbit[1] = 1;
                        s_counts[0] = n0;
                        s_counts[1] = C.nshots - n0;
                    }
                }
                ++ctr;
                __syncthreads();
                // collapse (src/vectorstate.rs:91-104), splitting into two columns
                const float f0 = (float)s_scale[0];
                const float f1 = s_ncols == 2 ? (float)s_scale[1] : 0.f;
                const bool two = s_ncols == 2;
                const uint64_t keep0 = s_keep[0] ? bit : 0;
                for (uint64_t i = threadIdx.x; i < N; i += kBatchThreads) {
                    const float2 v = col[0][i];
                    const bool b = (i & bit) != 0;
                    if (two) {
                        col[1][i] = b ? make_float2(v.x * f1, v.y * f1) : make_float2(0.f, 0.f);
                        col[0][i] = b ? make_float2(0.f, 0.f) : make_float2(v.x * f0, v.y * f0);
                    } else {
                        col[0][i] = ((i & bit) == keep0) ? make_float2(v.x * f0, v.y * f0) : make_float2(0.f, 0.f);
                    }
                }
                __syncthreads();
            } else if (kind == kBatchSample) {
                const uint64_t* cpos = args.cbit_tables + 64 * (uint64_t)sop.cpos;
                const uint64_t mask = ~sop.cmask;
                const uint64_t chunk = N < 256 ? N : 256;
                const uint64_t nch = N / chunk;
                double* excl = scratch;
                double* us = scratch + nch;
                uint64_t r0 = 0;
                for (int k = 0; k < s_ncols; ++k) {
                    const uint64_t m = s_counts[k];
                    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
                    for (uint64_t ch = warp; ch < nch; ch += kBatchWarps) {
                        const double sum = chunk_sum(col[k], ch * chunk, chunk, lane);
                        if (lane == 0) excl[ch] = sum;
                    }
                    __syncthreads();
                    const double total = block_scan_excl(excl, nch, red);
                    // ascending uniforms: normalised exponential spacings
                    for (uint64_t j = threadIdx.x; j <= m; j += kBatchThreads)
                        us[j] = -log1p(-stream_uniform(C.seed, ctr + j));
                    __syncthreads();
                    const double esum = block_scan_excl(us, m + 1, red);
                    // us[j] now holds S_{j-1}; S_j = us[j+1] for j < m
                    for (uint64_t j = warp; j < m; j += kBatchWarps) {
                        const double u = us[j + 1] / esum;
                        uint64_t idx;
                        if (sample_one((const float2*)col[k], chunk, excl, nch, total, u, lane, &idx)) {
                            const uint64_t r = r0 + j;
                            res[r] = (res[r] & mask) | outcome_word(idx, C.nbits, cpos);
                        }
                    }
                    ctr += m + 1;
                    r0 += m;
                    __syncthreads();
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_batch(const BatchArgs& a, int sm_count, cudaStream_t st)
{
    const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sm_count, (uint64_t)a.ncircuits);
    if (grid == 0) return cudaSuccess;
    k_batch<<<grid, kBatchThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace q1g
