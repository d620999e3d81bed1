// Batched execution of many independent circuits in one persistent launch.
//
// Each circuit is a short program over its own complex64 state of up to
// kBatchMaxCols run columns (src/vectorstate.rs:24-35): fused gate blocks,
// up to four mid-circuit measurements, each splitting every column by its
// outcome (src/vectorstate.rs:237-329), gates conditioned on a classical bit
// (src/vectorstate.rs:193-227; every run of a column holds the same bits)
// and a final measure_all (src/vectorstate.rs:106-161).  The kernel keeps one CTA per SM slot; a CTA
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
#include "warp_tile.cuh"

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

// Smallest k with Binomial(n, p) CDF(k) > u; the host's binomial_inv.  The
// CTA evaluates the probability terms of up to kBinomChunk consecutive k in
// parallel into `terms`; thread 0 then accumulates them in ascending k, the
// same sums in the same order as the one-thread loop, so the same k.  Called
// by every thread of the CTA with the same arguments.
constexpr int kBinomChunk = 4096;
static_assert(kBinomChunk <= kBatchWarps * (1 << 10), "the terms fit in the tile stage");

__device__ uint64_t binomial_inv_block(uint64_t n, double p, double u, double* terms, uint64_t* s_k)
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
    double cdf = 0.0;   // thread 0's running sum
    for (uint64_t k0 = lo; k0 <= hi; k0 += kBinomChunk) {
        const uint64_t cnt = hi - k0 + 1 < (uint64_t)kBinomChunk ? hi - k0 + 1 : (uint64_t)kBinomChunk;
        for (uint64_t j = threadIdx.x; j < cnt; j += kBatchThreads) {
            const double kk = (double)(k0 + j);
            terms[j] = exp(lnf - lgamma(kk + 1.0) - lgamma(nn - kk + 1.0) + kk * lp + (nn - kk) * lq);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t found = ~uint64_t(0);
            for (uint64_t j = 0; j < cnt; ++j) {
                cdf += terms[j];
                if (u < cdf) {
                    found = k0 + j;
                    break;
                }
            }
            *s_k = found;
        }
        __syncthreads();
        const uint64_t f = *s_k;
        __syncthreads();
        if (f != ~uint64_t(0)) return f;
    }
    return hi;
}

// States below 10 qubits (smaller than a warp tile): one unit (the 2^TB amplitudes a
// block mixes) per thread.  mat[r * D + s] is the block's entry (r, s).
template <int TB>
__device__ void dense_pass(float2* a, uint64_t n_amps, const BatchOp& op, const float2* mat)
{
    constexpr int D = 1 << TB;
    const uint64_t units = n_amps >> op.map.nz;
    for (uint64_t u = threadIdx.x; u < units; u += kBatchThreads) {
        const uint64_t i = expand_index(u, op.map);
        float2 xa[D], xb[D];
#pragma unroll
        for (int s = 0; s < D; ++s) {
            const float2 v = a[i | op.offs[s]];
            xa[s] = make_float2(v.x, v.x);
            xb[s] = make_float2(v.y, v.y);
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            float2 ac = make_float2(0.f, 0.f), bc = make_float2(0.f, 0.f);
#pragma unroll
            for (int s = 0; s < D; ++s) {
                const float2 e = lds_entry(mat + r * D + s);
                ac = __ffma2_rn(xa[s], e, ac);
                bc = __ffma2_rn(xb[s], e, bc);
            }
            a[i | op.offs[r]] = cdot_out(ac, bc);
        }
    }
}

template <int TB>
__device__ __forceinline__ void apply_dense(float2* a, uint64_t n_amps, const BatchOp& op, const float2* mat,
                                            float2* stage)
{
    if (op.tile.tiled) tiled_dense_c64<TB, true>(a, n_amps, op.tile, mat, stage, threadIdx.x >> 5, kBatchWarps);
    else dense_pass<TB>(a, n_amps, op, mat);
}

__global__ void __launch_bounds__(kBatchThreads, 1)
k_batch(BatchArgs args)
{
    __shared__ float2 smat[256];
    __shared__ BatchOp sop;
    __shared__ uint64_t s_n0;
    extern __shared__ float2 stage_all[];
    float2* stage = stage_all + (threadIdx.x >> 5) * (1 << 10);
    __shared__ double red[kBatchWarps];
    __shared__ int s_circ;
    // per run column: runs, classical bits of its runs, and during a
    // measurement the weight of outcome 0, the draw and the first new slot
    __shared__ int s_ncols, s_nnew;
    __shared__ uint64_t s_counts[kBatchMaxCols], s_colword[kBatchMaxCols], s_n0k[kBatchMaxCols];
    __shared__ double s_w0[kBatchMaxCols];
    __shared__ int s_newidx[kBatchMaxCols];
    double* scratch = args.scratch + (uint64_t)blockIdx.x * args.scratch_per_cta;
    // algorithmic bytes (each pass's reads and writes of amplitudes and
    // classical words), counted by thread 0 in shared memory (no register is
    // held across the passes) and summed over the CTAs
    __shared__ unsigned long long s_moved;
    __shared__ unsigned s_cpass;   // dense column passes of the current circuit
    if (threadIdx.x == 0) s_moved = 0;

    for (;;) {
        if (threadIdx.x == 0) s_circ = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int c = s_circ;
        __syncthreads();
        if (c >= args.ncircuits) break;
        const BatchCircuit C = args.circuits[c];
        const uint64_t N = uint64_t(1) << C.nbits;
        float2* const col0 = args.arena + C.state_off;
        auto col = [&](int k) { return col0 + (uint64_t)k * N; };
        uint64_t* res = args.results + C.res_off;
        for (uint64_t v = threadIdx.x; v < N / 2; v += kBatchThreads)
            reinterpret_cast<float4*>(col0)[v] = make_float4(v == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
        if (threadIdx.x == 0) {
            s_ncols = 1;
            s_counts[0] = C.nshots;
            s_colword[0] = 0;
        }
        uint64_t ctr = 0;   // position in the circuit's uniform stream
        if (threadIdx.x == 0) {
            s_moved += N * sizeof(float2);
            s_cpass = 0;
        }
        __syncthreads();
        for (uint32_t oi = C.op_begin; oi < C.op_end; ++oi) {
            {
                static_assert(sizeof(BatchOp) % 4 == 0, "BatchOp copies as 32-bit words");
                const uint32_t* src = reinterpret_cast<const uint32_t*>(args.ops + oi);
                uint32_t* dst = reinterpret_cast<uint32_t*>(&sop);
                for (int w = threadIdx.x; w < (int)(sizeof(BatchOp) / 4); w += kBatchThreads) dst[w] = src[w];
            }
            __syncthreads();
            const int kind = sop.kind;
            if (kind == kBatchDense) {
                const int D = 1 << sop.t;
                for (int e = threadIdx.x; e < D * D; e += kBatchThreads) smat[e] = args.mats[sop.mat + e];
                __syncthreads();
                for (int k = 0; k < s_ncols; ++k) {
                    if (sop.cond >= 0 && (int)((s_colword[k] >> sop.ccbit) & 1u) != sop.cond) continue;
                    if (threadIdx.x == 0) ++s_cpass;
                    switch (sop.t) {
                        case 1: apply_dense<1>(col(k), N, sop, smat, stage); break;
                        case 2: apply_dense<2>(col(k), N, sop, smat, stage); break;
                        case 3: apply_dense<3>(col(k), N, sop, smat, stage); break;
                        default: apply_dense<4>(col(k), N, sop, smat, stage); break;
                    }
                }
                __syncthreads();
            } else if (kind == kBatchMeasure) {
                // per column: P(bit = 0) (src/vectorstate.rs:252-261) and
                // n0 ~ Binomial(runs, P) from the next uniform of the stream
                const uint64_t bit = uint64_t(1) << sop.pos;
                const int nc = s_ncols;
                for (int k = 0; k < nc; ++k) {
                    double acc = 0.0;
                    const float4* c4 = reinterpret_cast<const float4*>(col(k));   // two amplitudes (N >= 2)
#pragma unroll 4
                    for (uint64_t v = threadIdx.x; v < N / 2; v += kBatchThreads) {
                        const float4 q = c4[v];
                        if (!((2 * v) & bit)) acc += (double)psq(make_float2(q.x, q.y));
                        if (!((2 * v + 1) & bit)) acc += (double)psq(make_float2(q.z, q.w));
                    }
                    const double w0 = block_reduce(acc, red);
                    const uint64_t n0 = binomial_inv_block(s_counts[k], fmin(w0, 1.0), stream_uniform(C.seed, ctr + k),
                                                           reinterpret_cast<double*>(stage_all), &s_n0);
                    if (threadIdx.x == 0) {
                        s_w0[k] = w0;
                        s_n0k[k] = n0;
                    }
                    __syncthreads();
                }
                ctr += nc;
                // results: a column's first n0 runs read 0, the rest 1
                // (src/vectorstate.rs:290-297)
                {
                    const uint64_t one = uint64_t(1) << sop.cbit;
                    uint64_t r0 = 0;
                    for (int k = 0; k < nc; ++k) {
                        const uint64_t m = s_counts[k], n0 = s_n0k[k];
                        for (uint64_t r = threadIdx.x; r < m; r += kBatchThreads)
                            res[r0 + r] = r < n0 ? (res[r0 + r] & ~one) : (res[r0 + r] | one);
                        r0 += m;
                    }
                }
                // the new columns: outcome 0 then outcome 1 of each old column,
                // the empty ones left out (src/vectorstate.rs:299-322)
                if (threadIdx.x == 0) {
                    int nn = 0;
                    for (int k = 0; k < nc; ++k) {
                        s_newidx[k] = nn;
                        nn += (s_n0k[k] > 0 ? 1 : 0) + (s_n0k[k] < s_counts[k] ? 1 : 0);
                    }
                    s_nnew = nn;
                    s_moved += (uint64_t)(2 * nc + nn) * N * sizeof(float2) + 2 * C.nshots * sizeof(uint64_t);
                }
                __syncthreads();
                // collapse (src/vectorstate.rs:91-104), in place from the last
                // column down: column k's new slots lie at or above k and
                // below the slots of the columns after it
                for (int k = nc - 1; k >= 0; --k) {
                    const uint64_t m = s_counts[k], n0 = s_n0k[k];
                    const bool has0 = n0 > 0, has1 = n0 < m;
                    const double w0 = s_w0[k];
                    const float f0 = has0 ? (float)(1.0 / sqrt(w0)) : 0.f;
                    const float f1 = has1 ? (float)(1.0 / sqrt(1.0 - w0)) : 0.f;
                    const int base = s_newidx[k];
                    const float4* src = reinterpret_cast<const float4*>(col(k));
                    float4* d0 = reinterpret_cast<float4*>(col(base));
                    float4* d1 = reinterpret_cast<float4*>(col(base + (has0 ? 1 : 0)));
#pragma unroll 4
                    for (uint64_t v = threadIdx.x; v < N / 2; v += kBatchThreads) {
                        const float4 q = src[v];
                        const bool b0 = ((2 * v) & bit) != 0, b1 = ((2 * v + 1) & bit) != 0;
                        if (has1)
                            d1[v] = make_float4(b0 ? q.x * f1 : 0.f, b0 ? q.y * f1 : 0.f, b1 ? q.z * f1 : 0.f,
                                                b1 ? q.w * f1 : 0.f);
                        if (has0)
                            d0[v] = make_float4(b0 ? 0.f : q.x * f0, b0 ? 0.f : q.y * f0, b1 ? 0.f : q.z * f0,
                                                b1 ? 0.f : q.w * f0);
                    }
                    __syncthreads();
                }
                // the column list (runs and classical bits) follows the split
                if (threadIdx.x == 0) {
                    const uint64_t one = uint64_t(1) << sop.cbit;
                    for (int k = nc - 1; k >= 0; --k) {
                        const uint64_t m = s_counts[k], n0 = s_n0k[k], w = s_colword[k] & ~one;
                        int slot = s_newidx[k];
                        if (n0 > 0) {
                            s_counts[slot] = n0;
                            s_colword[slot] = w;
                            ++slot;
                        }
                        if (n0 < m) {
                            s_counts[slot] = m - n0;
                            s_colword[slot] = w | one;
                        }
                    }
                    s_ncols = s_nnew;
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
                        const double sum = chunk_sum(col(k), ch * chunk, chunk, lane);
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
                        if (sample_one((const float2*)col(k), chunk, excl, nch, total, u, lane, &idx)) {
                            const uint64_t r = r0 + j;
                            res[r] = (res[r] & mask) | outcome_word(idx, C.nbits, cpos);
                        }
                    }
                    ctr += m + 1;
                    r0 += m;
                    if (threadIdx.x == 0) s_moved += N * sizeof(float2) + m * (chunk * sizeof(float2) + 2 * sizeof(uint64_t));
                    __syncthreads();
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_moved += (unsigned long long)s_cpass * 2 * N * sizeof(float2);
    }
    if (threadIdx.x == 0) atomicAdd(args.traffic, s_moved);
}

}  // namespace

constexpr size_t kBatchStageBytes = size_t(kBatchWarps) * (size_t(1) << 10) * sizeof(float2);

cudaError_t setup_batch_kernel()
{
    return cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchStageBytes);
}

cudaError_t launch_batch(const BatchArgs& a, int sm_count, cudaStream_t st)
{
    const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sm_count, (uint64_t)a.ncircuits);
    if (grid == 0) return cudaSuccess;
    k_batch<<<grid, kBatchThreads, kBatchStageBytes, st>>>(a);
    return cudaGetLastError();
}

}  // namespace q1g
