// Histogram of classical words (c_state) on the device: the counts of
// Circuit::histogram (src/circuit.rs:773-789) for large shot counts, where a
// host sort of 10^6 words costs tens of milliseconds.
//
// An open-addressing hash table in HBM with at least twice as many slots as
// words: each word claims a slot with atomicCAS (linear probing, bounded by
// the table size, which a table with free slots never reaches) and counts
// there.  The all-ones word marks empty slots, so it is counted on its own.
// Used slots are then compacted, in no particular order (the reference's
// histogram is a HashMap); a caller that wants them sorted sorts the
// distinct words.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "engine.h"

namespace q1g {

namespace {

constexpr uint64_t kEmpty = ~uint64_t(0);

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 33)) * 0xff51afd7ed558ccdULL;
    z = (z ^ (z >> 33)) * 0xc4ceb9fe1a85ec53ULL;
    return z ^ (z >> 33);
}

__global__ void k_hist_insert(const uint64_t* __restrict__ words, uint64_t n, unsigned long long* keys,
                              unsigned long long* cnt, uint64_t cap, unsigned long long* all_ones, int* err)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t w = words[i];
        if (w == kEmpty) {
            atomicAdd(all_ones, 1ull);
            continue;
        }
        uint64_t h = mix64(w) & (cap - 1);
        bool done = false;
        for (uint64_t probe = 0; probe < cap; ++probe) {
            const unsigned long long old = atomicCAS(&keys[h], (unsigned long long)kEmpty, (unsigned long long)w);
            if (old == kEmpty || old == w) {
                atomicAdd(&cnt[h], 1ull);
                done = true;
                break;
            }
            h = (h + 1) & (cap - 1);
        }
        if (!done) atomicExch(err, 1);
    }
}

__global__ void k_hist_compact(const unsigned long long* keys, const unsigned long long* cnt, uint64_t cap,
                               unsigned long long* out_keys, unsigned long long* out_cnt, unsigned long long* nout)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < cap; s += stride) {
        const unsigned long long k = keys[s];
        if (k == kEmpty) continue;
        const unsigned long long j = atomicAdd(nout, 1ull);
        out_keys[j] = k;
        out_cnt[j] = cnt[s];
    }
}

unsigned grid_for(uint64_t n)
{
    const uint64_t b = (n + 255) / 256;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 152 * 16));
}

}  // namespace

// Distinct words of words[0..n), in no particular order, with their counts;
// at most `capacity` of them are written, *nkeys receives how many there are.
void histogram_words(const uint64_t* words, size_t n, uint64_t* keys, uint64_t* counts, size_t capacity,
                     size_t* nkeys, cudaStream_t st)
{
    *nkeys = 0;
    if (n == 0) return;
    uint64_t cap = 1024;
    while (cap < 2 * (uint64_t)n) cap <<= 1;
    // words | table keys | table counts | compacted keys | compacted counts | 2 counters
    const size_t bytes = (n + 4 * cap + 2) * sizeof(uint64_t);
    DevBuf buf;
    buf.ensure(bytes);
    DevBuf errb;
    errb.ensure(sizeof(int));
    uint64_t* d_words = buf.as<uint64_t>();
    auto* d_keys = reinterpret_cast<unsigned long long*>(d_words + n);
    auto* d_cnt = d_keys + cap;
    auto* d_okeys = d_cnt + cap;
    auto* d_ocnt = d_okeys + cap;
    auto* d_ctr = d_ocnt + cap;      // [0] distinct words in the table, [1] all-ones count
    check_cuda(cudaMemcpyAsync(d_words, words, n * sizeof(uint64_t), cudaMemcpyHostToDevice, st), "upload words");
    check_cuda(cudaMemsetAsync(d_keys, 0xff, cap * sizeof(uint64_t), st), "clear table");
    check_cuda(cudaMemsetAsync(d_cnt, 0, cap * sizeof(uint64_t), st), "clear counts");
    check_cuda(cudaMemsetAsync(d_ctr, 0, 2 * sizeof(uint64_t), st), "clear counters");
    check_cuda(cudaMemsetAsync(errb.p, 0, sizeof(int), st), "clear error");
    k_hist_insert<<<grid_for(n), 256, 0, st>>>(d_words, n, d_keys, d_cnt, cap, d_ctr + 1, errb.as<int>());
    check_cuda(cudaGetLastError(), "histogram insert");
    k_hist_compact<<<grid_for(cap), 256, 0, st>>>(d_keys, d_cnt, cap, d_okeys, d_ocnt, d_ctr);
    check_cuda(cudaGetLastError(), "histogram compact");
    uint64_t ctr[2] = {0, 0};
    int err = 0;
    check_cuda(cudaMemcpyAsync(ctr, d_ctr, sizeof ctr, cudaMemcpyDeviceToHost, st), "read counters");
    check_cuda(cudaMemcpyAsync(&err, errb.p, sizeof err, cudaMemcpyDeviceToHost, st), "read error flag");
    check_cuda(cudaStreamSynchronize(st), "histogram");
    if (err) throw Error(Q1G_ERR_DEVICE, "histogram table full");
    const uint64_t m = ctr[0];
    const size_t total = (size_t)m + (ctr[1] ? 1 : 0);
    *nkeys = total;
    if (total > capacity)
        throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "histogram has " + std::to_string(total) + " distinct words, room for " +
                                                  std::to_string(capacity));
    if (m) {
        check_cuda(cudaMemcpyAsync(keys, d_okeys, m * sizeof(uint64_t), cudaMemcpyDeviceToHost, st), "read keys");
        check_cuda(cudaMemcpyAsync(counts, d_ocnt, m * sizeof(uint64_t), cudaMemcpyDeviceToHost, st), "read counts");
        check_cuda(cudaStreamSynchronize(st), "histogram");
    }
    if (ctr[1]) {
        keys[m] = kEmpty;
        counts[m] = ctr[1];
    }
}

}  // namespace q1g
