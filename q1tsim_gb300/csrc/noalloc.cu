// Shot sampling that allocates no memory.
//
// Some callers cannot call cudaMalloc while they sample. One is a host
// framework that owns all device memory through its own pool allocator and
// forbids allocations behind its back. Another is a latency-critical loop,
// where cudaMalloc/cudaFree would stall on device-wide synchronisation. A
// third is a service that must not fail half-way through a request because
// device memory ran out: it sizes everything up front.
//
// q1g_sample_shots_noalloc serves them. The caller passes the column of
// amplitudes, the sorted uniforms and the output arrays, all in device memory.
// The sampler's scratch lives in one file-scope device array, g_noalloc_scratch:
// the chunk sums, the FP64 prefix scratch and total, and the classical-bit
// table. The array belongs to this file's module. With CUDA's lazy module
// loading, the module (and with it the array, about 0.5 MB) is loaded onto a
// device by the first call on that device, when it looks up the array's
// address; it then stays until the process exits. A caller that hands all
// free device memory to its own pool makes that first call (nshots = 0 is
// enough) beforehand. The kernels are the same as q1g_peek_all_into's
// (measure_kernels.cu), so for the same column and uniforms the outcomes are
// identical.
#include <mutex>
#include <string>

#include "engine.h"

namespace q1g {

namespace {

// Largest state the fixed scratch can sample: 2^24 amplitudes, that is
// 65536 chunk sums of 256 amplitudes.
constexpr int kNoAllocMaxBits = 24;
constexpr size_t kNoAllocChunkSums = size_t(1) << (kNoAllocMaxBits - 8);
// chunk sums + prefix scratch and total + 64 classical-bit masks
constexpr size_t kNoAllocScratchDoubles = kNoAllocChunkSums + 256 + 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_noalloc_mutex;
void* g_noalloc_addr[64] = {nullptr};

// Device address of the scratch array on the current device.  Looked up once
// per device (cudaGetSymbolAddress, which allocates nothing) on that device's
// first call.
double* noalloc_scratch()
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) throw Error(Q1G_ERR_DEVICE, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            throw Error(Q1G_ERR_DEVICE, std::string("cudaGetSymbolAddress of the sampling scratch: ") +
                                            cudaGetErrorString(e));
        }
        g_noalloc_addr[dev] = p;
    }
    return static_cast<double*>(g_noalloc_addr[dev]);
}

// The classical-bit mask of every bit position, passed to the kernel by
// value (a kernel parameter), so that no host buffer has to outlive the call.
struct CbitTable {
    uint64_t mask[64];
};

__global__ void k_store_cbit_table(uint64_t* __restrict__ dst, const __grid_constant__ CbitTable t)
{
    if (threadIdx.x < 64) dst[threadIdx.x] = t.mask[threadIdx.x];
}

}  // namespace

void sample_shots_noalloc(const void* d_amps, int precision, size_t nr_bits, const double* d_sorted_uniforms,
                          size_t nshots, uint64_t* d_outcomes, uint64_t* d_words, const size_t* cbits,
                          cudaStream_t st)
{
    if (precision != kC128 && precision != kC64)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "precision must be Q1G_C128 or Q1G_C64");
    if (nr_bits > (size_t)kNoAllocMaxBits)
        throw Error(Q1G_ERR_INVALID_ARGUMENT,
                    "q1g_sample_shots_noalloc handles at most " + std::to_string(kNoAllocMaxBits) +
                        " qubits (its fixed scratch holds 2^" + std::to_string(kNoAllocMaxBits - 8) +
                        " chunk sums); got " + std::to_string(nr_bits));
    if (!d_amps) throw Error(Q1G_ERR_INVALID_ARGUMENT, "NULL pointer: d_amps");
    if (nshots && (!d_sorted_uniforms || !d_outcomes || !d_words))
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "NULL pointer: uniforms or outputs");
    CbitTable table{};
    for (size_t q = 0; q < nr_bits; ++q) {
        const size_t cb = cbits ? cbits[q] : q;
        if (cb >= 64) throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit index " + std::to_string(cb), cb);
        table.mask[nr_bits - 1 - q] = uint64_t(1) << cb;
    }
    // the first call on a device looks the array up (and so loads it), even
    // with no shots to sample
    double* scratch = noalloc_scratch();
    if (nshots == 0) return;
    const uint64_t n = uint64_t(1) << nr_bits;
    const uint64_t chunk = n < 256 ? n : 256;
    const uint64_t nchunks = n / chunk;
    double* d_sums = scratch;
    double* d_stmp = scratch + nchunks;
    double* d_total = d_stmp + scan_tmp_doubles(nchunks);
    uint64_t* d_cpos = reinterpret_cast<uint64_t*>(scratch + kNoAllocChunkSums + 256);
    // every word of the table is rewritten, so nothing left from an earlier
    // call is read; the chunk sums, prefix and total are rewritten too
    k_store_cbit_table<<<1, 64, 0, st>>>(d_cpos, table);
    check_cuda(cudaGetLastError(), "store classical-bit table");
    check_cuda(launch_chunk_sums_dense(d_amps, precision, n, chunk, d_sums, st), "chunk_sums");
    check_cuda(launch_exclusive_scan(d_sums, nchunks, d_stmp, d_total, st), "prefix_scan");
    SampleArgs a{};
    a.amps = d_amps;
    a.prec = precision;
    a.col_len = n;
    a.chunk = chunk;
    a.excl = d_sums;
    a.nchunks = nchunks;
    a.total = d_total;
    a.u = d_sorted_uniforms;
    a.nruns = nshots;
    a.outcome = d_outcomes;
    a.word = d_words;
    a.nbits = (int)nr_bits;
    a.d_cbit_of_pos = d_cpos;
    check_cuda(launch_sample(a, st), "sample");
}

}  // namespace q1g
