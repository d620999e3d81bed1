// Host runtime of the engine: the device-resident VectorState and plans.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <exception>
#include <utility>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/q1gpu.h"
#include "gate_plan.h"
#include "kernels.h"

namespace q1g {

struct Error : std::exception {
    int code;
    std::string msg;
    // The payload of the reference's error variant (src/error.rs:135-152),
    // e.g. InvalidQBit(a0), NotEnoughSpace(a0, a1); 0 where it has none.
    uint64_t a0 = 0, a1 = 0;
    Error(int c, std::string m) : code(c), msg(std::move(m)) {}
    Error(int c, std::string m, uint64_t x0, uint64_t x1 = 0) : code(c), msg(std::move(m)), a0(x0), a1(x1) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

void check_cuda(cudaError_t e, const char* what);

// Grow-only device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    void ensure(size_t b);
    void release();
    void swap(DevBuf& o)
    {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
    }
    ~DevBuf() { release(); }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Grow-only pinned host allocation.
struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    void ensure(size_t b);
    void release();
    ~HostBuf() { release(); }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

struct ProfTotals {
    uint64_t launches = 0;
    double ms = 0.0;
    double bytes = 0.0;
};

// Inverse CDF of Binomial(n, p) at u (the n0 draw of measure_into).
uint64_t binomial_inv(uint64_t n, double p, double u);
double stream_uniform_host(uint64_t seed, uint64_t counter);

}  // namespace q1g

struct q1g_plan;

struct q1g_state {
    int nbits = 0;
    uint64_t nshots = 0;
    int prec = q1g::kC128;
    bool fp64_exact = false;   // complex128: FP64 arithmetic instead of double-float pairs
    uint64_t tc_wait_ns = 0;   // longest wait of a tensor-core pass (0: the kernel's default, 60 s)
    uint64_t N = 1;
    uint64_t ncols = 1;
    std::vector<uint64_t> counts;
    // Columns collapsed onto basis states are kept as indices only
    // (the reference materialises them densely, src/vectorstate.rs:150-158).
    bool sparse = true;
    std::vector<uint64_t> basis{0};
    // Squared norm each column should have.  Gates are unitary, so this only
    // changes at construction and measurement; plans that ran on the tensor
    // cores rescale their result to it (their FP32 accumulation rounds toward
    // zero and shrinks the norm by ~1e-7 per block).
    std::vector<double> norms{1.0};
    // After tensor-core passes the columns' actual norms may be off from
    // `norms` by ~1e-7 per block (FP32 accumulation rounds toward zero).
    // The rescale is left pending: sampling in measure_all divides by each
    // column's total and a collapse leaves exact basis columns, unitary gates
    // commute with it, and a later plan's passes keep the same bound.
    // settle_norms() applies it where absolute amplitudes matter (download,
    // compare, single-qubit measurement, conditional gates).
    bool norm_pending = false;

    q1g::DevBuf amps, spare;
    q1g::DevBuf dscratch;   // doubles
    q1g::DevBuf uscratch;   // uint64
    q1g::DevBuf matbuf;     // one dense matrix
    q1g::DevBuf colbuf;     // CollapseCol table
    q1g::DevBuf errbuf;     // error flag of bounded device waits
    q1g::HostBuf hstage;    // pinned staging for results
    cudaStream_t stream = nullptr;
    bool own_stream = false;

    bool prof = false;
    struct Pending {
        std::string name;
        double bytes;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::map<std::string, q1g::ProfTotals> totals;

    // A plan's leading blocks on a basis state run on this smaller state of
    // the positions they touch (plan_run); its buffers are reused.
    std::unique_ptr<q1g_state> compact;
    // apply_unary_gate_all: the n one-qubit gates as one fused plan (kept
    // for the next call, which differs only in the matrix).
    std::unique_ptr<q1g_plan> unary_plan;

    q1g_state(int nbits_, uint64_t nshots_, int prec_);
    q1g_state(int nbits_, uint64_t nshots_, int prec_, cudaStream_t shared);   // runs on `shared`
    ~q1g_state();

    size_t bsz() const { return q1g::amp_bytes(prec); }
    // Host <-> device copies on the state's stream, counted: the bytes the
    // state's calls moved over the host link (q1g_state_transfer_bytes).
    uint64_t h2d_bytes = 0, d2h_bytes = 0;
    void h2d(void* dst, const void* src, size_t n, const char* what)
    {
        q1g::check_cuda(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, stream), what);
        h2d_bytes += n;
    }
    void d2h(void* dst, const void* src, size_t n, const char* what)
    {
        q1g::check_cuda(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, stream), what);
        d2h_bytes += n;
    }
    int sms = 0;
    int sm_count()
    {
        if (!sms) {
            int dev = 0;
            q1g::check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
            q1g::check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
        }
        return sms;
    }
    uint64_t total() const { return ncols * N; }
    char* col_ptr(uint64_t c) const { return amps.as<char>() + c * N * bsz(); }

    // Launch through `f` (returning cudaError_t), timed when profiling.
    template <class F>
    void launch(const char* name, double bytes, F f)
    {
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof) {
            q1g::check_cuda(cudaEventCreate(&a), "cudaEventCreate");
            q1g::check_cuda(cudaEventRecord(a, stream), "cudaEventRecord");
        }
        q1g::check_cuda(f(), name);
        if (prof) {
            q1g::check_cuda(cudaEventCreate(&b), "cudaEventCreate");
            q1g::check_cuda(cudaEventRecord(b, stream), "cudaEventRecord");
            pending.push_back({name, bytes, a, b});
        }
    }
    void collect_profile();

    void ensure_dense();
    void settle_norms();
    std::vector<double> measure_norms();   // each column's squared norm, FP64, now
    void apply_op(const q1g::GateOp& op, char* base, uint64_t total_amps);
    void apply_gate(const double* mat, size_t k, const size_t* bits, size_t nbits_given);
    void apply_unary_all(const double* mat);
    void fill_random_normal(uint64_t seed);
    void apply_conditional(const uint8_t* control, size_t ncontrol, const double* mat, size_t k,
                           const size_t* bits, size_t nbits_given);
    std::vector<double> zero_weights(size_t qbit);
    void measure(size_t qbit, size_t cbit, uint64_t* res, size_t res_len, const double* uniforms,
                 size_t nu, q1g_rng* rng, bool collapse);
    void measure_all(const size_t* cbits, size_t ncbits, uint64_t* res, size_t res_len,
                     const double* uniforms, size_t nu, q1g_rng* rng, bool collapse);
    void reset_all();
    void download(double* out, size_t len);
    void sync();
};

namespace q1g {
// Tensor-core lowering of a pass: one or two fused blocks (each <= 5
// qubits) whose positions fit in one 12-position tile.  Each block is padded
// with untouched tile positions to five gate positions; its other seven tile
// positions are its rows.
struct TcPass {
    IndexMap tilemap{};
    TcOffsets offs{};
    TcTileBox box{};                // the tile as a tensor-map box
    std::vector<uint16_t> images;   // nblocks x kTcImageHalves f16
    long cost = 0, ideal = 0;       // the layout's predicted bank wavefronts per warp (chain layouts)
    TcTileBox sbox{};               // the storers' box when offs.st_box
};
// A pass's lowering kept by its plan, with what it was made from.
struct TcPassMemo {
    int nblocks = 0;
    int nbits = -1;
    int slack = 0;          // 8 x conflict slack + pair mode the lowering was made for
    uint64_t ncols = 0;
    std::vector<int> bits[kTcMaxBlocks];
    std::vector<std::complex<double>> mats[kTcMaxBlocks];
    TcPass pass;
};
}  // namespace q1g

struct q1g_plan {
    int nbits = 0;
    int width = 0;
    int tensor_cores = 1;          // 1: complex64 dense blocks on tcgen05; 0: CUDA cores
    std::vector<std::vector<int>> gate_bits;
    std::vector<size_t> mat_off;   // offset (doubles) of each gate's matrix
    size_t mat_doubles = 0;
    std::vector<q1g::FusedBlock> blocks;
    std::vector<unsigned char> kinds;      // per gate: q1g::GateKind (phase runs, swap runs)
    // The leading blocks of the plan touch only the positions of prefix_mask
    // (at most nbits - 3 of them): on a basis state they run on a compact
    // state (prefix_plan, the same blocks on compact qubits).  Worked out on
    // the first run; reset when the grouping changes.
    bool prefix_known = false;
    size_t prefix_len = 0;
    uint64_t prefix_mask = 0;
    std::unique_ptr<q1g_plan> prefix_plan;
    std::vector<q1g::TcPassMemo> tc_memo;   // by 3 * first block + block count - 1 (plan_run)
    // Tensor-core tiling (q1g_plan_set_tc_tiling, tuned by autotune.py):
    // whether two blocks may share a pass (0 no; 1 the second block reads
    // the first's results from the staged tile; 2 from registers, by warp
    // shuffles; 3 as operands the first block's write-back stored in the
    // stage, with no split of its own; 4 the same in the four-group kernel,
    // whose single-block passes also keep A in shared memory; 5 as 4 with up
    // to three blocks per pass), how many tile positions a pair's tile may have at or above
    // 2 MB strides, and how many times the minimum bank wavefronts an
    // unpadded one-box tile may take.
    int tc_pairs = 4;
    int tc_max_high = 8;
    int tc_slack = 4;
    q1g::HostBuf hmats;            // pinned staging of dense matrices
    q1g::DevBuf dmats;
    cudaEvent_t staged = nullptr;  // last upload of hmats finished
    size_t last_h2d_bytes = 0;     // matrices uploaded by the last run
    ~q1g_plan();
};

namespace q1g {
void plan_run(q1g_plan* p, q1g_state* s, const double* mats, size_t n, bool subspace_prefix = true);
// Reorders a plan's blocks (blocks on disjoint qubits commute) so that blocks
// that can share a tensor-core pass follow each other, up to `group` of them
// (3 in pair mode 4, else 2); max_high as q1g_plan::tc_max_high.
void order_blocks_for_tc_pairs(std::vector<FusedBlock>& blocks, int nbits, int max_high, int group);
// noalloc.cu: the sampler whose scratch is a fixed device array.
void sample_shots_noalloc(const void* d_amps, int precision, size_t nr_bits, const double* d_sorted_uniforms,
                          size_t nshots, uint64_t* d_outcomes, uint64_t* d_words, const size_t* cbits,
                          cudaStream_t st);
// histogram.cu: distinct words in ascending order with their counts.
void histogram_words(const uint64_t* words, size_t n, uint64_t* keys, uint64_t* counts, size_t capacity,
                     size_t* nkeys, cudaStream_t st);
}
