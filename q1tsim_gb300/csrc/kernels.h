// Host-side launch interface of the engine's CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace q1g {

constexpr int kC128 = 0;   // complex128 amplitudes, FP64 arithmetic
constexpr int kC64 = 1;    // complex64 amplitudes, FP32 arithmetic

inline size_t amp_bytes(int prec) { return prec == kC128 ? 16 : 8; }

// Offsets of the 2^t target basis states of a DENSE update (t <= 5).
struct DenseOffsets {
    uint64_t off[32];
};

// ---- gate_kernels.cu: one gate per pass over `total` amplitudes
cudaError_t launch_pair(void* amps, int prec, uint64_t total, const IndexMap& map,
                        uint64_t o0, uint64_t o1, const double* m /*2x2 (re,im)*/,
                        cudaStream_t st);
cudaError_t launch_phase(void* amps, int prec, uint64_t total, const IndexMap& map,
                         double ph_re, double ph_im, cudaStream_t st);
// dmat: device matrix 2^tb x 2^tb, complex in the state's precision.
cudaError_t launch_dense(void* amps, int prec, uint64_t total, const IndexMap& map,
                         const DenseOffsets& offs, int tb, const void* dmat, cudaStream_t st);

// ---- fused_tc.cu: 5-qubit fused blocks on the tensor cores (complex64)
// Geometry of a tile of 2^12 amplitudes (5 gate + 7 row positions).  Tile
// coordinate bit b sits at position tpos[b]; it is row bit rowmask[b] or
// gate bit gatemask[b] (one of the two is zero).
struct TcOffsets {
    uint8_t tpos[12];
    uint32_t rowmask[12];
    uint32_t gatemask[12];
    uint32_t row_tbit[7];    // tile-coordinate mask of row bit r
    uint32_t jgate[32];      // tile coordinate of gate state g
    uint64_t koff[16];       // address offset of tile bits 8..11 = k
    uint32_t krow[16];       // row bits of tile bits 8..11 = k
    uint32_t kgate[16];      // gate bits of tile bits 8..11 = k
};
uint32_t fused_tc_smem_bytes();
// d_bimage: the block's 32 KB hi/lo image of the real 64x64 embedding in the
// kernel's swizzled layout; d_err: set to 1 if a bounded wait expired.
cudaError_t launch_fused_tc(float2* amps, uint64_t ntiles, const IndexMap& tilemap, const TcOffsets& offs,
                            const void* d_bimage, int* d_err, int sm_count, cudaStream_t st);
// Host: the 32 KB image for the 32x32 complex matrix m (row-major (re, im)).
void build_tc_image(const double* m, float* image);

// ---- state_kernels.cu: construction, conversion, collapse
cudaError_t launch_fill_basis(void* amps, int prec, uint64_t n_amps, const uint64_t* d_col_index,
                              uint64_t ncols, uint64_t col_len, cudaStream_t st);
cudaError_t launch_product_state(void* amps, int prec, int nbits, const double* d_coefs,
                                 cudaStream_t st);
cudaError_t launch_convert_c128_to_c64(float2* dst, const double2* src, uint64_t n, cudaStream_t st);
cudaError_t launch_convert_c64_to_c128(double2* dst, const float2* src, uint64_t n, cudaStream_t st);
// New column j = old column src_col[j] with amplitudes whose bit `pos` differs
// from keep[j] zeroed and the rest scaled by scale[j] (src/vectorstate.rs:91-104).
struct CollapseCol {
    uint64_t src_col;
    int keep;       // 0 or 1: the measured value this column keeps; -1: plain copy
    double scale;
};
cudaError_t launch_collapse_copy(void* dst, const void* src, int prec, uint64_t col_len, int pos,
                                 const CollapseCol* d_cols, uint64_t ncols, cudaStream_t st);

// ---- measure_kernels.cu
// Per-chunk FP64 sums of |a|^2.  The kernel walks `units` virtual indices j,
// reads amplitude expand_index(j, map) (so a map with zeroed positions reads
// only that sub-lattice, e.g. the qubit=0 half), and sums chunks of `chunk`
// consecutive j; chunk must divide the virtual column length.
cudaError_t launch_chunk_sums(const void* amps, int prec, uint64_t units, uint64_t chunk,
                              const IndexMap& map, double* out, cudaStream_t st);
// Chunk sums for shot sampling: `chunk` = min(2^n, 256) consecutive
// amplitudes per chunk, reduced as described in measure_kernels.cu.
cudaError_t launch_chunk_sums_dense(const void* amps, int prec, uint64_t total, uint64_t chunk, double* out,
                                    cudaStream_t st);
// Deterministic per-segment reduction: out[s] = sum of in[s*len .. (s+1)*len).
cudaError_t launch_segment_sums(const double* in, uint64_t nseg, uint64_t len, double* out,
                                cudaStream_t st);
// In-place exclusive prefix sum of n doubles; *total_out (device) = the sum.
// `tmp` must hold scan_tmp_doubles(n) doubles.
uint64_t scan_tmp_doubles(uint64_t n);
cudaError_t launch_exclusive_scan(double* data, uint64_t n, double* tmp, double* total_out,
                                  cudaStream_t st);
// Ascending uniforms by normalised exponential spacings from the SplitMix64
// stream (seed, counter0): out[j] = S_j / S_m, S_j = sum_{k<=j} -log1p(-u_k),
// for j < m, drawing m+1 uniforms.
// tmp: 2*(m+1) + scan_tmp_doubles(m+1) + 1 doubles.
cudaError_t launch_sorted_uniforms(uint64_t seed, uint64_t counter0, uint64_t m, double* out,
                                   double* tmp, cudaStream_t st);
// One warp per run: outcome[r] = first index i of the column with inclusive
// prefix > u[r] * total, found through the chunk prefix (excl), a warp scan
// of the chunk's group sums and a scan of the group; word[r] = classical
// word of the outcome.  `chunk` must be the one used for the chunk sums.
struct SampleArgs {
    const void* amps;       // the column
    int prec;
    uint64_t col_len;       // 2^n
    uint64_t chunk;
    const double* excl;     // exclusive chunk prefix, nchunks entries
    uint64_t nchunks;
    const double* total;    // device scalar
    const double* u;        // sorted uniforms of the column's runs
    uint64_t nruns;
    uint64_t* outcome;      // per run
    uint64_t* word;         // per run
    int nbits;
    const uint64_t* d_cbit_of_pos;  // classical bit mask for each bit position
};
cudaError_t launch_sample(const SampleArgs& a, cudaStream_t st);
// ---- batch.cu: many circuits in one persistent launch (complex64)
enum { kBatchDense = 0, kBatchMeasure = 1, kBatchSample = 2 };
struct BatchOp {
    int kind;
    int t;            // dense: target qubits (1..4)
    int cond;         // dense: -1 all columns, else only columns whose measured bit equals it
    int pos;          // measure: bit position
    int cbit;         // measure: classical bit
    uint32_t mat;     // dense: first float2 of the 2^t x 2^t matrix in the pool
    uint32_t cpos;    // sample: index of the 64-entry classical-bit table
    int pad_;
    uint64_t cmask;   // sample: classical bits the outcome overwrites
    IndexMap map;     // dense: the gate positions, zeroed
    uint64_t offs[16];
};
struct BatchCircuit {
    uint64_t state_off;   // amplitude offset of column 0 (column 1 follows)
    uint64_t res_off;     // first classical word of this circuit's runs
    uint32_t op_begin, op_end;
    int nbits;
    int pad_;
    uint64_t nshots;
    uint64_t seed;        // SplitMix64 stream of this circuit's uniforms
};
struct BatchArgs {
    float2* arena;
    uint64_t* results;
    const BatchCircuit* circuits;   // in queue order
    int ncircuits;
    const BatchOp* ops;
    const float2* mats;
    const uint64_t* cbit_tables;
    double* scratch;
    uint64_t scratch_per_cta;
    unsigned* queue;
};
cudaError_t launch_batch(const BatchArgs& a, int sm_count, cudaStream_t st);

// Per-block partials (6 doubles per block) comparing two states; wa and wb
// weight the probabilities in the total-variation term.
cudaError_t launch_compare(const void* a, int prec_a, const void* b, int prec_b, uint64_t n, double wa, double wb,
                           double* part, unsigned blocks, cudaStream_t st);
// Multiply column c by scales[c] (device array of ncols doubles).
cudaError_t launch_scale_columns(void* amps, int prec, uint64_t col_len, uint64_t ncols, const double* d_scales,
                                 cudaStream_t st);

}  // namespace q1g
