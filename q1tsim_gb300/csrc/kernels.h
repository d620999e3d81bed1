// Host-side launch interface of the engine's CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <vector>
#include <stdint.h>

#include <complex>

#include "common.cuh"
#include "warp_tile.h"

namespace q1g {

constexpr int kC128 = 0;   // complex128 amplitudes, FP64 arithmetic
constexpr int kC64 = 1;    // complex64 amplitudes, FP32 arithmetic

inline size_t amp_bytes(int prec) { return prec == kC128 ? 16 : 8; }

// Offsets of the 2^t target basis states of a DENSE update (t <= 5).
struct DenseOffsets {
    uint64_t off[32];
};

// ---- gate_kernels.cu: one gate per pass over `total` amplitudes
// complex128 updates run on double-float pairs (df64.cuh) unless
// fp64_exact, which keeps FP64 arithmetic.
cudaError_t launch_pair(void* amps, int prec, uint64_t total, const IndexMap& map,
                        uint64_t o0, uint64_t o1, const double* m /*2x2 (re,im)*/,
                        cudaStream_t st, bool fp64_exact = false);
cudaError_t launch_phase(void* amps, int prec, uint64_t total, const IndexMap& map,
                         double ph_re, double ph_im, cudaStream_t st, bool fp64_exact = false);
// dmat: device matrix 2^tb x 2^tb, complex in the state's precision.
cudaError_t launch_dense(void* amps, int prec, uint64_t total, const IndexMap& map,
                         const DenseOffsets& offs, int tb, const void* dmat, cudaStream_t st);

// ---- phase_run.cu: a run of diagonal gates as one pass (complex64, <= 32 qubits)
// out: the 2048 complex factors of phi = c + L0 + x_pivot L1, lin0/lin1 the
// coefficients of L0/L1 per bit position (nbits each).
void phase_run_tables(int nbits, double c, const double* lin0, const double* lin1, float2* out);
// pivot_pos -1: no x_pivot term.  q_pos >= 0: then the 2x2 matrix m2 ((re, im)
// row-major) on the pairs along position q_pos, in the same pass.
cudaError_t launch_phase_run(float2* amps, uint64_t total, int nbits, int pivot_pos, const void* dtab, int q_pos,
                             const double* m2, int sm_count, cudaStream_t st);

// ---- swap_run.cu: a run of swaps on disjoint qubit pairs as one pass
// Layout of the pass (host): tiles of 1024 amplitudes over 10 positions
// closed under the swaps, the swaps outside them, and the stage offsets of
// every local index (wphys) and of the source of every destination (rphys).
struct SwapTile {
    int nouter;                 // swapped pairs outside the tile
    int pad_;
    int pa[32], pb[32];         // their positions
    uint64_t gbit[5];           // amplitude offset of slot bit b (positions 0..4 are the lane bits)
    IndexMap tile_map;          // the tile's 10 positions, zeroed
    uint16_t wphys[1024];
    uint16_t rphys[1024];
};
static_assert(sizeof(SwapTile) % 8 == 0, "SwapTile copies as 32-bit words");
// False when the pass does not apply (fewer than 10 qubits, pairs not disjoint).
bool swap_run_layout(SwapTile& t, const int* pa, const int* pb, int npairs, int nbits, int amp_bytes);
// dtile: the SwapTile in device memory; amp_bytes 8 (complex64) or 16.
cudaError_t launch_swap_run(void* amps, int amp_bytes, uint64_t total, const void* dtile, int sm_count,
                            cudaStream_t st);

// ---- dense_tiled.cu: uncontrolled dense blocks in warp tiles (warp_tile.h)
// True when the tiled kernel takes the block: no controls; complex64 on
// >= 10 qubits with t = 3 or 4, or t <= 2 with a gate at position 0 or 1
// (higher 1-2 qubit blocks are coalesced, and faster, per unit); complex128
// on >= 9 qubits with t <= 3 (double-float pairs).
bool dense_tiled_applies(int prec, int nbits, int t, const IndexMap& map, bool fp64_exact);
// The kernel's matrix image of a 2^t x 2^t complex matrix m (interleaved
// doubles): complex64 entries, or complex128 double-float terms followed by
// the FP64 matrix.
size_t dense_tiled_matrix_bytes(int prec, int t);
void dense_tiled_matrix(int prec, int t, const double* m, void* out);
cudaError_t launch_dense_tiled(void* amps, int prec, uint64_t total, int nbits, const IndexMap& map,
                               const DenseOffsets& offs, int t, const void* dmat, int sm_count, cudaStream_t st);

// ---- fused_tc.cu: 5-qubit fused blocks on the tensor cores (complex64)
// Geometry of one tensor-core pass over tiles of 2^12 amplitudes.  Tile
// coordinate x enumerates the tile's 12 positions in ascending order; its low
// run_bits bits are positions 0..run_bits-1, so a tile is nruns contiguous
// runs of 2^run_bits amplitudes at run_off[r] from the tile base.  A pass
// applies nblocks (1 or 2) 5-qubit blocks in turn to each staged tile; block
// b's 5 gate positions and 7 row positions all lie in the tile.
//
// In shared memory a staged tile keeps coordinate x at byte
// 8x + 16 (x >> pad_shift) (pad_shift 31: unpadded).  The padding moves rows
// that are a multiple of 32 amplitudes apart onto different banks; it is
// chosen per pass by tc_choose_padding.  Tiles are copied in npieces pieces
// of 2^piece_bits amplitudes (contiguous in both memories).
// Blocks one tensor-core pass may apply in turn (three only in the
// four-group kernel's direct chain).
constexpr int kTcMaxBlocks = 3;
struct TcBlockGeom {
    uint32_t jrow_bit[7];    // tile coordinate of row bit r (any order: rows are independent)
    uint32_t vec2;           // 1 if gate bit 0 is tile bit 0 (gate pairs adjacent)
    uint32_t jgate[32];      // tile coordinate of gate state g
    uint32_t rowoff[7];      // staged byte offset of row bit r
    uint32_t pad0_;
    uint32_t gateoff[32];    // staged byte offset of gate state g
};
struct TcOffsets {
    uint32_t run_bits;
    uint32_t nruns;
    uint32_t nblocks;
    uint32_t pad_shift;
    uint32_t piece_bits;
    uint32_t npieces;
    uint32_t nstages;        // filled in by launch_fused_tc
    uint32_t stage_bytes;
    uint32_t use_tma;        // 1: one tensor-map copy per tile (set by launch_fused_tc)
    uint32_t tshift[5];      // tensor-map coordinate d = (tile >> tshift[d]) & tmask[d]
    uint32_t tmask[5];
    // operand scales (tc_operand_scales): amplitudes enter the first block
    // as f16 times ascale; (D_main + 2^-11 D_corr) * unscale after the last
    float ascale;
    float unscale;
    // Two-block passes whose second block takes the first block's results
    // from registers (a plan's pair mode 2): the rows are laid out so that the tile bits that
    // change between gate and row role are lane bits, and register bit a of
    // a row swaps with lane bit swap_lane[a] (-1: kept) by warp shuffles.
    // The second block's gate order (its image, gateoff) is the register
    // order after the swaps.
    uint32_t shuffle;
    int32_t swap_lane[5];
    // Passes whose later blocks read their operands from shared memory (a
    // plan's pair modes 3 and 4): block b's write-back splits its results
    // into hi/lo f16 pairs and stores them straight into the stage as block
    // b+1's A operand (K-major, SWIZZLE_128B, hi plane then lo plane), at
    // byte (XOR over the thread's row bits i of scat_row[b][i]) XOR
    // scat_gate[b][g] for its output gate state g.  Block b+1's row and gate
    // orders are the ones that layout implies.
    uint32_t direct;
    uint64_t wait_ns;        // longest any wait may last (set by launch_fused_tc)
    uint64_t run_off[32];
    TcBlockGeom blk[kTcMaxBlocks];
    uint32_t scat_row[kTcMaxBlocks - 1][7];
    uint32_t scat_gate[kTcMaxBlocks - 1][32];
    // consumer groups of the kernel: 2 (0 means 2), or 4 with every A
    // operand in shared memory (plan pair mode 4; stage_bytes a multiple of
    // 1024)
    uint32_t groups;
    // 1: the storers copy the tile with a second tensor map (TcStoreBox), the
    // last block's staged offsets following its layout; coordinates as
    // tshift / tmask
    uint32_t st_box;
    uint32_t st_tshift[5];
    uint32_t st_tmask[5];
    // Four groups: how the first block's split deals the tile to a group's
    // 128 threads (tc_split_map).  Thread t (lane bits 0-4, warp bits 5-6
    // of t) reads its 32 amplitudes at staged offset (sum over t's bits i of
    // sp_thoff[i]) + sp_regoff[j] (register j: bits 0-1 are the block's gate
    // bits 0-1, so that registers 4q..4q+3 fill one 16-byte operand chunk)
    // and stores chunk q of each plane at (XOR over t's bits of sp_athr[i])
    // XOR sp_achunk[q].  sp_vec2: registers 2m, 2m+1 are adjacent in the
    // stage (16-byte loads).
    uint32_t sp_vec2;
    uint32_t sp_thoff[7];
    uint32_t sp_athr[7];
    uint32_t sp_achunk[8];
    uint32_t sp_regoff[32];
    // The last block's write-back with lane-permuted stores (a linear,
    // unpadded layout only; all zero otherwise): a thread whose lane has
    // bits r stores, at step j of each half row, its output gate state
    // j ^ wx, wx = XOR over its lane bits r of wb_xor[r] (gate bits 0-3;
    // 1-3 where the block stores 16 bytes per step).  Rows whose staged
    // offsets share banks then store to different banks at every step.
    uint32_t wb_xor[5];
};
// A tile as a box of a rank-5 tensor map over the state: dimensions follow
// the runs of tile / non-tile positions (tile runs split every 8 positions,
// the column index merged into the top dimension).  usable = 0 when more
// than 5 dimensions would be needed.
struct TcTileBox {
    int usable;
    uint64_t gdim[5];
    uint64_t gstride[5];     // bytes, dimensions 1..4
    uint32_t box[5];
    uint32_t tshift[5];
    uint32_t tmask[5];
};
TcTileBox tc_tile_box(const int* tile_pos /* 12, ascending */, int nbits, uint64_t ncols);
// A second box of the same tile for the stores: the tile's positions cut into
// dimensions of at most 8 positions in another order (dimension 0, which
// starts at position 0, first), so that in shared memory the tile bits lie
// in another order: tile bit j at element bit sbit[j].  Only the last
// block's write-back writes this layout, and only the storers read it.
struct TcStoreBox {
    TcTileBox box;
    int sbit[12];
};
// Store boxes for a tile whose last block has gate bits `gates` (tile bits):
// the identity order first, then orders that put that block's row bits in
// the low shared-memory bits (usable boxes only).
std::vector<TcStoreBox> tc_store_boxes(const int* tile_pos, int nbits, uint64_t ncols, uint32_t gates);
// Picks pad_shift (and piece_bits, npieces, stage_bytes, the blocks' staged
// offsets) that minimise shared-memory bank conflicts of the per-row reads.
// With tma_ok (the tile is one tensor-map box) an unpadded tile is kept when
// its conflicts stay within conflict_slack times the minimum: one tensor copy
// per tile beats padded piece copies.
void tc_choose_padding(TcOffsets& offs, bool tma_ok, int conflict_slack = 2);
// Row layout of a shuffled two-block pass (TcOffsets::shuffle): from block
// 0's gate order (jgate) and block 1's gate set, sets both blocks' row bits
// (lanes: the lowest common rows, then the bits that swap; warps: the other
// two common rows), swap_lane[k] for block 0's register bits, and block 1's
// gate order after the swaps (jgate, vec2), its register bit k holding tile
// bit reg1[k].  False if the blocks do not have five gate bits each.
bool tc_shuffle_layout(TcBlockGeom& b0, TcBlockGeom& b1, int32_t* swap_lane, int* reg1);
// Layout of a two-block pass in pair mode 3 (TcOffsets::direct): from block
// 0's gate order and block 1's gate set, picks the padding (as
// tc_choose_padding does, the same preference for one tensor-map copy) and
// both blocks' row orders and block 1's gate order (gbit1[k] = tile bit of
// its gate bit k) with the fewest predicted bank wavefronts over block 0's
// reads, its scattered operand stores and block 1's write-back; sets
// offs.direct, the scatter tables, block 1's jgate/vec2 and every staged
// offset.  Returns false when the blocks do not have 5 gate bits each.
bool tc_direct_layout(TcOffsets& offs, bool tma_ok, int conflict_slack, int* gbit1);
// Layout of a direct pass of the four-group kernel (2 or 3 blocks; the first
// block's split is dealt by tc_split_map, so its reads do not constrain its
// row order): picks the padding as tc_direct_layout does, block 0's row
// order and, for each later block, its gate order (gbits[b][k] = tile bit of
// its gate bit k) and row order, with the fewest predicted bank wavefronts
// over the scatters from block to block and the last block's write-back;
// sets offs.direct, the scatter tables, the later blocks' jgate/vec2 and
// every staged offset; *cost / *ideal: the chosen layout's predicted
// wavefronts per warp and their minimum.  With `stores` (an unpadded tile
// that is one box), the last block's write-back is evaluated in each store
// box and *store is the chosen one's index (its staged offsets are set from
// that box's sbit; -1: the load layout).  False when a block does not have
// 5 gate bits.
bool tc_chain_layout(TcOffsets& offs, bool tma_ok, int conflict_slack, int (*gbits)[5], long* cost = nullptr,
                     long* ideal = nullptr, const std::vector<TcStoreBox>* stores = nullptr, int* store = nullptr);
// Deal of the first block's tile to the threads of a four-group pass
// (TcOffsets::sp_*), after its layout (padding, row orders, scatter tables)
// is chosen: picks the block's gate bits 0-1 and the tile bits that vary
// across a warp's lanes so that its loads and its 16-byte operand stores
// take the fewest predicted bank wavefronts (the gate order is otherwise
// ascending); updates block 0's jgate, vec2, gate offsets and, in a direct
// pair, the scatter table.  gbit0[k]: tile bit of block 0's gate bit k.
void tc_split_map(TcOffsets& offs, int* gbit0);
// Byte offset of operand element (row r, K index k) in a K-major,
// SWIZZLE_128B f16 matrix of 128-byte rows (8-row groups of 1024 B).
inline uint32_t tc_sw128_offset(uint32_t r, uint32_t k)
{
    return (r >> 3) * 1024u + (r & 7u) * 128u + ((((k >> 3) ^ r) & 7u) << 4) + (k & 7u) * 2u;
}
// d_bimage: nblocks consecutive 16 KB f16 hi/lo images of the blocks' real
// 64x64 embeddings in the kernel's swizzled layout; d_err: set to 1 if a
// bounded wait expired.  wait_ns: longest any of the kernel's waits may
// last before it gives up (0: the default, 60 s).
// box: the tile as a tensor-map box (used for unpadded passes when usable);
// store_box: the storers' box when offs.st_box.
constexpr uint64_t kTcDefaultWaitNs = 60000000000ull;
cudaError_t launch_fused_tc(float2* amps, uint64_t ntiles, const IndexMap& tilemap, const TcOffsets& offs,
                            const TcTileBox& box, const void* d_bimage, int* d_err, int sm_count,
                            cudaStream_t st, uint64_t wait_ns = 0, const TcTileBox* store_box = nullptr);
// Host: the 16 KB image (8192 f16) for the 32x32 complex matrix m
// (row-major (re, im)), entries times 2^scale_log2: kTcLastBScaleLog2 for
// the last block of a pass, 0 for the one before (whose output stays scaled).
constexpr size_t kTcImageHalves = 8192;
constexpr int kTcLastBScaleLog2 = 14;
void build_tc_image(const double* m, uint16_t* image, int scale_log2);
// Host: offs.ascale / dmain / dcorr for states whose columns have squared
// norms at most max_norm.
void tc_operand_scales(double max_norm, TcOffsets& offs);
// Host: whether every row of the dim x dim block has 2-norm <= 1 (so that no
// amplitude outgrows its column norm, as the operand scale assumes).
bool tc_block_bounded(const std::complex<double>* m, int dim);

// ---- state_kernels.cu: construction, conversion, collapse
cudaError_t launch_fill_basis(void* amps, int prec, uint64_t n_amps, const uint64_t* d_col_index,
                              uint64_t ncols, uint64_t col_len, cudaStream_t st);
// Bit positions of a subspace: bit k of a compact index is position pos[k].
struct SubspacePositions {
    int n;
    int pos[48];
};
// Writes the full state of 2^nbits_full amplitudes: the amplitudes of
// `compact` at deposit(c) | fixed, zero elsewhere.  With at most
// kFillMaxExcluded positions outside the subspace one pass writes every
// amplitude; otherwise a memset and a scatter.
constexpr int kFillMaxExcluded = 8;
cudaError_t launch_scatter_subspace(void* full, const void* compact, int prec, int nbits_full, int nbits_compact,
                                   const SubspacePositions& sp, uint64_t fixed, cudaStream_t st);
cudaError_t launch_product_state(void* amps, int prec, int nbits, const double* d_coefs,
                                 cudaStream_t st);
cudaError_t launch_convert_c128_to_c64(float2* dst, const double2* src, uint64_t n, cudaStream_t st);
// total amplitudes with re, im i.i.d. N(0,1) from the SplitMix64 stream
// `seed` (amplitude i: Box-Muller of uniforms 2i, 2i+1); not normalised.
cudaError_t launch_random_normal(void* amps, int prec, uint64_t total, uint64_t seed, cudaStream_t st);
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
// tmp: segment_sums_tmp_doubles(nseg, len) doubles (none for short segments).
uint64_t segment_sums_tmp_doubles(uint64_t nseg, uint64_t len);
cudaError_t launch_segment_sums(const double* in, uint64_t nseg, uint64_t len, double* out, double* tmp,
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
    // nruns device words for each shot's chunk: with it the shots' chunks
    // come from one merge of the sorted targets with the prefix (a
    // separate launch) instead of a search per shot; nullptr: the search
    uint32_t* chunk_of;
};
cudaError_t launch_sample(const SampleArgs& a, cudaStream_t st);
// ---- batch.cu: many circuits in one persistent launch (complex64)
enum { kBatchDense = 0, kBatchMeasure = 1, kBatchSample = 2 };
struct BatchOp {
    int kind;
    int t;            // dense: target qubits (1..4)
    int cond;         // dense: -1 all columns, else only columns whose classical bit ccbit equals it
    int pos;          // measure: bit position
    int cbit;         // measure: classical bit
    uint32_t mat;     // dense: first float2 of the 2^t x 2^t matrix in the pool
    uint32_t cpos;    // sample: index of the 64-entry classical-bit table
    int ccbit;        // dense with cond >= 0: the classical bit tested
    uint64_t cmask;   // sample: classical bits the outcome overwrites
    IndexMap map;     // dense: the gate positions, zeroed
    uint64_t offs[16];
    // dense on states of >= 10 qubits: warp tiles of 1024 amplitudes
    // (warp_tile.h); tile.tiled = 0 below that
    WarpTile tile;
};

// Run columns a batched circuit may reach: each mid-circuit measurement
// splits every column in two, so at most four measurements per circuit.
constexpr int kBatchMaxCols = 16;
struct BatchCircuit {
    uint64_t state_off;   // amplitude offset of column 0 (the others follow, 2^nbits apart)
    uint64_t res_off;     // first classical word of this circuit's runs
    uint32_t op_begin, op_end;
    int nbits;
    int maxcols;          // column slots reserved in the arena
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
    unsigned long long* traffic;    // algorithmic bytes the launch moves in device memory (summed)
};
cudaError_t setup_batch_kernel();   // opt the batch kernel in to its shared-memory stage
cudaError_t launch_batch(const BatchArgs& a, int sm_count, cudaStream_t st);

// Per-block partials (6 doubles per block) comparing two states; wa and wb
// weight the probabilities in the total-variation term.
cudaError_t launch_compare(const void* a, int prec_a, const void* b, int prec_b, uint64_t n, double wa, double wb,
                           double* part, unsigned blocks, cudaStream_t st);
// Multiply column c by scales[c] (device array of ncols doubles).
cudaError_t launch_scale_columns(void* amps, int prec, uint64_t col_len, uint64_t ncols, const double* d_scales,
                                 cudaStream_t st);

}  // namespace q1g
