/*
 * q1gpu.h -- C ABI of the GB300 statevector engine for q1tsim.
 *
 * The engine replaces q1tsim's coefficient-vector backend, `VectorState`,
 * behind the `QuState` trait (src/qustate.rs:5-89, src/vectorstate.rs:164-416).
 * Each entry point below is the call a `QuState` implementation (Rust over
 * `extern "C"`, or Python over ctypes) makes for one trait method; the
 * reference item it replaces is cited beside it.
 *
 * Conventions
 *  - Plain pointers and sizes; no library-allocated return values.  The caller
 *    owns every host buffer and every handle (free with q1g_state_free /
 *    q1g_plan_free).  Outputs go into caller-provided arrays, as
 *    `measure_into(res: &mut Array1<u64>)` does (src/vectorstate.rs:237-238).
 *  - Every function returns a status code (Q1G_OK = 0).  The codes map 1:1 onto
 *    `crate::error::Error` variants (src/error.rs:135-152) plus device-side
 *    conditions; q1g_last_error() gives the message of the calling thread's
 *    last failure.  Nothing panics or aborts across the ABI.
 *  - Qubit 0 is the most significant bit of the amplitude index
 *    (src/gates.rs:133-141).  Gate matrices are 2^k x 2^k complex row-major
 *    arrays of (re, im) doubles whose first bit is bits[0] (src/gates.rs:40-53).
 *  - Sampling consumes host-supplied uniforms in [0, 1) when `uniforms` is
 *    non-NULL, else draws from the SplitMix64 stream `rng`, which it advances.
 *    Identical uniforms give identical shot outcomes.
 *  - A handle is used from one host thread at a time (a q1tsim Circuit is
 *    single-threaded, src/gates/parameter.rs:23-31).  Work runs on the
 *    handle's CUDA stream; results returned to host memory are synchronised.
 */
#ifndef Q1GPU_H
#define Q1GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  1..7 mirror crate::error::Error (src/error.rs:135-152). */
enum q1g_status {
    Q1G_OK = 0,
    Q1G_ERR_INVALID_NR_BITS = 1,             /* Error::InvalidNrBits */
    Q1G_ERR_INVALID_QBIT = 2,                /* Error::InvalidQBit */
    Q1G_ERR_INVALID_CBIT = 3,                /* Error::InvalidCBit */
    Q1G_ERR_INVALID_NR_CONTROL_BITS = 4,     /* Error::InvalidNrControlBits */
    Q1G_ERR_INVALID_NR_MEASUREMENT_BITS = 5, /* Error::InvalidNrMeasurementBits */
    Q1G_ERR_NOT_ENOUGH_SPACE = 6,            /* Error::NotEnoughSpace */
    Q1G_ERR_NOT_EXECUTED = 7,                /* Error::NotExecuted */
    Q1G_ERR_INVALID_ARGUMENT = 8,            /* NULL pointer, bad size or precision */
    Q1G_ERR_OUT_OF_MEMORY = 9,               /* device allocation or HBM budget */
    Q1G_ERR_DEVICE = 10,                     /* CUDA error */
    Q1G_ERR_TIMEOUT = 11                     /* a bounded device wait expired */
};

/* Amplitude precision of a state. */
enum q1g_precision {
    Q1G_C128 = 0, /* complex128 amplitudes, the drop-in mode: double-float arithmetic
                     (pairs of FP32, a quarter of the warps on the FP64 pipe) within
                     1e-12 by default, FP64 with q1g_state_set_fp64_exact */
    Q1G_C64 = 1   /* complex64 amplitudes, FP32 arithmetic, fused blocks on tensor cores */
};

typedef struct q1g_state q1g_state;
typedef struct q1g_plan q1g_plan;

/* SplitMix64 counter stream: draw k returns mix(seed + (counter+1)*gamma)
 * as a 53-bit uniform and increments counter.  Stands in for the `rng: &mut R`
 * argument of the QuState methods (src/qustate.rs:31-80). */
typedef struct q1g_rng {
    uint64_t seed;
    uint64_t counter;
} q1g_rng;

/* Message of the calling thread's last failed call ("" if none). */
const char* q1g_last_error(void);
/* Payload of the calling thread's last failed call, as the reference's
 * error variant carries it (src/error.rs:135-152), so that a binding can
 * rebuild the Error by value: InvalidNrBits(a0 = bits given, a1 = bits of
 * the gate), InvalidQBit(a0), InvalidCBit(a0), InvalidNrControlBits(a0 =
 * control bits given, a1 = runs), InvalidNrMeasurementBits(a0 = classical
 * bits given, a1 = qubits), NotEnoughSpace(a0 = result length, a1 = runs)
 * (src/vectorstate.rs:112-116, 172, 199, 242-246).  0 where the variant has
 * no payload.  Either pointer may be NULL. */
void q1g_last_error_args(uint64_t* a0, uint64_t* a1);
/* Library version (major*10000 + minor*100 + patch). */
int q1g_version(void);
/* Visible device: SM count and memory.  Any pointer may be NULL. */
int q1g_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes);

/* ---- construction: VectorState::new / from_qubit_coefs (src/vectorstate.rs:41-83) */

/* |0...0> on nr_bits qubits measured over nr_shots runs (src/vectorstate.rs:41-53). */
int q1g_state_new(size_t nr_bits, size_t nr_shots, int precision, q1g_state** out);
/* Product state; coefs = nr_bits pairs (c0, c1) of complex numbers, i.e.
 * 4*nr_bits doubles, each pair normalised (src/vectorstate.rs:62-83). */
int q1g_state_from_qubit_coefs(const double* coefs, size_t nr_bits, size_t nr_shots,
                               int precision, q1g_state** out);
/* Arbitrary initial state: 2^nr_bits complex (re, im) doubles, used as given.
 * No reference counterpart: the reference API cannot express it. */
int q1g_state_from_amplitudes(const double* amps, size_t nr_bits, size_t nr_shots,
                              int precision, q1g_state** out);
void q1g_state_free(q1g_state* s);

/* Run the state's work on a caller-owned cudaStream_t (NULL: the state's own). */
int q1g_state_set_stream(q1g_state* s, void* cuda_stream);
/* complex128 arithmetic of 1-qubit and diagonal updates: 0 (default) =
 * double-float pairs on the FP32 pipe (about 47 significant bits, within the
 * 1e-12 amplitude contract; GB300's FP64 pipe is a third of the HBM rate),
 * 1 = FP64 (the reference's own rounding, src/gates.rs:121-152).  No
 * reference counterpart. */
int q1g_state_set_fp64_exact(q1g_state* s, int exact);
/* Replaces every column by a random unit vector drawn on the device: the
 * real and imaginary parts of each amplitude i.i.d. N(0,1) (Box-Muller on
 * the SplitMix64 stream `seed`, amplitude i of column c from draws
 * 2(cN+i) and 2(cN+i)+1; FP64 math for Q1G_C128, FP32 for Q1G_C64), then
 * each column normalised in FP64.  Run counts are kept.  No counterpart in
 * the reference, whose constructors give |0...0> or product states only
 * (src/vectorstate.rs:41-83); it is from_amplitudes without the upload. */
int q1g_state_fill_random_normal(q1g_state* s, uint64_t seed);
/* Each column's squared norm, summed in FP64, into out[0..ncols). */
int q1g_state_column_norms(q1g_state* s, double* out, size_t len);
/* The state's amplitudes in device memory, densified and with any pending
 * norm correction applied: interleaved (re, im) in the state's precision,
 * column c at element c * 2^nr_bits, *bytes in all.  Valid until a call that
 * changes the state's shape (a measurement, a reset).  Work on the pointer
 * after this call returns, on a stream ordered after the state's; a caller
 * that wrote amplitudes calls q1g_state_amplitudes_written before the state's
 * next call.  It serves an exchange between shards of a larger state (the
 * sharded state of q1tsim_gb300/sharded.py). */
int q1g_state_device_amplitudes(q1g_state* s, void** ptr, size_t* bytes);
/* The caller changed the amplitudes in place: the state takes their column
 * norms as the norms its later tensor-core plans keep. */
int q1g_state_amplitudes_written(q1g_state* s);
int q1g_state_synchronize(q1g_state* s);
/* nr_bits, nr_shots, number of state columns, precision.  Any pointer may be NULL. */
int q1g_state_info(const q1g_state* s, size_t* nr_bits, size_t* nr_shots, size_t* ncols,
                   int* precision);
/* Run count of each column (VectorState::counts, src/vectorstate.rs:31-32). */
int q1g_state_counts(const q1g_state* s, uint64_t* out, size_t len);
/* Copy the state to host as complex128, column-major: out[(c*2^n + i)*2 + {0,1}]. */
int q1g_state_download(q1g_state* s, double* out, size_t len);

/* Accuracy of state b against state a (same qubit and column count), computed
 * on the device in FP64 over all amplitudes: out[0] = max |a_i - b_i|,
 * out[1] = 1 - |<a|b>|^2 / (<a|a><b|b>) (infidelity), out[2] = total-variation
 * distance of the outcome probabilities, out[3] = <a|a>, out[4] = <b|b>.
 * No reference counterpart: it reports the error of a complex64 run against
 * the complex128 one. */
int q1g_state_compare(q1g_state* a, q1g_state* b, double* out5);

/* ---- QuState methods (src/qustate.rs:5-89) */

/* apply_gate (src/vectorstate.rs:166-178 -> src/gates.rs:121-152).
 * k = nr_affected_bits of the gate; nbits must equal k (else INVALID_NR_BITS). */
int q1g_apply_gate(q1g_state* s, const double* mat, size_t k, const size_t* bits, size_t nbits);
/* apply_unary_gate_all (src/vectorstate.rs:180-189); mat is 2x2. */
int q1g_apply_unary_gate_all(q1g_state* s, const double* mat);
/* apply_conditional_gate (src/vectorstate.rs:193-227, src/qustate.rs:100-127):
 * control holds one byte per run (nonzero = apply); ncontrol must equal nr_shots. */
int q1g_apply_conditional_gate(q1g_state* s, const uint8_t* control, size_t ncontrol,
                               const double* mat, size_t k, const size_t* bits, size_t nbits);
/* measure_into (src/vectorstate.rs:237-329): one uniform per state column. */
int q1g_measure_into(q1g_state* s, size_t qbit, size_t cbit, uint64_t* res, size_t res_len,
                     const double* uniforms, size_t n_uniforms, q1g_rng* rng);
/* peek_into (src/vectorstate.rs:346-393): like measure_into, state unchanged. */
int q1g_peek_into(q1g_state* s, size_t qbit, size_t cbit, uint64_t* res, size_t res_len,
                  const double* uniforms, size_t n_uniforms, q1g_rng* rng);
/* measure_all_into (src/vectorstate.rs:106-161, 340-344): one uniform per run.
 * Within a column, runs receive outcomes in ascending basis-index order; the
 * state collapses onto one basis column per distinct outcome. */
int q1g_measure_all_into(q1g_state* s, const size_t* cbits, size_t ncbits, uint64_t* res,
                         size_t res_len, const double* uniforms, size_t n_uniforms,
                         q1g_rng* rng);
/* peek_all_into (src/vectorstate.rs:395-400): like measure_all_into, state unchanged. */
int q1g_peek_all_into(q1g_state* s, const size_t* cbits, size_t ncbits, uint64_t* res,
                      size_t res_len, const double* uniforms, size_t n_uniforms, q1g_rng* rng);
/* reset (src/vectorstate.rs:402-408): measure, then X where the result was 1. */
int q1g_reset(q1g_state* s, size_t bit, const double* uniforms, size_t n_uniforms, q1g_rng* rng);
/* reset_all (src/vectorstate.rs:410-415). */
int q1g_reset_all(q1g_state* s);

/* ---- gate sequences: the lowering point of Circuit::do_execute_with
 * (src/circuit.rs:643-653).  A plan holds the structure of a run of gates
 * (qubits per gate) and, for fusion_width > 0, their grouping into fused
 * blocks of at most fusion_width qubits (<= 5).  q1g_plan_run takes the
 * gate matrices for this execution, since parameters may change between
 * executions (src/gates/parameter.rs:23-75).  Fused blocks without controls
 * run in warp tiles: complex64 blocks of up to 4 qubits (5-qubit blocks on
 * the tensor cores), complex128 blocks of up to 3 qubits on double-float
 * pairs; larger complex128 blocks, and every block of a state set to
 * q1g_state_set_fp64_exact, use FP64 arithmetic, so complex128 plans are
 * best made with fusion_width <= 3. */

/* ks[g] = qubits of gate g; bits_flat = all gates' qubits concatenated. */
int q1g_plan_create(size_t nr_bits, size_t ngates, const size_t* ks, const size_t* bits_flat,
                    int fusion_width, q1g_plan** out);
void q1g_plan_free(q1g_plan* p);
/* Number of passes (fused blocks or single gates) the plan launches. */
/* Tells a plan what some of its gates always are, and regroups a fused plan
 * (fusion_width > 0) around them:
 * - Q1G_GATE_DIAGONAL (phases, controlled phases): a run of at least 3
 *   consecutive diagonal gates on at most two qubits each, whose two-qubit
 *   gates share one qubit, becomes one pass that multiplies every amplitude
 *   by the run's phase function, together with a following 1-qubit gate
 *   (complex64 states of up to 32 qubits; other states apply the run gate by
 *   gate);
 * - Q1G_GATE_SWAP: a run of at least 2 consecutive swaps on disjoint qubit
 *   pairs becomes one permutation pass (states of 10 qubits or more).
 * q1g_plan_run fails with Q1G_ERR_INVALID_ARGUMENT if a marked gate's matrix
 * is not what its kind says (a diagonal of unit-modulus entries, the swap
 * permutation). */
enum q1g_gate_kind { Q1G_GATE_GENERAL = 0, Q1G_GATE_DIAGONAL = 1, Q1G_GATE_SWAP = 2 };
int q1g_plan_set_gate_kinds(q1g_plan* p, const unsigned char* kinds, size_t ngates);
int q1g_plan_info(const q1g_plan* p, size_t* ngates, size_t* nblocks);
/* Block i of the plan: its qubits (ascending; *nq in/out) and the indices of
 * the gates it absorbed, in application order (*ng in/out). */
int q1g_plan_block(const q1g_plan* p, size_t i, size_t* qubits, size_t* nq, size_t* gates,
                   size_t* ng);
/* The fused 2^m x 2^m matrix of block i (m = its qubit count, qubits
 * ascending, first qubit the most significant index bit) for the gate
 * matrices mats_flat, written row-major as (re, im) doubles into out
 * (*n_out in: capacity in doubles, out: 2 * 4^m).  Host only, no device
 * work.  No reference counterpart: it exposes the matrix the fusion pass
 * (src/circuit.rs:651-653 runs the gates one by one) applies in one pass. */
int q1g_plan_block_matrix(const q1g_plan* p, size_t i, const double* mats_flat, size_t n_doubles, double* out,
                          size_t* n_out);
/* mats_flat = all gates' matrices concatenated ((re, im) doubles). */
int q1g_plan_run(q1g_plan* p, q1g_state* s, const double* mats_flat, size_t n_doubles);
/* Kernel for dense complex64 blocks of >= 3 qubits on states of >= 12 qubits:
 * 1 (default) = tcgen05 tensor cores (FP32-accurate: three f16 products of
 * 11-bit operand halves), 0 = CUDA cores (FP32). */
int q1g_plan_set_tensor_cores(q1g_plan* p, int enable);
/* Tiling of the plan's tensor-core passes (tuned per circuit structure by
 * q1tsim_gb300/autotune.py): allow_pairs lets two consecutive blocks whose
 * qubits fit one 12-position tile share a pass (0: no; 1: the
 * second block reads the first one's results back from the staged tile; 2:
 * from registers, the rows re-dealt by warp shuffles; 3: the first block's
 * write-back stores them as the second block's f16 operands in shared
 * memory, which its MMAs read directly; 4, the default: the same in a
 * kernel with four consumer groups, every pass's operands in shared
 * memory; 5: as 4, and three consecutive blocks share a pass where their
 * tile has runs of at least 64 bytes); a pair's tile may hold at
 * most max_high_positions positions at or above 2 MB strides (default 8: at
 * most 256 large pages per tile); an unpadded tile, one tensor-map copy, is
 * kept while its shared-memory bank wavefronts stay within conflict_slack
 * times the minimum (default 4), else it is padded and copied in pieces.
 * No counterpart in the reference. */
int q1g_plan_set_tc_tiling(q1g_plan* p, int allow_pairs, int max_high_positions, int conflict_slack);

/* ---- batches of independent circuits: one persistent launch, replayed from a
 * CUDA graph.  Each circuit runs on its own complex64 state of at most 16 run
 * columns.  A circuit is a program of gates, up to four mid-circuit Z
 * measurements, each splitting every run column by its outcome (measure_into,
 * src/vectorstate.rs:237-329), gates conditioned on one classical bit
 * (apply_conditional_gate, src/vectorstate.rs:193-227: every run of a column
 * holds the same bits, 0 for bits no measurement wrote), and a final
 * measure_all (src/vectorstate.rs:106-161).  This is what
 * Circuit::execute (src/circuit.rs:562-762) does for each circuit, for many
 * circuits at once.  Uniforms come from the SplitMix64 stream `seed` of each
 * circuit, drawn in the order the single-state entry points draw them. */
typedef struct q1g_batch q1g_batch;

enum q1g_batch_op {
    Q1G_OP_GATE = 0,        /* bits: k qubits; matrix 2^k x 2^k (k <= 4) */
    Q1G_OP_MEASURE = 1,     /* args: (qubit, cbit) */
    Q1G_OP_CONDITIONAL = 2, /* bits + matrix as a gate; args: (cbit, value 0/1) */
    Q1G_OP_MEASURE_ALL = 3  /* bits: the nr_bits classical bits (cbits[q] for qubit q); must be last */
};

/* fusion_width: 1..4 qubits per fused block. */
int q1g_batch_create(int fusion_width, q1g_batch** out);
void q1g_batch_free(q1g_batch* b);
/* Add one circuit.  kinds/nbits/args have nops entries (args: 2 per op);
 * bits_flat and mats_flat concatenate the ops' bits and matrices. */
int q1g_batch_add_circuit(q1g_batch* b, size_t nr_bits, size_t nr_shots, uint64_t seed, size_t nops,
                          const int* kinds, const size_t* nbits, const size_t* bits_flat,
                          const double* mats_flat, const size_t* args);
/* Run every circuit; results = each circuit's classical words, circuits in
 * the order added, runs in column order (the c_state of src/circuit.rs). */
int q1g_batch_run(q1g_batch* b, uint64_t* results, size_t len);
/* Circuits, total runs, device arena bytes, lowered ops, device time of the
 * last run in ms.  Any pointer may be NULL. */
int q1g_batch_info(const q1g_batch* b, size_t* ncircuits, size_t* total_runs, size_t* arena_bytes,
                   size_t* nops, double* last_ms);
/* Algorithmic device-memory bytes of the last run: every pass's amplitude
 * reads and writes (gate blocks, measurement, collapse, sampling) and the
 * classical words it updates, as counted by the kernel. */
int q1g_batch_traffic(const q1g_batch* b, uint64_t* bytes);

/* ---- profiling: per-kernel CUDA-event timing on the state's stream */
int q1g_profile_enable(q1g_state* s, int enable);
/* Kernel family names and totals since the last reset.  For entry i < *n:
 * names[i] (up to 31 chars + NUL in a 32-byte slot), launches, total device ms and
 * algorithmic bytes moved.  *n is in/out: capacity in, entries out. */
int q1g_profile_report(q1g_state* s, char* names, uint64_t* launches, double* ms,
                       double* bytes, size_t* n);
int q1g_profile_reset(q1g_state* s);
/* Bytes the state's calls copied host -> device and device -> host since it
 * was made or last reset (reset != 0 clears the counters after reading):
 * gate matrices, uniforms, tables and amplitudes in; outcomes, words,
 * weights, flags and amplitudes out.  Either pointer may be NULL. */
int q1g_state_transfer_bytes(q1g_state* s, uint64_t* h2d, uint64_t* d2h, int reset);
/* Longest time any wait inside a tensor-core pass of this state may last
 * before the pass gives up: its CTAs stop, drain the copies and MMAs still
 * in flight, release their tensor memory, and the plan fails with
 * Q1G_ERR_TIMEOUT, leaving the amplitudes undefined (reset or rebuild the
 * state).  seconds <= 0 restores the default, 60 s.  No counterpart in the
 * reference, whose CPU loop has no waits. */
int q1g_state_set_wait_limit(q1g_state* s, double seconds);

/* ---- shot sampling that allocates nothing.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc, such as a
 * framework whose pool allocator owns all device memory, or a
 * latency-critical loop that must not stall on an allocation.
 *
 * Samples nshots outcomes from one column of 2^nr_bits amplitudes (precision
 * Q1G_C128 or Q1G_C64) in device memory, using the ascending uniforms in
 * [0, 1) at d_sorted_uniforms (device).  It writes d_outcomes[r] (the basis
 * index) and d_words[r] (the classical word: qubit q's bit at cbits[q];
 * cbits NULL means cbits[q] = q, as VectorState::measure_all).  The kernels and
 * results are those of q1g_peek_all_into for the same column and uniforms.
 *
 * Scratch: a fixed device array inside the library, about 0.5 MB, holding up
 * to nr_bits = 24 (larger states are rejected with Q1G_ERR_INVALID_ARGUMENT).
 * The first call on a device looks up the array's address
 * (cudaGetSymbolAddress).  With CUDA's lazy module loading that lookup is what
 * loads the array onto the device, so the first call does take device memory;
 * every GPU keeps the array until the process exits.  Make that first call
 * (nshots = 0 is enough) before handing device memory to a pool.  All calls
 * share the one array and it keeps the last call's contents (every call
 * rewrites what it reads), so calls that overlap on the GPU race; serialise
 * them (one stream).  The call is asynchronous on
 * cuda_stream (NULL: the legacy default stream) and calls no cudaMalloc,
 * cudaFree or other allocating routine. */
int q1g_sample_shots_noalloc(const void* d_amps, int precision, size_t nr_bits,
                             const double* d_sorted_uniforms, size_t nshots, uint64_t* d_outcomes,
                             uint64_t* d_words, const size_t* cbits, void* cuda_stream);

/* Histogram of classical words, computed on the device (replaces the count
 * loop of Circuit::histogram, src/circuit.rs:773-789, for large shot counts):
 * the distinct words of the host array words[0..n), in no particular order
 * (the reference's histogram is a HashMap), with their counts, into keys[]
 * and counts[].  *nkeys receives the number of
 * distinct words; when it exceeds capacity the call fails with
 * Q1G_ERR_NOT_ENOUGH_SPACE and writes nothing else.  Runs on cuda_stream
 * (NULL: the legacy default stream) and returns when the result is on the
 * host. */
int q1g_histogram(const uint64_t* words, size_t n, uint64_t* keys, uint64_t* counts, size_t capacity,
                  size_t* nkeys, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* Q1GPU_H */
