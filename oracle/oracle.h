/*
 * CPU oracle for the q1tsim coefficient-vector backend (TEST INFRASTRUCTURE).
 *
 * This is a plain-C, single-threaded, complex128 restatement of q1tsim's
 * `VectorState` (src/vectorstate.rs:24-416) and of the gate-application
 * drivers it calls (src/gates.rs:53-152, 210-326).  It exists only to check
 * the CUDA engine: tests, the smoke check and the bench's CPU-baseline leg
 * load it; the product library never links or calls it.
 *
 * Sampling streams of the reference (rand 0.7 WeightedIndex, rand_distr 0.2
 * Binomial, unseeded thread_rng) cannot be reproduced, so this oracle takes
 * host-supplied uniforms (or a SplitMix64 counter stream) and defines shot
 * outcomes as inverse-CDF draws of those uniforms; amplitude arithmetic is
 * pinned to the reference's known-answer tests (1e-15), sampling to its
 * statistical tests.
 */
#ifndef Q1TSIM_ORACLE_H
#define Q1TSIM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: the same numbering as the engine's C-ABI (q1gpu.h). */
enum {
    OR_OK = 0,
    OR_INVALID_NR_BITS = 1,
    OR_INVALID_QBIT = 2,
    OR_INVALID_CBIT = 3,
    OR_INVALID_NR_CONTROL_BITS = 4,
    OR_INVALID_NR_MEASUREMENT_BITS = 5,
    OR_NOT_ENOUGH_SPACE = 6,
    OR_NOT_EXECUTED = 7,
    OR_INVALID_ARGUMENT = 8,
    OR_OUT_OF_MEMORY = 9
};

typedef struct oracle_state oracle_state;

/* SplitMix64 counter stream: rng[0] = seed, rng[1] = counter (advanced). */
double oracle_uniform(uint64_t seed, uint64_t counter);

/* src/vectorstate.rs:41-53 */
oracle_state* oracle_new(size_t nr_bits, size_t nr_shots);
/* src/vectorstate.rs:62-83; coefs = 2*nr_bits complex numbers as (re, im) */
oracle_state* oracle_from_qubit_coefs(const double* coefs, size_t nr_bits, size_t nr_shots);
/* No reference counterpart: arbitrary normalised initial state (2^n complex). */
oracle_state* oracle_from_amplitudes(const double* amps, size_t nr_bits, size_t nr_shots);
void oracle_free(oracle_state* s);

size_t oracle_nr_bits(const oracle_state* s);
size_t oracle_nr_cols(const oracle_state* s);
void oracle_counts(const oracle_state* s, uint64_t* out);
/* Column-major copy of the state: out[(col*N + i)*2 + {0,1}]. */
int oracle_get_states(const oracle_state* s, double* out, size_t len);
/* Basis index of each column if the state is held as collapsed basis
 * columns, else -1 entries; returns 1 if sparse, 0 if dense. */
int oracle_is_sparse(const oracle_state* s);

/* src/vectorstate.rs:166-178 -> src/gates.rs:121-152 (k = nr_affected_bits,
 * mat = 2^k x 2^k complex row-major as (re, im) pairs). */
int oracle_apply_gate(oracle_state* s, const double* mat, size_t k,
                      const size_t* bits, size_t nbits);
/* src/vectorstate.rs:180-189 */
int oracle_apply_unary_gate_all(oracle_state* s, const double* mat);
/* src/vectorstate.rs:193-227 with src/qustate.rs:100-127 */
int oracle_apply_conditional_gate(oracle_state* s, const uint8_t* control, size_t ncontrol,
                                  const double* mat, size_t k,
                                  const size_t* bits, size_t nbits);
/* src/vectorstate.rs:237-329.  uniforms: one per column (or NULL -> rng). */
int oracle_measure_into(oracle_state* s, size_t qbit, size_t cbit,
                        uint64_t* res, size_t res_len,
                        const double* uniforms, size_t nu, uint64_t* rng);
/* src/vectorstate.rs:346-393 */
int oracle_peek_into(const oracle_state* s, size_t qbit, size_t cbit,
                     uint64_t* res, size_t res_len,
                     const double* uniforms, size_t nu, uint64_t* rng);
/* src/vectorstate.rs:106-161,340-344.  uniforms: one per run (or NULL). */
int oracle_measure_all_into(oracle_state* s, const size_t* cbits, size_t ncbits,
                            uint64_t* res, size_t res_len,
                            const double* uniforms, size_t nu, uint64_t* rng);
/* src/vectorstate.rs:395-400 */
int oracle_peek_all_into(oracle_state* s, const size_t* cbits, size_t ncbits,
                         uint64_t* res, size_t res_len,
                         const double* uniforms, size_t nu, uint64_t* rng);
/* src/vectorstate.rs:402-408 */
int oracle_reset(oracle_state* s, size_t bit, const double* uniforms, size_t nu, uint64_t* rng);
/* src/vectorstate.rs:410-415 */
void oracle_reset_all(oracle_state* s);

/* Helpers restated from src/support.rs:50-75 and src/qustate.rs:100-127. */
uint64_t oracle_reverse_bits(uint64_t idx, size_t nr_bits);
uint64_t oracle_shuffle_bits(uint64_t idx, const size_t* bits, size_t nbits);
/* Inverse CDF of Binomial(n, p) at uniform u (the n0 draw of measure_into). */
uint64_t oracle_binomial_inv(uint64_t n, double p, double u);

#ifdef __cplusplus
}
#endif
#endif
