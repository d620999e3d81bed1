/*
 * CPU oracle for the q1tsim coefficient-vector backend (TEST INFRASTRUCTURE:
 * only tests/, the smoke check and the bench's CPU-baseline leg use it).
 *
 * Single-threaded complex128 restatement of q1tsim's VectorState
 * (src/vectorstate.rs) following the reference's own algorithm: the state is a
 * row-major (2^n x ncols) matrix (src/cmatrix.rs:20-22, src/vectorstate.rs:24-35),
 * one-qubit gates run block by block (src/gates.rs:133-141), multi-qubit gates
 * gather through a bit permutation, apply the dense matrix, and scatter back
 * (src/gates.rs:53-80, 142-151, src/permutation.rs:141-163).  This is also the
 * "reference algorithm" timed as the CPU baseline.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct oracle_state {
    size_t nr_bits;
    size_t nr_shots;
    size_t ncols;
    uint64_t* counts;
    double* states;   /* dense: (i*ncols + j)*2 + {re,im}; NULL when sparse */
    uint64_t* basis;  /* sparse (collapsed) columns: basis index per column */
};

/* Beyond this many bytes a measure_all collapse keeps basis columns sparse
 * instead of materialising the reference's dense (2^n x #distinct) matrix
 * (src/vectorstate.rs:150-158). */
#define ORACLE_DENSE_COLLAPSE_LIMIT ((size_t)1 << 30)

/* ------------------------------------------------------------------ RNG */

/* SplitMix64 (Steele, Lea & Flood 2014; Vigna's constants): output k of the
 * stream seeded with `seed` is mix(seed + (k+1) * golden_gamma). */
static uint64_t splitmix_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double oracle_uniform(uint64_t seed, uint64_t counter)
{
    uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    return (double)(splitmix_mix(z) >> 11) * (1.0 / 9007199254740992.0);
}

static double rng_next(uint64_t* rng)
{
    double u = oracle_uniform(rng[0], rng[1]);
    rng[1] += 1;
    return u;
}

/* ------------------------------------------------------------- helpers */

/* src/support.rs:50-61 */
uint64_t oracle_reverse_bits(uint64_t idx, size_t nr_bits)
{
    uint64_t res = 0;
    for (size_t i = 0; i < nr_bits; ++i) {
        res |= (idx & 1) << (nr_bits - 1 - i);
        idx >>= 1;
    }
    return res;
}

/* src/support.rs:65-75 */
uint64_t oracle_shuffle_bits(uint64_t idx, const size_t* bits, size_t nbits)
{
    uint64_t res = 0;
    for (size_t i = 0; i < nbits; ++i) {
        res |= (idx & 1) << bits[i];
        idx >>= 1;
    }
    return res;
}

/* Inverse CDF of Binomial(n, p) at u: the smallest k with CDF(k) > u.  The
 * pmf is evaluated in log space (lgamma) from 40 sigma below the mean, where
 * the neglected mass is below 1e-300.  Stands in for rand_distr 0.2
 * Binomial::new(count, w0.min(1.0)) (src/vectorstate.rs:271, 379). */
uint64_t oracle_binomial_inv(uint64_t n, double p, double u)
{
    if (n == 0 || p <= 0.0) return 0;
    if (p >= 1.0) return n;
    double nn = (double)n;
    double mean = nn * p;
    double sd = sqrt(nn * p * (1.0 - p));
    double lo_d = floor(mean - 40.0 * sd - 40.0);
    double hi_d = ceil(mean + 40.0 * sd + 40.0);
    uint64_t lo = lo_d < 0.0 ? 0 : (uint64_t)lo_d;
    uint64_t hi = hi_d > nn ? n : (uint64_t)hi_d;
    double lp = log(p), lq = log1p(-p);
    double lnf = lgamma(nn + 1.0);
    double cdf = 0.0;
    for (uint64_t k = lo; k <= hi; ++k) {
        double kk = (double)k;
        double lpmf = lnf - lgamma(kk + 1.0) - lgamma(nn - kk + 1.0) + kk * lp + (nn - kk) * lq;
        cdf += exp(lpmf);
        if (u < cdf) return k;
    }
    return hi;
}

static int cmp_double(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* ------------------------------------------------------- construction */

static oracle_state* alloc_state(size_t nr_bits, size_t nr_shots, size_t ncols, int dense)
{
    oracle_state* s = (oracle_state*)calloc(1, sizeof(oracle_state));
    if (!s) return NULL;
    s->nr_bits = nr_bits;
    s->nr_shots = nr_shots;
    s->ncols = ncols;
    s->counts = (uint64_t*)calloc(ncols ? ncols : 1, sizeof(uint64_t));
    if (dense) {
        size_t n = (size_t)1 << nr_bits;
        s->states = (double*)calloc(n * ncols * 2, sizeof(double));
        if (!s->states) { free(s->counts); free(s); return NULL; }
    } else {
        s->basis = (uint64_t*)calloc(ncols ? ncols : 1, sizeof(uint64_t));
    }
    return s;
}

/* src/vectorstate.rs:41-53 */
oracle_state* oracle_new(size_t nr_bits, size_t nr_shots)
{
    oracle_state* s = alloc_state(nr_bits, nr_shots, 1, 1);
    if (!s) return NULL;
    s->states[0] = 1.0;
    s->counts[0] = nr_shots;
    return s;
}

/* src/vectorstate.rs:62-83: kron of per-qubit normalised (c0, c1) pairs,
 * qubit 0 most significant (src/cmatrix.rs:39-52). */
oracle_state* oracle_from_qubit_coefs(const double* coefs, size_t nr_bits, size_t nr_shots)
{
    oracle_state* s = alloc_state(nr_bits, nr_shots, 1, 1);
    if (!s) return NULL;
    size_t len = 1;
    s->states[0] = 1.0;
    s->states[1] = 0.0;
    for (size_t q = 0; q < nr_bits; ++q) {
        double a0r = coefs[4 * q + 0], a0i = coefs[4 * q + 1];
        double a1r = coefs[4 * q + 2], a1i = coefs[4 * q + 3];
        double norm = sqrt(a0r * a0r + a0i * a0i + a1r * a1r + a1i * a1i);
        /* num-complex Complex / f64 divides both parts */
        a0r /= norm; a0i /= norm; a1r /= norm; a1i /= norm;
        /* new[i*2 + b] = old[i] * bit[b], walking backwards in place */
        for (size_t ii = len; ii-- > 0;) {
            double xr = s->states[2 * ii], xi = s->states[2 * ii + 1];
            s->states[2 * (2 * ii + 1) + 0] = a1r * xr - a1i * xi;
            s->states[2 * (2 * ii + 1) + 1] = a1r * xi + a1i * xr;
            s->states[2 * (2 * ii) + 0] = a0r * xr - a0i * xi;
            s->states[2 * (2 * ii) + 1] = a0r * xi + a0i * xr;
        }
        len *= 2;
    }
    s->counts[0] = nr_shots;
    return s;
}

oracle_state* oracle_from_amplitudes(const double* amps, size_t nr_bits, size_t nr_shots)
{
    oracle_state* s = alloc_state(nr_bits, nr_shots, 1, 1);
    if (!s) return NULL;
    size_t n = (size_t)1 << nr_bits;
    memcpy(s->states, amps, n * 2 * sizeof(double));
    s->counts[0] = nr_shots;
    return s;
}

void oracle_free(oracle_state* s)
{
    if (!s) return;
    free(s->counts);
    free(s->states);
    free(s->basis);
    free(s);
}

size_t oracle_nr_bits(const oracle_state* s) { return s->nr_bits; }
size_t oracle_nr_cols(const oracle_state* s) { return s->ncols; }
int oracle_is_sparse(const oracle_state* s) { return s->states == NULL; }

void oracle_counts(const oracle_state* s, uint64_t* out)
{
    memcpy(out, s->counts, s->ncols * sizeof(uint64_t));
}

int oracle_get_states(const oracle_state* s, double* out, size_t len)
{
    size_t n = (size_t)1 << s->nr_bits;
    if (len < n * s->ncols * 2) return OR_NOT_ENOUGH_SPACE;
    if (!s->states) {
        memset(out, 0, n * s->ncols * 2 * sizeof(double));
        for (size_t j = 0; j < s->ncols; ++j) out[(j * n + s->basis[j]) * 2] = 1.0;
        return OR_OK;
    }
    for (size_t j = 0; j < s->ncols; ++j)
        for (size_t i = 0; i < n; ++i) {
            out[(j * n + i) * 2 + 0] = s->states[(i * s->ncols + j) * 2 + 0];
            out[(j * n + i) * 2 + 1] = s->states[(i * s->ncols + j) * 2 + 1];
        }
    return OR_OK;
}

/* A state collapsed onto sparse basis columns becomes dense again before any
 * operation that needs amplitudes. */
static int densify(oracle_state* s)
{
    if (s->states) return OR_OK;
    size_t n = (size_t)1 << s->nr_bits;
    s->states = (double*)calloc(n * s->ncols * 2, sizeof(double));
    if (!s->states) return OR_OUT_OF_MEMORY;
    for (size_t j = 0; j < s->ncols; ++j) s->states[(s->basis[j] * s->ncols + j) * 2] = 1.0;
    free(s->basis);
    s->basis = NULL;
    return OR_OK;
}

/* --------------------------------------------------------- gate apply */

/* Default dense Gate::apply_mat_slice (src/gates.rs:273-326) on a row range
 * of a row-major matrix with `ncols` columns: the rows split into 2^k equal
 * blocks s_j and block i becomes sum_j s_j * mat[i][j], accumulated in the
 * reference's order (s_0*m_i0 + s_1*m_i1 + ...). */
static void dense_apply_rows(double* rows, size_t nrows, size_t ncols,
                             const double* mat, size_t k, double* tmp)
{
    size_t dim = (size_t)1 << k;
    size_t n = nrows >> k;
    size_t blk = n * ncols;  /* complex elements per block */
    memcpy(tmp, rows, nrows * ncols * 2 * sizeof(double));
    for (size_t i = 0; i < dim; ++i) {
        double* dst = rows + i * blk * 2;
        for (size_t e = 0; e < blk; ++e) {
            double accr = 0.0, acci = 0.0;
            for (size_t j = 0; j < dim; ++j) {
                double mr = mat[(i * dim + j) * 2], mi = mat[(i * dim + j) * 2 + 1];
                double xr = tmp[(j * blk + e) * 2], xi = tmp[(j * blk + e) * 2 + 1];
                double pr = xr * mr - xi * mi;
                double pi = xr * mi + xi * mr;
                if (j == 0) { accr = pr; acci = pi; }
                else { accr += pr; acci += pi; }
            }
            dst[e * 2] = accr;
            dst[e * 2 + 1] = acci;
        }
    }
}

/* Permutation of src/gates.rs:53-80 as an index table: position `j` of the
 * permuted vector holds old index perm[j]; the gate bits become the top bits
 * (bits[0] most significant) and the other qubits keep their order. */
static size_t* bit_permutation(size_t nr_bits, const size_t* bits, size_t k)
{
    size_t n = (size_t)1 << nr_bits;
    size_t* perm = (size_t*)malloc(n * sizeof(size_t));
    if (!perm) return NULL;
    size_t rest_pos[64];
    size_t nrest = 0;
    for (size_t q = 0; q < nr_bits; ++q) {
        int is_gate = 0;
        for (size_t m = 0; m < k; ++m) if (bits[m] == q) is_gate = 1;
        if (!is_gate) rest_pos[nrest++] = nr_bits - 1 - q;  /* old bit position */
    }
    for (size_t j = 0; j < n; ++j) {
        size_t gate_idx = j >> (nr_bits - k);
        size_t rest = j & (((size_t)1 << (nr_bits - k)) - 1);
        size_t old = 0;
        for (size_t m = 0; m < k; ++m)
            old |= ((gate_idx >> (k - 1 - m)) & 1) << (nr_bits - 1 - bits[m]);
        for (size_t r = 0; r < nrest; ++r)
            old |= ((rest >> (nrest - 1 - r)) & 1) << rest_pos[r];
        perm[j] = old;
    }
    return perm;
}

/* src/gates.rs:121-152 for a row-major (2^nr_bits x ncols) matrix.  When
 * `only_col` >= 0 the gate is applied to that single column only, as
 * apply_gate_slice (src/gates.rs:86-115) does for conditional gates. */
static int apply_gate_matrix(double* states, size_t nr_bits, size_t ncols, long only_col,
                             const double* mat, size_t k, const size_t* bits)
{
    size_t n = (size_t)1 << nr_bits;
    size_t c0 = only_col >= 0 ? (size_t)only_col : 0;
    size_t nc = only_col >= 0 ? 1 : ncols;
    if (k == 1) {
        size_t block = (size_t)1 << (nr_bits - bits[0]);
        size_t nblocks = (size_t)1 << bits[0];
        double* buf = (double*)malloc(block * nc * 2 * sizeof(double));
        double* tmp = (double*)malloc(block * nc * 2 * sizeof(double));
        if (!buf || !tmp) { free(buf); free(tmp); return OR_OUT_OF_MEMORY; }
        for (size_t b = 0; b < nblocks; ++b) {
            /* gather the block's rows (of the selected columns) */
            for (size_t r = 0; r < block; ++r)
                for (size_t c = 0; c < nc; ++c) {
                    size_t src = ((b * block + r) * ncols + c0 + c) * 2;
                    buf[(r * nc + c) * 2] = states[src];
                    buf[(r * nc + c) * 2 + 1] = states[src + 1];
                }
            dense_apply_rows(buf, block, nc, mat, 1, tmp);
            for (size_t r = 0; r < block; ++r)
                for (size_t c = 0; c < nc; ++c) {
                    size_t dst = ((b * block + r) * ncols + c0 + c) * 2;
                    states[dst] = buf[(r * nc + c) * 2];
                    states[dst + 1] = buf[(r * nc + c) * 2 + 1];
                }
        }
        free(buf);
        free(tmp);
        return OR_OK;
    }
    size_t* perm = bit_permutation(nr_bits, bits, k);
    double* work = (double*)malloc(n * nc * 2 * sizeof(double));
    double* tmp = (double*)malloc(n * nc * 2 * sizeof(double));
    if (!perm || !work || !tmp) { free(perm); free(work); free(tmp); return OR_OUT_OF_MEMORY; }
    for (size_t j = 0; j < n; ++j)
        for (size_t c = 0; c < nc; ++c) {
            size_t src = (perm[j] * ncols + c0 + c) * 2;
            work[(j * nc + c) * 2] = states[src];
            work[(j * nc + c) * 2 + 1] = states[src + 1];
        }
    dense_apply_rows(work, n, nc, mat, k, tmp);
    for (size_t j = 0; j < n; ++j)
        for (size_t c = 0; c < nc; ++c) {
            size_t dst = (perm[j] * ncols + c0 + c) * 2;
            states[dst] = work[(j * nc + c) * 2];
            states[dst + 1] = work[(j * nc + c) * 2 + 1];
        }
    free(perm);
    free(work);
    free(tmp);
    return OR_OK;
}

static int check_bits(const oracle_state* s, size_t k, const size_t* bits, size_t nbits)
{
    if (nbits != k) return OR_INVALID_NR_BITS;
    for (size_t m = 0; m < nbits; ++m)
        if (bits[m] >= s->nr_bits) return OR_INVALID_QBIT;
    return OR_OK;
}

/* src/vectorstate.rs:166-178 */
int oracle_apply_gate(oracle_state* s, const double* mat, size_t k,
                      const size_t* bits, size_t nbits)
{
    int rc = check_bits(s, k, bits, nbits);
    if (rc) return rc;
    if ((rc = densify(s))) return rc;
    return apply_gate_matrix(s->states, s->nr_bits, s->ncols, -1, mat, k, bits);
}

/* src/vectorstate.rs:180-189 */
int oracle_apply_unary_gate_all(oracle_state* s, const double* mat)
{
    for (size_t b = 0; b < s->nr_bits; ++b) {
        int rc = oracle_apply_gate(s, mat, 1, &b, 1);
        if (rc) return rc;
    }
    return OR_OK;
}

/* src/qustate.rs:100-127: (column, length, apply) run-length triplets. */
typedef struct { size_t col; size_t len; int apply; } cond_range;

static cond_range* collect_conditional_ranges(const uint64_t* counts, size_t ncols,
                                              const uint8_t* control, size_t* nranges)
{
    size_t cap = 16, nr = 0, off = 0;
    cond_range* r = (cond_range*)malloc(cap * sizeof(cond_range));
    for (size_t icol = 0; icol < ncols; ++icol) {
        size_t count = counts[icol];
        if (count == 0) continue;
        size_t begin = off;
        int prev = control[off] != 0;
        for (size_t ib = off + 1; ib < off + count; ++ib) {
            int c = control[ib] != 0;
            if (c != prev) {
                if (nr == cap) { cap *= 2; r = (cond_range*)realloc(r, cap * sizeof(cond_range)); }
                r[nr].col = icol; r[nr].len = ib - begin; r[nr].apply = prev; ++nr;
                begin = ib;
                prev = !prev;
            }
        }
        if (begin < off + count) {
            if (nr == cap) { cap *= 2; r = (cond_range*)realloc(r, cap * sizeof(cond_range)); }
            r[nr].col = icol; r[nr].len = off + count - begin; r[nr].apply = prev; ++nr;
        }
        off += count;
    }
    *nranges = nr;
    return r;
}

/* src/vectorstate.rs:193-227 */
int oracle_apply_conditional_gate(oracle_state* s, const uint8_t* control, size_t ncontrol,
                                  const double* mat, size_t k,
                                  const size_t* bits, size_t nbits)
{
    if (ncontrol != s->nr_shots) return OR_INVALID_NR_CONTROL_BITS;
    int rc = check_bits(s, k, bits, nbits);
    if (rc) return rc;
    if ((rc = densify(s))) return rc;
    size_t nr;
    cond_range* ranges = collect_conditional_ranges(s->counts, s->ncols, control, &nr);
    size_t n = (size_t)1 << s->nr_bits;
    double* ns = (double*)calloc(n * (nr ? nr : 1) * 2, sizeof(double));
    uint64_t* nc = (uint64_t*)calloc(nr ? nr : 1, sizeof(uint64_t));
    if (!ns || !nc) { free(ns); free(nc); free(ranges); return OR_OUT_OF_MEMORY; }
    for (size_t j = 0; j < nr; ++j) {
        for (size_t i = 0; i < n; ++i) {
            ns[(i * nr + j) * 2] = s->states[(i * s->ncols + ranges[j].col) * 2];
            ns[(i * nr + j) * 2 + 1] = s->states[(i * s->ncols + ranges[j].col) * 2 + 1];
        }
        nc[j] = ranges[j].len;
    }
    for (size_t j = 0; j < nr; ++j)
        if (ranges[j].apply) {
            rc = apply_gate_matrix(ns, s->nr_bits, nr, (long)j, mat, k, bits);
            if (rc) { free(ns); free(nc); free(ranges); return rc; }
        }
    free(s->states);
    free(s->counts);
    s->states = ns;
    s->counts = nc;
    s->ncols = nr;
    free(ranges);
    return OR_OK;
}

/* --------------------------------------------------------- measurement */

/* P(qbit = 0) per column (src/vectorstate.rs:249-261 / 358-370). */
static void zero_weights(const oracle_state* s, size_t qbit, double* w0s)
{
    size_t block = (size_t)1 << (s->nr_bits - qbit - 1);
    size_t nblocks = (size_t)1 << qbit;
    for (size_t c = 0; c < s->ncols; ++c) w0s[c] = 0.0;
    if (!s->states) {
        for (size_t c = 0; c < s->ncols; ++c)
            w0s[c] = ((s->basis[c] >> (s->nr_bits - 1 - qbit)) & 1) ? 0.0 : 1.0;
        return;
    }
    for (size_t b = 0; b < nblocks; ++b)
        for (size_t r = 0; r < block; ++r) {
            size_t i = 2 * b * block + r;
            for (size_t c = 0; c < s->ncols; ++c) {
                double re = s->states[(i * s->ncols + c) * 2], im = s->states[(i * s->ncols + c) * 2 + 1];
                w0s[c] += re * re + im * im;
            }
        }
}

static int draw_column_uniforms(size_t ncols, const double* uniforms, size_t nu,
                                uint64_t* rng, double* out)
{
    if (uniforms) {
        if (nu < ncols) return OR_INVALID_ARGUMENT;
        memcpy(out, uniforms, ncols * sizeof(double));
    } else {
        if (!rng) return OR_INVALID_ARGUMENT;
        for (size_t c = 0; c < ncols; ++c) out[c] = rng_next(rng);
    }
    return OR_OK;
}

/* src/vectorstate.rs:91-104 on one column `j` of a row-major matrix. */
static void collapse_column(double* states, size_t ncols, size_t j, size_t block,
                            size_t nblocks, size_t offset, double norm_sq)
{
    size_t off = offset;
    for (size_t b = 0; b < nblocks; ++b) {
        for (size_t r = off; r < off + block; ++r) {
            states[(r * ncols + j) * 2] = 0.0;
            states[(r * ncols + j) * 2 + 1] = 0.0;
        }
        off += 2 * block;
    }
    double f = 1.0 / sqrt(norm_sq);
    size_t n = 2 * block * nblocks;
    for (size_t r = 0; r < n; ++r) {
        /* Complex * Complex(f, 0) */
        double re = states[(r * ncols + j) * 2], im = states[(r * ncols + j) * 2 + 1];
        states[(r * ncols + j) * 2] = re * f - im * 0.0;
        states[(r * ncols + j) * 2 + 1] = re * 0.0 + im * f;
    }
}

/* src/vectorstate.rs:237-329 */
int oracle_measure_into(oracle_state* s, size_t qbit, size_t cbit,
                        uint64_t* res, size_t res_len,
                        const double* uniforms, size_t nu, uint64_t* rng)
{
    if (qbit >= s->nr_bits) return OR_INVALID_QBIT;
    if (res_len < s->nr_shots) return OR_NOT_ENOUGH_SPACE;
    int rc = densify(s);
    if (rc) return rc;
    size_t n = (size_t)1 << s->nr_bits;
    size_t block = (size_t)1 << (s->nr_bits - qbit - 1);
    size_t nblocks = (size_t)1 << qbit;
    double* w0s = (double*)malloc(s->ncols * sizeof(double));
    double* us = (double*)malloc(s->ncols * sizeof(double));
    uint64_t* n0s = (uint64_t*)malloc(s->ncols * sizeof(uint64_t));
    if ((rc = draw_column_uniforms(s->ncols, uniforms, nu, rng, us))) {
        free(w0s); free(us); free(n0s); return rc;
    }
    zero_weights(s, qbit, w0s);
    size_t new_nr = 0;
    for (size_t c = 0; c < s->ncols; ++c) {
        double p = w0s[c] < 1.0 ? w0s[c] : 1.0;
        n0s[c] = oracle_binomial_inv(s->counts[c], p, us[c]);
        new_nr += (n0s[c] == 0 || n0s[c] == s->counts[c]) ? 1 : 2;
    }
    uint64_t one_mask = (uint64_t)1 << cbit;
    double* ns = (double*)calloc(n * new_nr * 2, sizeof(double));
    uint64_t* nc = (uint64_t*)calloc(new_nr, sizeof(uint64_t));
    size_t new_idx = 0, res_start = 0;
    for (size_t c = 0; c < s->ncols; ++c) {
        double w0 = w0s[c];
        uint64_t n0 = n0s[c], count = s->counts[c];
        for (size_t r = res_start; r < res_start + n0; ++r) res[r] &= ~one_mask;
        for (size_t r = res_start + n0; r < res_start + count; ++r) res[r] |= one_mask;
        res_start += count;
        for (size_t i = 0; i < n; ++i) {
            ns[(i * new_nr + new_idx) * 2] = s->states[(i * s->ncols + c) * 2];
            ns[(i * new_nr + new_idx) * 2 + 1] = s->states[(i * s->ncols + c) * 2 + 1];
        }
        if (n0 == count) {
            collapse_column(ns, new_nr, new_idx, block, nblocks, block, w0);
            nc[new_idx] = count;
        } else if (n0 == 0) {
            collapse_column(ns, new_nr, new_idx, block, nblocks, 0, 1.0 - w0);
            nc[new_idx] = count;
        } else {
            collapse_column(ns, new_nr, new_idx, block, nblocks, block, w0);
            nc[new_idx] = n0;
            ++new_idx;
            for (size_t i = 0; i < n; ++i) {
                ns[(i * new_nr + new_idx) * 2] = s->states[(i * s->ncols + c) * 2];
                ns[(i * new_nr + new_idx) * 2 + 1] = s->states[(i * s->ncols + c) * 2 + 1];
            }
            collapse_column(ns, new_nr, new_idx, block, nblocks, 0, 1.0 - w0);
            nc[new_idx] = count - n0;
        }
        ++new_idx;
    }
    free(s->states);
    free(s->counts);
    s->states = ns;
    s->counts = nc;
    s->ncols = new_nr;
    free(w0s); free(us); free(n0s);
    return OR_OK;
}

/* src/vectorstate.rs:346-393 */
int oracle_peek_into(const oracle_state* s, size_t qbit, size_t cbit,
                     uint64_t* res, size_t res_len,
                     const double* uniforms, size_t nu, uint64_t* rng)
{
    if (qbit >= s->nr_bits) return OR_INVALID_QBIT;
    if (res_len < s->nr_shots) return OR_NOT_ENOUGH_SPACE;
    double* w0s = (double*)malloc(s->ncols * sizeof(double));
    double* us = (double*)malloc(s->ncols * sizeof(double));
    int rc = draw_column_uniforms(s->ncols, uniforms, nu, rng, us);
    if (rc) { free(w0s); free(us); return rc; }
    zero_weights(s, qbit, w0s);
    uint64_t one_mask = (uint64_t)1 << cbit;
    size_t res_start = 0;
    for (size_t c = 0; c < s->ncols; ++c) {
        double p = w0s[c] < 1.0 ? w0s[c] : 1.0;
        uint64_t n0 = oracle_binomial_inv(s->counts[c], p, us[c]);
        for (size_t r = res_start; r < res_start + n0; ++r) res[r] &= ~one_mask;
        for (size_t r = res_start + n0; r < res_start + s->counts[c]; ++r) res[r] |= one_mask;
        res_start += s->counts[c];
    }
    free(w0s); free(us);
    return OR_OK;
}

/* Ascending uniforms for `m` runs of one column.  From explicit uniforms:
 * the column's slice, sorted.  From the stream: order statistics by
 * normalised exponential spacings, r_j = S_j / S_m with S_j the running sum
 * of E_k = -log1p(-u_k) over m+1 draws. */
static int column_sorted_uniforms(size_t m, const double* uniforms, size_t off,
                                  uint64_t* rng, double* out)
{
    if (uniforms) {
        memcpy(out, uniforms + off, m * sizeof(double));
        qsort(out, m, sizeof(double), cmp_double);
        return OR_OK;
    }
    if (!rng) return OR_INVALID_ARGUMENT;
    double sum = 0.0;
    for (size_t j = 0; j < m; ++j) {
        sum += -log1p(-rng_next(rng));
        out[j] = sum;
    }
    sum += -log1p(-rng_next(rng));
    for (size_t j = 0; j < m; ++j) out[j] /= sum;
    return OR_OK;
}

/* src/vectorstate.rs:106-161.  Column c's runs take ascending uniforms, so
 * their outcomes come out in ascending basis-index order; each distinct
 * outcome then becomes one collapsed column with its multiplicity. */
static int measure_all_helper(oracle_state* s, const size_t* cbits, size_t ncbits,
                              uint64_t* res, size_t res_len,
                              const double* uniforms, size_t nu, uint64_t* rng, int collapse)
{
    if (res_len < s->nr_shots) return OR_NOT_ENOUGH_SPACE;
    if (ncbits != s->nr_bits) return OR_INVALID_NR_MEASUREMENT_BITS;
    if (uniforms && nu < s->nr_shots) return OR_INVALID_ARGUMENT;
    size_t n = (size_t)1 << s->nr_bits;
    uint64_t mask = 0;
    for (size_t q = 0; q < ncbits; ++q) mask |= (uint64_t)1 << cbits[q];
    mask = ~mask;

    double* cum = (double*)malloc(n * sizeof(double));
    double* us = (double*)malloc((s->nr_shots ? s->nr_shots : 1) * sizeof(double));
    uint64_t* outc = (uint64_t*)malloc((s->nr_shots ? s->nr_shots : 1) * sizeof(uint64_t));
    if (!cum || !us || !outc) { free(cum); free(us); free(outc); return OR_OUT_OF_MEMORY; }

    size_t off = 0;
    for (size_t c = 0; c < s->ncols; ++c) {
        size_t m = s->counts[c];
        int rc = column_sorted_uniforms(m, uniforms, off, rng, us + off);
        if (rc) { free(cum); free(us); free(outc); return rc; }
        if (!s->states) {
            for (size_t r = 0; r < m; ++r) outc[off + r] = s->basis[c];
        } else {
            /* WeightedIndex over |a_i|^2: cumulative weights, then the first
             * index whose inclusive prefix exceeds u * total. */
            double acc = 0.0;
            size_t last_nz = 0;
            for (size_t i = 0; i < n; ++i) {
                double re = s->states[(i * s->ncols + c) * 2], im = s->states[(i * s->ncols + c) * 2 + 1];
                double w = re * re + im * im;
                if (w > 0.0) last_nz = i;
                acc += w;
                cum[i] = acc;
            }
            for (size_t r = 0; r < m; ++r) {
                double target = us[off + r] * acc;
                size_t lo = 0, hi = n;  /* first i with cum[i] > target */
                while (lo < hi) {
                    size_t mid = (lo + hi) / 2;
                    if (cum[mid] > target) hi = mid; else lo = mid + 1;
                }
                outc[off + r] = lo < n ? lo : last_nz;
            }
        }
        off += m;
    }
    /* outcome -> classical word (src/vectorstate.rs:135-148) */
    for (size_t r = 0; r < s->nr_shots; ++r) {
        uint64_t rev = oracle_reverse_bits(outc[r], s->nr_bits);
        uint64_t perm = oracle_shuffle_bits(rev, cbits, ncbits);
        res[r] = (res[r] & mask) | perm;
    }
    if (collapse) {
        size_t nd = 0;
        /* distinct (column, outcome) runs in order; a column boundary always
         * starts a new collapsed column */
        uint64_t* didx = (uint64_t*)malloc((s->nr_shots ? s->nr_shots : 1) * sizeof(uint64_t));
        uint64_t* dcnt = (uint64_t*)malloc((s->nr_shots ? s->nr_shots : 1) * sizeof(uint64_t));
        off = 0;
        for (size_t c = 0; c < s->ncols; ++c) {
            size_t m = s->counts[c];
            for (size_t r = 0; r < m; ++r) {
                if (r == 0 || outc[off + r] != outc[off + r - 1]) {
                    didx[nd] = outc[off + r];
                    dcnt[nd] = 0;
                    ++nd;
                }
                dcnt[nd - 1] += 1;
            }
            off += m;
        }
        free(s->states);
        free(s->basis);
        free(s->counts);
        s->states = NULL;
        s->basis = NULL;
        s->ncols = nd;
        s->counts = dcnt;
        if (n * nd * 2 * sizeof(double) <= ORACLE_DENSE_COLLAPSE_LIMIT) {
            s->states = (double*)calloc(n * (nd ? nd : 1) * 2, sizeof(double));
            for (size_t j = 0; j < nd; ++j) s->states[(didx[j] * nd + j) * 2] = 1.0;
            free(didx);
        } else {
            s->basis = didx;
        }
    }
    free(cum); free(us); free(outc);
    return OR_OK;
}

int oracle_measure_all_into(oracle_state* s, const size_t* cbits, size_t ncbits,
                            uint64_t* res, size_t res_len,
                            const double* uniforms, size_t nu, uint64_t* rng)
{
    return measure_all_helper(s, cbits, ncbits, res, res_len, uniforms, nu, rng, 1);
}

int oracle_peek_all_into(oracle_state* s, const size_t* cbits, size_t ncbits,
                         uint64_t* res, size_t res_len,
                         const double* uniforms, size_t nu, uint64_t* rng)
{
    return measure_all_helper(s, cbits, ncbits, res, res_len, uniforms, nu, rng, 0);
}

/* src/vectorstate.rs:402-408: measure, then X on the runs that read 1. */
int oracle_reset(oracle_state* s, size_t bit, const double* uniforms, size_t nu, uint64_t* rng)
{
    uint64_t* m = (uint64_t*)calloc(s->nr_shots ? s->nr_shots : 1, sizeof(uint64_t));
    int rc = oracle_measure_into(s, bit, 0, m, s->nr_shots, uniforms, nu, rng);
    if (rc) { free(m); return rc; }
    uint8_t* control = (uint8_t*)malloc(s->nr_shots ? s->nr_shots : 1);
    for (size_t r = 0; r < s->nr_shots; ++r) control[r] = m[r] != 0;
    static const double xmat[8] = {0, 0, 1, 0, 1, 0, 0, 0};
    rc = oracle_apply_conditional_gate(s, control, s->nr_shots, xmat, 1, &bit, 1);
    free(m);
    free(control);
    return rc;
}

/* src/vectorstate.rs:410-415 */
void oracle_reset_all(oracle_state* s)
{
    free(s->states);
    free(s->basis);
    free(s->counts);
    s->basis = NULL;
    s->ncols = 1;
    s->counts = (uint64_t*)calloc(1, sizeof(uint64_t));
    s->counts[0] = s->nr_shots;
    s->states = (double*)calloc(((size_t)1 << s->nr_bits) * 2, sizeof(double));
    s->states[0] = 1.0;
}
