// extern "C" entry points declared in include/q1gpu.h.  Every call is
// guarded: C++ exceptions become status codes plus a thread-local message,
// so nothing unwinds across the ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "batch.h"
#include "engine.h"

namespace q1g {

namespace {
thread_local std::string g_last_error;
thread_local uint64_t g_last_args[2] = {0, 0};

template <class F>
int guarded(F f)
{
    try {
        f();
        return Q1G_OK;
    } catch (const Error& e) {
        g_last_error = e.msg;
        g_last_args[0] = e.a0;
        g_last_args[1] = e.a1;
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_args[0] = g_last_args[1] = 0;
        g_last_error = "host allocation failed";
        return Q1G_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_last_args[0] = g_last_args[1] = 0;
        g_last_error = e.what();
        return Q1G_ERR_INVALID_ARGUMENT;
    } catch (...) {
        g_last_args[0] = g_last_args[1] = 0;
        g_last_error = "unknown error";
        return Q1G_ERR_INVALID_ARGUMENT;
    }
}

void need(const void* p, const char* what)
{
    if (!p) throw Error(Q1G_ERR_INVALID_ARGUMENT, std::string("NULL pointer: ") + what);
}

void check_new(size_t nr_bits, int precision)
{
    if (precision != Q1G_C128 && precision != Q1G_C64)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "precision must be Q1G_C128 or Q1G_C64");
    if (nr_bits > 40) throw Error(Q1G_ERR_INVALID_ARGUMENT, "at most 40 qubits per state");
}

}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

}  // namespace q1g

using namespace q1g;

extern "C" {

const char* q1g_last_error(void) { return g_last_error.c_str(); }

void q1g_last_error_args(uint64_t* a0, uint64_t* a1)
{
    if (a0) *a0 = g_last_args[0];
    if (a1) *a1 = g_last_args[1];
}

int q1g_version(void) { return 100; }

int q1g_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes)
{
    return guarded([&] {
        int dev = 0;
        check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (sm_count) check_cuda(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev), "attr");
        size_t f = 0, t = 0;
        check_cuda(cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
        if (free_bytes) *free_bytes = f;
        if (total_bytes) *total_bytes = t;
    });
}

int q1g_state_new(size_t nr_bits, size_t nr_shots, int precision, q1g_state** out)
{
    return guarded([&] {
        need(out, "out");
        check_new(nr_bits, precision);
        *out = new q1g_state((int)nr_bits, nr_shots, precision);
    });
}

int q1g_state_from_qubit_coefs(const double* coefs, size_t nr_bits, size_t nr_shots, int precision,
                               q1g_state** out)
{
    return guarded([&] {
        need(out, "out");
        need(coefs, "coefs");
        check_new(nr_bits, precision);
        // normalise each qubit's (c0, c1) pair (src/vectorstate.rs:69-73)
        std::vector<double> c(coefs, coefs + 4 * nr_bits);
        for (size_t q = 0; q < nr_bits; ++q) {
            double* p = c.data() + 4 * q;
            const double norm = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
            for (int j = 0; j < 4; ++j) p[j] /= norm;
        }
        auto* s = new q1g_state((int)nr_bits, nr_shots, precision);
        try {
            s->dscratch.ensure(std::max<size_t>(c.size(), 1) * sizeof(double));
            s->h2d(s->dscratch.p, c.data(), c.size() * sizeof(double), "upload coefs");
            s->amps.ensure(s->N * s->bsz());
            s->launch("product_state", double(s->N * s->bsz()), [&] {
                return launch_product_state(s->amps.p, s->prec, (int)nr_bits, s->dscratch.as<double>(), s->stream);
            });
            s->sync();
            s->sparse = false;
            s->basis.clear();
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}

int q1g_state_from_amplitudes(const double* amps, size_t nr_bits, size_t nr_shots, int precision,
                              q1g_state** out)
{
    return guarded([&] {
        need(out, "out");
        need(amps, "amps");
        check_new(nr_bits, precision);
        auto* s = new q1g_state((int)nr_bits, nr_shots, precision);
        try {
            s->amps.ensure(s->N * s->bsz());
            if (precision == Q1G_C128) {
                s->h2d(s->amps.p, amps, s->N * 16, "upload amplitudes");
            } else {
                s->spare.ensure(s->N * 16);
                s->h2d(s->spare.p, amps, s->N * 16, "upload amplitudes");
                s->launch("convert", double(s->N * 24), [&] {
                    return launch_convert_c128_to_c64(s->amps.as<float2>(), s->spare.as<double2>(), s->N, s->stream);
                });
            }
            s->sync();
            if (s->spare.bytes > (size_t(1) << 30)) s->spare.release();
            s->sparse = false;
            s->basis.clear();
            double nrm = 0.0;
            for (uint64_t i = 0; i < 2 * s->N; ++i) nrm += amps[i] * amps[i];
            s->norms.assign(1, nrm);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}

void q1g_state_free(q1g_state* s) { delete s; }

int q1g_state_set_fp64_exact(q1g_state* s, int exact)
{
    return guarded([&] {
        need(s, "state");
        s->fp64_exact = exact != 0;
    });
}

int q1g_state_set_stream(q1g_state* s, void* cuda_stream)
{
    return guarded([&] {
        need(s, "state");
        s->sync();
        if (cuda_stream) {
            if (s->own_stream) cudaStreamDestroy(s->stream);
            s->stream = (cudaStream_t)cuda_stream;
            s->own_stream = false;
        } else if (!s->own_stream) {
            check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            s->own_stream = true;
        }
        if (s->compact) s->compact->stream = s->stream;
    });
}

int q1g_state_synchronize(q1g_state* s)
{
    return guarded([&] {
        need(s, "state");
        s->sync();
    });
}

int q1g_state_info(const q1g_state* s, size_t* nr_bits, size_t* nr_shots, size_t* ncols, int* precision)
{
    return guarded([&] {
        need(s, "state");
        if (nr_bits) *nr_bits = s->nbits;
        if (nr_shots) *nr_shots = s->nshots;
        if (ncols) *ncols = s->ncols;
        if (precision) *precision = s->prec;
    });
}

int q1g_state_counts(const q1g_state* s, uint64_t* out, size_t len)
{
    return guarded([&] {
        need(s, "state");
        need(out, "out");
        if (len < s->counts.size()) throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "counts buffer too small");
        std::copy(s->counts.begin(), s->counts.end(), out);
    });
}

int q1g_state_download(q1g_state* s, double* out, size_t len)
{
    return guarded([&] {
        need(s, "state");
        need(out, "out");
        s->download(out, len);
    });
}

int q1g_state_compare(q1g_state* a, q1g_state* b, double* out5)
{
    return guarded([&] {
        need(a, "a");
        need(b, "b");
        need(out5, "out5");
        if (a->nbits != b->nbits || a->ncols != b->ncols)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "states differ in shape");
        a->ensure_dense();
        b->ensure_dense();
        a->settle_norms();
        b->settle_norms();
        b->sync();
        const uint64_t n = a->ncols * a->N;
        const uint64_t want = (n + 255) / 256;
        const unsigned blocks = (unsigned)std::min<uint64_t>(want ? want : 1, 152 * 16);
        DevBuf part;
        part.ensure(6 * blocks * sizeof(double));
        std::vector<double> h(6 * blocks);
        auto pass = [&](double wa, double wb, double* sums, double* mx) {
            check_cuda(launch_compare(a->amps.p, a->prec, b->amps.p, b->prec, n, wa, wb, part.as<double>(), blocks,
                                      a->stream),
                       "compare");
            a->d2h(h.data(), part.p, h.size() * sizeof(double), "download compare");
            a->sync();
            for (int k = 0; k < 5; ++k) sums[k] = 0.0;
            *mx = 0.0;
            for (unsigned i = 0; i < blocks; ++i) {
                for (int k = 0; k < 5; ++k) sums[k] += h[6 * i + k];
                *mx = std::max(*mx, h[6 * i + 5]);
            }
        };
        double s[5], mx = 0.0, s2[5], mx2 = 0.0;
        pass(1.0, 1.0, s, &mx);
        // second pass: total variation between the normalised distributions
        pass(1.0 / s[0], 1.0 / s[1], s2, &mx2);
        s[4] = s2[4];
        out5[0] = mx;
        out5[1] = 1.0 - (s[2] * s[2] + s[3] * s[3]) / (s[0] * s[1]);
        out5[2] = 0.5 * s[4];
        out5[3] = s[0];
        out5[4] = s[1];
    });
}

int q1g_apply_gate(q1g_state* s, const double* mat, size_t k, const size_t* bits, size_t nbits)
{
    return guarded([&] {
        need(s, "state");
        need(mat, "mat");
        if (nbits) need(bits, "bits");
        s->apply_gate(mat, k, bits, nbits);
    });
}

int q1g_apply_unary_gate_all(q1g_state* s, const double* mat)
{
    return guarded([&] {
        need(s, "state");
        need(mat, "mat");
        s->apply_unary_all(mat);
    });
}

int q1g_apply_conditional_gate(q1g_state* s, const uint8_t* control, size_t ncontrol, const double* mat,
                               size_t k, const size_t* bits, size_t nbits)
{
    return guarded([&] {
        need(s, "state");
        need(mat, "mat");
        if (ncontrol) need(control, "control");
        if (nbits) need(bits, "bits");
        s->apply_conditional(control, ncontrol, mat, k, bits, nbits);
    });
}

int q1g_measure_into(q1g_state* s, size_t qbit, size_t cbit, uint64_t* res, size_t res_len,
                     const double* uniforms, size_t n_uniforms, q1g_rng* rng)
{
    return guarded([&] {
        need(s, "state");
        if (res_len) need(res, "res");
        s->measure(qbit, cbit, res, res_len, uniforms, n_uniforms, rng, true);
    });
}

int q1g_peek_into(q1g_state* s, size_t qbit, size_t cbit, uint64_t* res, size_t res_len,
                  const double* uniforms, size_t n_uniforms, q1g_rng* rng)
{
    return guarded([&] {
        need(s, "state");
        if (res_len) need(res, "res");
        s->measure(qbit, cbit, res, res_len, uniforms, n_uniforms, rng, false);
    });
}

int q1g_measure_all_into(q1g_state* s, const size_t* cbits, size_t ncbits, uint64_t* res, size_t res_len,
                         const double* uniforms, size_t n_uniforms, q1g_rng* rng)
{
    return guarded([&] {
        need(s, "state");
        if (ncbits) need(cbits, "cbits");
        if (res_len) need(res, "res");
        s->measure_all(cbits, ncbits, res, res_len, uniforms, n_uniforms, rng, true);
    });
}

int q1g_peek_all_into(q1g_state* s, const size_t* cbits, size_t ncbits, uint64_t* res, size_t res_len,
                      const double* uniforms, size_t n_uniforms, q1g_rng* rng)
{
    return guarded([&] {
        need(s, "state");
        if (ncbits) need(cbits, "cbits");
        if (res_len) need(res, "res");
        s->measure_all(cbits, ncbits, res, res_len, uniforms, n_uniforms, rng, false);
    });
}

int q1g_reset(q1g_state* s, size_t bit, const double* uniforms, size_t n_uniforms, q1g_rng* rng)
{
    return guarded([&] {
        need(s, "state");
        std::vector<uint64_t> m(s->nshots, 0);
        s->measure(bit, 0, m.data(), m.size(), uniforms, n_uniforms, rng, true);
        std::vector<uint8_t> control(s->nshots);
        for (size_t r = 0; r < m.size(); ++r) control[r] = m[r] != 0;
        static const double xmat[8] = {0, 0, 1, 0, 1, 0, 0, 0};
        s->apply_conditional(control.data(), control.size(), xmat, 1, &bit, 1);
    });
}

int q1g_reset_all(q1g_state* s)
{
    return guarded([&] {
        need(s, "state");
        s->reset_all();
    });
}

int q1g_plan_create(size_t nr_bits, size_t ngates, const size_t* ks, const size_t* bits_flat, int fusion_width,
                    q1g_plan** out)
{
    return guarded([&] {
        need(out, "out");
        if (ngates) {
            need(ks, "ks");
            need(bits_flat, "bits_flat");
        }
        if (fusion_width < 0 || fusion_width > 5)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "fusion_width must be in 0..5");
        auto* p = new q1g_plan();
        p->nbits = (int)nr_bits;
        p->width = fusion_width;
        size_t bo = 0;
        for (size_t g = 0; g < ngates; ++g) {
            std::vector<int> b(ks[g]);
            for (size_t j = 0; j < ks[g]; ++j) {
                if (bits_flat[bo + j] >= nr_bits) {
                    delete p;
                    throw Error(Q1G_ERR_INVALID_QBIT, "Invalid qubit index " + std::to_string(bits_flat[bo + j]),
                                bits_flat[bo + j]);
                }
                b[j] = (int)bits_flat[bo + j];
            }
            bo += ks[g];
            p->mat_off.push_back(p->mat_doubles);
            p->mat_doubles += 2 * (size_t(1) << (2 * ks[g]));
            p->gate_bits.push_back(b);
        }
        if (fusion_width > 0) {
            p->blocks = fuse(p->gate_bits, (int)nr_bits, fusion_width);
            order_blocks_for_tc_pairs(p->blocks, (int)nr_bits, p->tc_max_high, p->tc_pairs == 5 ? 3 : 2);
        } else {
            for (size_t g = 0; g < ngates; ++g) {
                FusedBlock b;
                b.qubits = p->gate_bits[g];
                b.gates = {(int)g};
                p->blocks.push_back(b);
            }
        }
        *out = p;
    });
}

void q1g_plan_free(q1g_plan* p) { delete p; }

int q1g_plan_info(const q1g_plan* p, size_t* ngates, size_t* nblocks)
{
    return guarded([&] {
        need(p, "plan");
        if (ngates) *ngates = p->gate_bits.size();
        if (nblocks) *nblocks = p->blocks.size();
    });
}

int q1g_plan_set_gate_kinds(q1g_plan* p, const unsigned char* kinds, size_t ngates)
{
    return guarded([&] {
        need(p, "plan");
        if (ngates) need(kinds, "kinds");
        if (ngates != p->gate_bits.size())
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "one kind per gate of the plan");
        for (size_t g = 0; g < ngates; ++g) {
            if (kinds[g] > Q1G_GATE_SWAP) throw Error(Q1G_ERR_INVALID_ARGUMENT, "unknown gate kind");
            if (kinds[g] == Q1G_GATE_SWAP && p->gate_bits[g].size() != 2)
                throw Error(Q1G_ERR_INVALID_ARGUMENT, "a swap acts on two qubits");
        }
        p->kinds.assign(kinds, kinds + ngates);
        if (p->width > 0) {
            p->blocks = fuse_runs(p->gate_bits, p->kinds, p->nbits, p->width);
            order_blocks_for_tc_pairs(p->blocks, p->nbits, p->tc_max_high, p->tc_pairs == 5 ? 3 : 2);
        }
        p->prefix_known = false;
        p->prefix_plan.reset();
    });
}

int q1g_plan_block(const q1g_plan* p, size_t i, size_t* qubits, size_t* nq, size_t* gates, size_t* ng)
{
    return guarded([&] {
        need(p, "plan");
        need(nq, "nq");
        need(ng, "ng");
        if (i >= p->blocks.size()) throw Error(Q1G_ERR_INVALID_ARGUMENT, "block index out of range");
        const auto& b = p->blocks[i];
        if (*nq < b.qubits.size() || *ng < b.gates.size())
            throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "block buffers too small");
        for (size_t j = 0; j < b.qubits.size(); ++j) qubits[j] = (size_t)b.qubits[j];
        for (size_t j = 0; j < b.gates.size(); ++j) gates[j] = (size_t)b.gates[j];
        *nq = b.qubits.size();
        *ng = b.gates.size();
    });
}

int q1g_plan_block_matrix(const q1g_plan* p, size_t i, const double* mats_flat, size_t n_doubles, double* out,
                          size_t* n_out)
{
    return guarded([&] {
        need(p, "plan");
        need(n_out, "n_out");
        if (n_doubles) need(mats_flat, "mats_flat");
        if (i >= p->blocks.size()) throw Error(Q1G_ERR_INVALID_ARGUMENT, "block index out of range");
        if (n_doubles != p->mat_doubles)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "expected " + std::to_string(p->mat_doubles) + " matrix doubles");
        const auto& b = p->blocks[i];
        if (b.phase_run || b.qubits.size() > 10)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "a phase-run block has no dense matrix");
        const size_t dim = size_t(1) << b.qubits.size();
        if (*n_out < 2 * dim * dim) throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "output buffer too small");
        need(out, "out");
        std::vector<q1g::SeqGate> gates(p->gate_bits.size());
        for (int gi : b.gates) {
            const size_t gd = size_t(1) << p->gate_bits[gi].size();
            gates[gi].bits = p->gate_bits[gi];
            gates[gi].mat.resize(gd * gd);
            const double* m = mats_flat + p->mat_off[gi];
            for (size_t e = 0; e < gd * gd; ++e) gates[gi].mat[e] = q1g::cd(m[2 * e], m[2 * e + 1]);
        }
        const auto mat = q1g::block_matrix(b, gates);
        for (size_t e = 0; e < mat.size(); ++e) {
            out[2 * e] = mat[e].real();
            out[2 * e + 1] = mat[e].imag();
        }
        *n_out = 2 * dim * dim;
    });
}

int q1g_plan_set_tc_tiling(q1g_plan* p, int allow_pairs, int max_high_positions, int conflict_slack)
{
    return guarded([&] {
        need(p, "plan");
        if (max_high_positions < 0 || max_high_positions > 12)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "max_high_positions must be in 0..12");
        if (conflict_slack < 1 || conflict_slack > 64)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "conflict_slack must be in 1..64");
        if (allow_pairs < 0 || allow_pairs > 5)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "allow_pairs must be in 0..5", (uint64_t)allow_pairs);
        // the block order is made for the passes' size (three blocks in mode
        // 5): reorder the blocks when that changes
        const bool regroup = (allow_pairs == 5) != (p->tc_pairs == 5);
        p->tc_pairs = allow_pairs;
        p->tc_max_high = max_high_positions;
        p->tc_slack = conflict_slack;
        if (regroup) order_blocks_for_tc_pairs(p->blocks, p->nbits, p->tc_max_high, p->tc_pairs == 5 ? 3 : 2);
        // the compact prefix plan copies the tiling when it is made
        p->prefix_known = false;
        p->prefix_plan.reset();
    });
}

int q1g_plan_set_tensor_cores(q1g_plan* p, int enable)
{
    return guarded([&] {
        need(p, "plan");
        p->tensor_cores = enable != 0;
        p->prefix_known = false;
        p->prefix_plan.reset();
    });
}

int q1g_plan_run(q1g_plan* p, q1g_state* s, const double* mats_flat, size_t n_doubles)
{
    return guarded([&] {
        need(p, "plan");
        need(s, "state");
        if (n_doubles) need(mats_flat, "mats_flat");
        plan_run(p, s, mats_flat, n_doubles);
    });
}

int q1g_batch_create(int fusion_width, q1g_batch** out)
{
    return guarded([&] {
        need(out, "out");
        if (fusion_width < 1 || fusion_width > 4)
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "batch fusion_width must be in 1..4");
        auto* b = new q1g_batch();
        b->width = fusion_width;
        *out = b;
    });
}

void q1g_batch_free(q1g_batch* b) { delete b; }

int q1g_batch_add_circuit(q1g_batch* b, size_t nr_bits, size_t nr_shots, uint64_t seed, size_t nops,
                          const int* kinds, const size_t* nbits, const size_t* bits_flat, const double* mats_flat,
                          const size_t* args)
{
    return guarded([&] {
        need(b, "batch");
        if (nops) {
            need(kinds, "kinds");
            need(nbits, "nbits");
            need(args, "args");
        }
        batch_add_circuit(b, nr_bits, nr_shots, seed, nops, kinds, nbits, bits_flat, mats_flat, args);
    });
}

int q1g_batch_run(q1g_batch* b, uint64_t* results, size_t len)
{
    return guarded([&] {
        need(b, "batch");
        batch_run(b, results, len);
    });
}

int q1g_batch_info(const q1g_batch* b, size_t* ncircuits, size_t* total_runs, size_t* arena_bytes, size_t* nops,
                   double* last_ms)
{
    return guarded([&] {
        need(b, "batch");
        uint64_t runs = 0;
        for (const auto& c : b->circuits) runs += c.nshots;
        if (ncircuits) *ncircuits = b->circuits.size();
        if (total_runs) *total_runs = runs;
        if (arena_bytes) {
            uint64_t amps = 0;
            for (const auto& c : b->circuits) amps += 2 * (uint64_t(1) << c.nbits);
            *arena_bytes = amps * sizeof(float2);
        }
        if (nops) *nops = b->ops.size();
        if (last_ms) *last_ms = b->last_ms;
    });
}

int q1g_batch_traffic(const q1g_batch* b, uint64_t* bytes)
{
    return guarded([&] {
        need(b, "batch");
        need(bytes, "bytes");
        *bytes = b->last_traffic;
    });
}

int q1g_sample_shots_noalloc(const void* d_amps, int precision, size_t nr_bits, const double* d_sorted_uniforms,
                             size_t nshots, uint64_t* d_outcomes, uint64_t* d_words, const size_t* cbits,
                             void* cuda_stream)
{
    return guarded([&] {
        sample_shots_noalloc(d_amps, precision, nr_bits, d_sorted_uniforms, nshots, d_outcomes, d_words, cbits,
                             (cudaStream_t)cuda_stream);
    });
}

int q1g_histogram(const uint64_t* words, size_t n, uint64_t* keys, uint64_t* counts, size_t capacity,
                  size_t* nkeys, void* cuda_stream)
{
    return guarded([&] {
        need(nkeys, "nkeys");
        if (n) {
            need(words, "words");
            need(keys, "keys");
            need(counts, "counts");
        }
        histogram_words(words, n, keys, counts, capacity, nkeys, (cudaStream_t)cuda_stream);
    });
}

int q1g_profile_enable(q1g_state* s, int enable)
{
    return guarded([&] {
        need(s, "state");
        s->prof = enable != 0;
    });
}

int q1g_profile_report(q1g_state* s, char* names, uint64_t* launches, double* ms, double* bytes, size_t* n)
{
    return guarded([&] {
        need(s, "state");
        need(n, "n");
        s->collect_profile();
        size_t i = 0;
        for (const auto& kv : s->totals) {
            if (i >= *n) break;
            if (names) {
                std::memset(names + 32 * i, 0, 32);
                std::strncpy(names + 32 * i, kv.first.c_str(), 31);
            }
            if (launches) launches[i] = kv.second.launches;
            if (ms) ms[i] = kv.second.ms;
            if (bytes) bytes[i] = kv.second.bytes;
            ++i;
        }
        *n = i;
    });
}

int q1g_profile_reset(q1g_state* s)
{
    return guarded([&] {
        need(s, "state");
        s->collect_profile();
        s->totals.clear();
    });
}

int q1g_state_column_norms(q1g_state* s, double* out, size_t len)
{
    return guarded([&] {
        need(s, "state");
        if (len) need(out, "out");
        if (len < s->ncols) throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "norms buffer too small", len, s->ncols);
        s->settle_norms();
        const std::vector<double> v = s->measure_norms();
        std::copy(v.begin(), v.end(), out);
    });
}

int q1g_state_device_amplitudes(q1g_state* s, void** ptr, size_t* bytes)
{
    return guarded([&] {
        need(s, "state");
        need(ptr, "ptr");
        s->ensure_dense();
        s->settle_norms();
        s->sync();
        *ptr = s->amps.p;
        if (bytes) *bytes = s->total() * s->bsz();
    });
}

int q1g_state_amplitudes_written(q1g_state* s)
{
    return guarded([&] {
        need(s, "state");
        if (s->sparse) throw Error(Q1G_ERR_INVALID_ARGUMENT, "the state has no dense amplitudes to write");
        s->norm_pending = false;
        s->norms = s->measure_norms();
    });
}

int q1g_state_fill_random_normal(q1g_state* s, uint64_t seed)
{
    return guarded([&] {
        need(s, "state");
        s->fill_random_normal(seed);
    });
}

int q1g_state_set_wait_limit(q1g_state* s, double seconds)
{
    return guarded([&] {
        need(s, "state");
        if (!(seconds > 0.0)) {
            s->tc_wait_ns = 0;
        } else {
            const double ns = seconds * 1e9;
            s->tc_wait_ns = ns < 1.0 ? 1 : (ns > 3.6e12 ? (uint64_t)3.6e12 : (uint64_t)ns);
        }
    });
}

int q1g_state_transfer_bytes(q1g_state* s, uint64_t* h2d, uint64_t* d2h, int reset)
{
    return guarded([&] {
        need(s, "state");
        // the compact state that runs a plan's leading blocks counts apart
        uint64_t in = 0, out = 0;
        for (q1g_state* x = s; x; x = x->compact.get()) {
            in += x->h2d_bytes;
            out += x->d2h_bytes;
            if (reset) x->h2d_bytes = x->d2h_bytes = 0;
        }
        if (h2d) *h2d = in;
        if (d2h) *d2h = out;
    });
}

}  // extern "C"
