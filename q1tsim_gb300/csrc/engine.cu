// Device-resident VectorState: the host runtime behind the C ABI.
//
// Semantics follow q1tsim's VectorState (src/vectorstate.rs:24-416) column by
// column; only the representation changes: columns are contiguous in HBM,
// collapsed basis columns are kept as indices, and every amplitude pass is
// one of the kernels in gate_kernels.cu / state_kernels.cu / measure_kernels.cu.
#include "engine.h"

#include <algorithm>
#include <memory>
#include <set>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace q1g {

void check_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    const int code = (e == cudaErrorMemoryAllocation) ? Q1G_ERR_OUT_OF_MEMORY : Q1G_ERR_DEVICE;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

void DevBuf::ensure(size_t b)
{
    if (b <= bytes) return;
    release();
    if (b == 0) return;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(Q1G_ERR_OUT_OF_MEMORY,
                    "device allocation of " + std::to_string(b) + " bytes failed: " + cudaGetErrorString(e));
    }
    p = q;
    bytes = b;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

void HostBuf::ensure(size_t b)
{
    if (b <= bytes) return;
    release();
    if (b == 0) return;
    void* q = nullptr;
    cudaError_t e = cudaMallocHost(&q, b);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(Q1G_ERR_OUT_OF_MEMORY, "pinned host allocation failed");
    }
    p = q;
    bytes = b;
}

void HostBuf::release()
{
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
}

namespace {

uint64_t splitmix_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

}  // namespace

double stream_uniform_host(uint64_t seed, uint64_t counter)
{
    const uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    return (double)(splitmix_mix(z) >> 11) * (1.0 / 9007199254740992.0);
}

// Smallest k with CDF(k) > u, pmf in log space from 40 sigma below the mean.
// Stands in for rand_distr::Binomial (src/vectorstate.rs:271, 379).
uint64_t binomial_inv(uint64_t n, double p, double u)
{
    if (n == 0 || p <= 0.0) return 0;
    if (p >= 1.0) return n;
    const double nn = (double)n;
    const double mean = nn * p;
    const double sd = std::sqrt(nn * p * (1.0 - p));
    const double lo_d = std::floor(mean - 40.0 * sd - 40.0);
    const double hi_d = std::ceil(mean + 40.0 * sd + 40.0);
    const uint64_t lo = lo_d < 0.0 ? 0 : (uint64_t)lo_d;
    const uint64_t hi = hi_d > nn ? n : (uint64_t)hi_d;
    const double lp = std::log(p), lq = std::log1p(-p);
    const double lnf = std::lgamma(nn + 1.0);
    double cdf = 0.0;
    for (uint64_t k = lo; k <= hi; ++k) {
        const double kk = (double)k;
        const double lpmf = lnf - std::lgamma(kk + 1.0) - std::lgamma(nn - kk + 1.0) + kk * lp + (nn - kk) * lq;
        cdf += std::exp(lpmf);
        if (u < cdf) return k;
    }
    return hi;
}

}  // namespace q1g

using namespace q1g;

q1g_state::q1g_state(int nbits_, uint64_t nshots_, int prec_)
    : nbits(nbits_), nshots(nshots_), prec(prec_), N(uint64_t(1) << nbits_), ncols(1),
      counts{nshots_}
{
    check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    own_stream = true;
}

q1g_state::q1g_state(int nbits_, uint64_t nshots_, int prec_, cudaStream_t shared)
    : nbits(nbits_), nshots(nshots_), prec(prec_), N(uint64_t(1) << nbits_), ncols(1), counts{nshots_},
      stream(shared), own_stream(false)
{
}

q1g_state::~q1g_state()
{
    compact.reset();   // it runs on this state's stream: free it while the stream exists
    unary_plan.reset();
    if (stream) cudaStreamSynchronize(stream);
    for (auto& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    if (own_stream && stream) cudaStreamDestroy(stream);
}

void q1g_state::sync()
{
    check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
}

void q1g_state::collect_profile()
{
    if (pending.empty()) return;
    sync();
    for (auto& p : pending) {
        float ms = 0.f;
        check_cuda(cudaEventElapsedTime(&ms, p.a, p.b), "cudaEventElapsedTime");
        auto& t = totals[p.name];
        t.launches += 1;
        t.ms += ms;
        t.bytes += p.bytes;
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    pending.clear();
}

void q1g_state::ensure_dense()
{
    if (!sparse) return;
    amps.ensure(ncols * N * bsz());
    uscratch.ensure(ncols * sizeof(uint64_t));
    h2d(uscratch.p, basis.data(), ncols * sizeof(uint64_t), "upload basis");
    launch("fill_basis", double(ncols * N * bsz()), [&] {
        return launch_fill_basis(amps.p, prec, ncols * N, uscratch.as<uint64_t>(), ncols, N, stream);
    });
    // The basis list must stay alive until the copy ran: wait here.
    sync();
    sparse = false;
    basis.clear();
}

void q1g_state::apply_op(const GateOp& op, char* base, uint64_t total_amps)
{
    const double b2 = 2.0 * bsz();
    switch (op.kind) {
        case GateOp::Noop:
            return;
        case GateOp::Pair:
            launch(prec == kC128 ? (fp64_exact ? "pair_c128_fp64" : "pair_c128") : "pair_c64",
                   b2 * op.touched(total_amps), [&] {
                return launch_pair(base, prec, total_amps, op.map, op.o0, op.o1, op.m2, stream, fp64_exact);
            });
            return;
        case GateOp::Phase:
            launch(prec == kC128 ? (fp64_exact ? "phase_c128_fp64" : "phase_c128") : "phase_c64",
                   b2 * op.touched(total_amps), [&] {
                return launch_phase(base, prec, total_amps, op.map, op.ph[0], op.ph[1], stream, fp64_exact);
            });
            return;
        case GateOp::Dense: {
            const size_t d = size_t(1) << op.t;
            std::vector<double> hm(2 * d * d);
            for (size_t e = 0; e < d * d; ++e) {
                hm[2 * e] = op.dense[e].real();
                hm[2 * e + 1] = op.dense[e].imag();
            }
            if (dense_tiled_applies(prec, nbits, op.t, op.map, fp64_exact)) {
                std::vector<unsigned char> img(dense_tiled_matrix_bytes(prec, op.t));
                dense_tiled_matrix(prec, op.t, hm.data(), img.data());
                matbuf.ensure(img.size());
                h2d(matbuf.p, img.data(), img.size(), "upload matrix");
                sync();
                launch(prec == kC128 ? "dense_tiled_c128" : "dense_tiled_c64", b2 * op.touched(total_amps), [&] {
                    return launch_dense_tiled(base, prec, total_amps, nbits, op.map, op.offs, op.t, matbuf.p,
                                              sm_count(), stream);
                });
                return;
            }
            if (prec == kC64) {
                std::vector<float> hf(hm.begin(), hm.end());
                matbuf.ensure(hf.size() * sizeof(float));
                h2d(matbuf.p, hf.data(), hf.size() * sizeof(float), "upload matrix");
                sync();
            } else {
                matbuf.ensure(hm.size() * sizeof(double));
                h2d(matbuf.p, hm.data(), hm.size() * sizeof(double), "upload matrix");
                sync();
            }
            launch(prec == kC128 ? "dense_c128" : "dense_c64", b2 * op.touched(total_amps), [&] {
                return launch_dense(base, prec, total_amps, op.map, op.offs, op.t, matbuf.p, stream);
            });
            return;
        }
    }
}

static void check_gate_bits(int nbits, size_t k, const size_t* bits, size_t nbits_given)
{
    if (nbits_given != k)
        throw Error(Q1G_ERR_INVALID_NR_BITS,
                    "Expected " + std::to_string(k) + " bits for the gate, got " + std::to_string(nbits_given),
                    nbits_given, k);
    for (size_t m = 0; m < nbits_given; ++m)
        if (bits[m] >= (size_t)nbits)
            throw Error(Q1G_ERR_INVALID_QBIT, "Invalid qubit index " + std::to_string(bits[m]), bits[m]);
    for (size_t m = 0; m < nbits_given; ++m)
        for (size_t j = m + 1; j < nbits_given; ++j)
            if (bits[m] == bits[j])
                throw Error(Q1G_ERR_INVALID_ARGUMENT, "qubit " + std::to_string(bits[m]) + " given twice");
}

static GateOp classify_host(const double* mat, size_t k, const size_t* bits, int nbits)
{
    const size_t dim = size_t(1) << k;
    std::vector<cd> m(dim * dim);
    for (size_t e = 0; e < dim * dim; ++e) m[e] = cd(mat[2 * e], mat[2 * e + 1]);
    std::vector<int> b(k);
    for (size_t j = 0; j < k; ++j) b[j] = (int)bits[j];
    return classify(m.data(), (int)k, b.data(), nbits);
}

void q1g_state::apply_gate(const double* mat, size_t k, const size_t* bits, size_t nbits_given)
{
    check_gate_bits(nbits, k, bits, nbits_given);
    const GateOp op = classify_host(mat, k, bits, nbits);
    if (op.kind == GateOp::Noop) return;
    ensure_dense();
    apply_op(op, amps.as<char>(), total());
}

// src/vectorstate.rs:180-189: the same one-qubit gate on every qubit.  The
// reference makes one pass per qubit.  The gates act on different qubits, so
// they commute and fuse into blocks of up to five qubits (complex64: one
// tensor-core pass per block, 6 passes at 30 qubits) or three (complex128:
// double-float warp tiles).  With FP64 arithmetic requested, the gates run
// one by one, as the reference rounds.
void q1g_state::apply_unary_all(const double* mat)
{
    using namespace q1g;
    if (fp64_exact || nbits < 2) {
        for (size_t b = 0; b < (size_t)nbits; ++b) apply_gate(mat, 1, &b, 1);
        return;
    }
    const int width = prec == kC64 ? 5 : 3;
    if (!unary_plan || unary_plan->nbits != nbits || unary_plan->width != width) {
        auto p = std::make_unique<q1g_plan>();
        p->nbits = nbits;
        p->width = width;
        for (int q = 0; q < nbits; ++q) {
            p->mat_off.push_back(p->mat_doubles);
            p->mat_doubles += 8;
            p->gate_bits.push_back({q});
        }
        p->blocks = fuse(p->gate_bits, nbits, width);
        order_blocks_for_tc_pairs(p->blocks, nbits, p->tc_max_high, p->tc_pairs == 5 ? 3 : 2);
        unary_plan = std::move(p);
    }
    std::vector<double> mats(8 * (size_t)nbits);
    for (int q = 0; q < nbits; ++q) std::copy(mat, mat + 8, mats.begin() + 8 * (size_t)q);
    plan_run(unary_plan.get(), this, mats.data(), mats.size());
}

// Every column becomes a random unit vector: re and im of each amplitude
// i.i.d. N(0,1) (column c takes amplitudes c*N .. c*N+N-1 of the stream),
// then normalised -- the column rescale that settles pending norms.
void q1g_state::fill_random_normal(uint64_t seed)
{
    using namespace q1g;
    const uint64_t t = total();
    amps.ensure(t * bsz());
    launch("random_normal", double(t * bsz()),
           [&] { return launch_random_normal(amps.p, prec, t, seed, stream); });
    sparse = false;
    basis.clear();
    norms.assign(ncols, 1.0);
    norm_pending = true;
    settle_norms();
}

// src/qustate.rs:100-127: (column, length, apply) runs of equal control bits.
struct CondRange {
    uint64_t col, len;
    bool apply;
};

static std::vector<CondRange> conditional_ranges(const std::vector<uint64_t>& counts,
                                                 const uint8_t* control)
{
    std::vector<CondRange> r;
    uint64_t off = 0;
    for (uint64_t c = 0; c < counts.size(); ++c) {
        const uint64_t count = counts[c];
        if (count == 0) continue;
        uint64_t begin = off;
        bool prev = control[off] != 0;
        for (uint64_t ib = off + 1; ib < off + count; ++ib) {
            const bool cur = control[ib] != 0;
            if (cur != prev) {
                r.push_back({c, ib - begin, prev});
                begin = ib;
                prev = cur;
            }
        }
        if (begin < off + count) r.push_back({c, off + count - begin, prev});
        off += count;
    }
    return r;
}

void q1g_state::apply_conditional(const uint8_t* control, size_t ncontrol, const double* mat,
                                  size_t k, const size_t* bits, size_t nbits_given)
{
    settle_norms();
    if (ncontrol != nshots)
        throw Error(Q1G_ERR_INVALID_NR_CONTROL_BITS,
                    "Expected " + std::to_string(nshots) + " control bits, got " + std::to_string(ncontrol), ncontrol,
                    nshots);
    check_gate_bits(nbits, k, bits, nbits_given);
    const GateOp op = classify_host(mat, k, bits, nbits);
    const auto ranges = conditional_ranges(counts, control);
    bool same_layout = ranges.size() == ncols;
    for (size_t j = 0; same_layout && j < ranges.size(); ++j) same_layout = ranges[j].col == j;
    if (same_layout && op.kind == GateOp::Noop) return;
    ensure_dense();
    if (!same_layout) {
        const uint64_t nr = ranges.size();
        std::vector<CollapseCol> cols(nr);
        for (uint64_t j = 0; j < nr; ++j) cols[j] = {ranges[j].col, -1, 1.0};
        spare.ensure(nr * N * bsz());
        colbuf.ensure(nr * sizeof(CollapseCol));
        h2d(colbuf.p, cols.data(), nr * sizeof(CollapseCol), "upload columns");
        launch("column_copy", 2.0 * nr * N * bsz(), [&] {
            return launch_collapse_copy(spare.p, amps.p, prec, N, 0, colbuf.as<CollapseCol>(), nr, stream);
        });
        sync();
        amps.swap(spare);
        if (spare.bytes > (size_t(1) << 30)) spare.release();
        ncols = nr;
    }
    if (!same_layout) {
        std::vector<double> nn(ranges.size());
        for (size_t j = 0; j < ranges.size(); ++j) nn[j] = norms[ranges[j].col];
        norms.swap(nn);
    }
    counts.resize(ranges.size());
    for (size_t j = 0; j < ranges.size(); ++j) counts[j] = ranges[j].len;
    for (size_t j = 0; j < ranges.size(); ++j)
        if (ranges[j].apply) apply_op(op, col_ptr(j), N);
}

std::vector<double> q1g_state::zero_weights(size_t qbit)
{
    const int pos = nbits - 1 - (int)qbit;
    std::vector<double> w0(ncols, 0.0);
    if (sparse) {
        for (uint64_t c = 0; c < ncols; ++c) w0[c] = ((basis[c] >> pos) & 1) ? 0.0 : 1.0;
        return w0;
    }
    IndexMap m{};
    m.nz = 1;
    m.zpos[0] = pos;
    m.setmask = 0;
    const uint64_t half = N / 2;
    const uint64_t chunk = std::min<uint64_t>(half, 4096);
    const uint64_t nchunks = ncols * (half / chunk);
    const uint64_t ntmp = segment_sums_tmp_doubles(ncols, half / chunk);
    dscratch.ensure((nchunks + ncols + ntmp) * sizeof(double));
    double* d = dscratch.as<double>();
    launch("qubit_weights", double(ncols * half * bsz()), [&] {
        return launch_chunk_sums(amps.p, prec, ncols * half, chunk, m, d, stream);
    });
    check_cuda(launch_segment_sums(d, ncols, half / chunk, d + nchunks, d + nchunks + ncols, stream),
               "segment_sums");
    hstage.ensure(ncols * sizeof(double));
    d2h(hstage.p, d + nchunks, ncols * sizeof(double), "download weights");
    sync();
    std::memcpy(w0.data(), hstage.p, ncols * sizeof(double));
    return w0;
}

void q1g_state::measure(size_t qbit, size_t cbit, uint64_t* res, size_t res_len,
                        const double* uniforms, size_t nu, q1g_rng* rng, bool collapse)
{
    if (qbit >= (size_t)nbits) throw Error(Q1G_ERR_INVALID_QBIT, "Invalid qubit index " + std::to_string(qbit), qbit);
    settle_norms();     // P(0) is the half's weight against the column's norm
    if (res_len < nshots)
        throw Error(Q1G_ERR_NOT_ENOUGH_SPACE,
                    "Unable to store " + std::to_string(nshots) + " measurements in array of size " +
                        std::to_string(res_len),
                    res_len, nshots);
    if (cbit >= 64) throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit index " + std::to_string(cbit), cbit);
    if (uniforms ? nu < ncols : rng == nullptr)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "need one uniform per state column or an rng");
    std::vector<double> us(ncols);
    for (uint64_t c = 0; c < ncols; ++c)
        us[c] = uniforms ? uniforms[c] : stream_uniform_host(rng->seed, rng->counter++);
    const std::vector<double> w0 = zero_weights(qbit);
    std::vector<uint64_t> n0(ncols);
    uint64_t new_nr = 0;
    for (uint64_t c = 0; c < ncols; ++c) {
        n0[c] = binomial_inv(counts[c], std::min(w0[c], 1.0), us[c]);
        new_nr += (n0[c] == 0 || n0[c] == counts[c]) ? 1 : 2;
    }
    // results: first n0 runs of a column read 0, the rest 1 (src/vectorstate.rs:290-297)
    const uint64_t one = uint64_t(1) << cbit;
    uint64_t rs = 0;
    for (uint64_t c = 0; c < ncols; ++c) {
        for (uint64_t r = rs; r < rs + n0[c]; ++r) res[r] &= ~one;
        for (uint64_t r = rs + n0[c]; r < rs + counts[c]; ++r) res[r] |= one;
        rs += counts[c];
    }
    if (!collapse) return;
    // collapse (src/vectorstate.rs:299-322, 91-104)
    std::vector<CollapseCol> cols;
    std::vector<uint64_t> nc;
    std::vector<uint64_t> nbasis;
    cols.reserve(new_nr);
    for (uint64_t c = 0; c < ncols; ++c) {
        const double w = w0[c];
        if (n0[c] == counts[c]) {
            cols.push_back({c, 0, 1.0 / std::sqrt(w)});
            nc.push_back(counts[c]);
        } else if (n0[c] == 0) {
            cols.push_back({c, 1, 1.0 / std::sqrt(1.0 - w)});
            nc.push_back(counts[c]);
        } else {
            cols.push_back({c, 0, 1.0 / std::sqrt(w)});
            nc.push_back(n0[c]);
            cols.push_back({c, 1, 1.0 / std::sqrt(1.0 - w)});
            nc.push_back(counts[c] - n0[c]);
        }
    }
    if (sparse) {
        // basis columns are unchanged by their own (certain) outcome
        counts = nc;
        return;
    }
    norms.assign(new_nr, 1.0);
    const int pos = nbits - 1 - (int)qbit;
    const bool split = new_nr != ncols;
    colbuf.ensure(new_nr * sizeof(CollapseCol));
    h2d(colbuf.p, cols.data(), new_nr * sizeof(CollapseCol), "upload columns");
    if (!split) {
        launch("collapse", 2.0 * ncols * N * bsz(), [&] {
            return launch_collapse_copy(amps.p, amps.p, prec, N, pos, colbuf.as<CollapseCol>(), new_nr, stream);
        });
    } else {
        spare.ensure(new_nr * N * bsz());
        launch("collapse", double(new_nr + ncols) * N * bsz(), [&] {
            return launch_collapse_copy(spare.p, amps.p, prec, N, pos, colbuf.as<CollapseCol>(), new_nr, stream);
        });
    }
    sync();
    if (split) {
        amps.swap(spare);
        if (spare.bytes > (size_t(1) << 30)) spare.release();
    }
    ncols = new_nr;
    counts = nc;
}

void q1g_state::measure_all(const size_t* cbits, size_t ncbits, uint64_t* res, size_t res_len,
                            const double* uniforms, size_t nu, q1g_rng* rng, bool collapse)
{
    if (res_len < nshots)
        throw Error(Q1G_ERR_NOT_ENOUGH_SPACE,
                    "Unable to store " + std::to_string(nshots) + " measurements in array of size " +
                        std::to_string(res_len),
                    res_len, nshots);
    if (ncbits != (size_t)nbits)
        throw Error(Q1G_ERR_INVALID_NR_MEASUREMENT_BITS,
                    "Expected " + std::to_string(nbits) + " measurement bits, got " + std::to_string(ncbits), ncbits,
                    nbits);
    for (size_t q = 0; q < ncbits; ++q)
        if (cbits[q] >= 64)
            throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit index " + std::to_string(cbits[q]), cbits[q]);
    if (uniforms ? nu < nshots : rng == nullptr)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "need one uniform per run or an rng");
    uint64_t mask = 0;
    std::vector<uint64_t> cbit_of_pos(64, 0);
    for (size_t q = 0; q < ncbits; ++q) {
        mask |= uint64_t(1) << cbits[q];
        cbit_of_pos[nbits - 1 - q] = uint64_t(1) << cbits[q];
    }
    mask = ~mask;
    auto word_of = [&](uint64_t idx) {
        uint64_t w = 0;
        for (int p = 0; p < nbits; ++p)
            if ((idx >> p) & 1) w |= cbit_of_pos[p];
        return w;
    };

    // per-run outcome indices: the pinned download of the dense sampler, or
    // the basis columns of a sparse state
    std::vector<uint64_t> outc;
    const uint64_t* h_outc = nullptr;
    if (sparse) {
        outc.resize(nshots);
        h_outc = outc.data();
        uint64_t off = 0;
        for (uint64_t c = 0; c < ncols; ++c) {
            for (uint64_t r = 0; r < counts[c]; ++r) outc[off + r] = basis[c];
            if (!uniforms) rng->counter += counts[c] + 1;
            off += counts[c];
        }
        for (uint64_t r = 0; r < nshots; ++r) res[r] = (res[r] & mask) | word_of(outc[r]);
    } else if (nshots > 0) {
        const uint64_t chunk = std::min<uint64_t>(N, 256);
        const uint64_t ncc = N / chunk;  // chunks per column
        uint64_t mmax = 0;
        for (auto c : counts) mmax = std::max(mmax, c);
        const uint64_t scan_tmp = scan_tmp_doubles(ncc) + 1;
        const uint64_t spc_tmp = 2 * (mmax + 1) + scan_tmp_doubles(mmax + 1) + 1;
        const uint64_t nd = ncols * ncc + ncols + scan_tmp + nshots + spc_tmp;
        dscratch.ensure(nd * sizeof(double));
        double* d_sums = dscratch.as<double>();
        double* d_tot = d_sums + ncols * ncc;
        double* d_stmp = d_tot + ncols;
        double* d_u = d_stmp + scan_tmp;
        double* d_spc = d_u + nshots;
        uscratch.ensure((2 * nshots + 64 + nshots / 2 + 1) * sizeof(uint64_t));
        uint64_t* d_out = uscratch.as<uint64_t>();
        uint64_t* d_word = d_out + nshots;
        uint64_t* d_cpos = d_word + nshots;
        uint32_t* d_chunk = reinterpret_cast<uint32_t*>(d_cpos + 64);   // each shot's chunk
        h2d(d_cpos, cbit_of_pos.data(), 64 * sizeof(uint64_t), "upload cbits");
        launch("chunk_sums", double(ncols * N * bsz()), [&] {
            return launch_chunk_sums_dense(amps.p, prec, ncols * N, chunk, d_sums, stream);
        });
        for (uint64_t c = 0; c < ncols; ++c)
            launch("prefix_scan", 2.0 * ncc * sizeof(double), [&] {
                return launch_exclusive_scan(d_sums + c * ncc, ncc, d_stmp, d_tot + c, stream);
            });
        std::vector<double> hu;
        if (uniforms) {
            hu.assign(uniforms, uniforms + nshots);
            uint64_t off = 0;
            for (uint64_t c = 0; c < ncols; ++c) {
                std::sort(hu.begin() + off, hu.begin() + off + counts[c]);
                off += counts[c];
            }
            h2d(d_u, hu.data(), nshots * sizeof(double), "upload uniforms");
        } else {
            uint64_t off = 0;
            for (uint64_t c = 0; c < ncols; ++c) {
                const uint64_t m = counts[c];
                launch("sorted_uniforms", 0.0, [&] {
                    return launch_sorted_uniforms(rng->seed, rng->counter, m, d_u + off, d_spc, stream);
                });
                rng->counter += m + 1;
                off += m;
            }
        }
        uint64_t off = 0;
        for (uint64_t c = 0; c < ncols; ++c) {
            SampleArgs a{};
            a.amps = col_ptr(c);
            a.prec = prec;
            a.col_len = N;
            a.chunk = chunk;
            a.excl = d_sums + c * ncc;
            a.nchunks = ncc;
            a.total = d_tot + c;
            a.u = d_u + off;
            a.nruns = counts[c];
            a.outcome = d_out + off;
            a.word = d_word + off;
            a.nbits = nbits;
            a.d_cbit_of_pos = d_cpos;
            a.chunk_of = d_chunk + off;
            launch("sample", double(counts[c] * chunk * bsz()), [&] { return launch_sample(a, stream); });
            off += counts[c];
        }
        hstage.ensure(2 * nshots * sizeof(uint64_t));
        d2h(hstage.p, d_out, 2 * nshots * sizeof(uint64_t), "download outcomes");
        sync();
        h_outc = hstage.as<uint64_t>();
        if (!collapse) {
            const uint64_t* h_word = h_outc + nshots;
            for (uint64_t r = 0; r < nshots; ++r) res[r] = (res[r] & mask) | h_word[r];
            return;
        }
    }
    if (!collapse) return;
    // one basis column per distinct (column, outcome), in order: outcomes are
    // sorted within a column, so a column's distinct outcomes are its runs of
    // equal ones (about 10^6 at 30 qubits and 10^6 shots, two for a GHZ
    // state).  One pass writes the words and appends the runs to
    // basis/counts, whose capacity carries over between runs: no second
    // pass, and no zero fill of a resize.  The reservation is capped (2^20
    // entries, 8 MB each): many shots of few outcomes keep no large buffer,
    // and more distinct outcomes grow the vectors as they come.
    const uint64_t* h_word = sparse ? nullptr : h_outc + nshots;
    const std::vector<uint64_t> runs(counts.begin(), counts.end());
    basis.clear();
    counts.clear();
    basis.reserve(std::min<uint64_t>(nshots, uint64_t(1) << 20));
    counts.reserve(std::min<uint64_t>(nshots, uint64_t(1) << 20));
    uint64_t off = 0;
    for (uint64_t c = 0; c < runs.size(); ++c) {
        const uint64_t end = off + runs[c];
        for (uint64_t r = off; r < end; ++r) {
            if (h_word) res[r] = (res[r] & mask) | h_word[r];
            if (r == off || h_outc[r] != h_outc[r - 1]) {
                basis.push_back(h_outc[r]);
                counts.push_back(1);
            } else {
                ++counts.back();
            }
        }
        off = end;
    }
    sparse = true;
    norm_pending = false;
    ncols = basis.size();
    norms.assign(ncols, 1.0);
}

void q1g_state::reset_all()
{
    norm_pending = false;
    sparse = true;
    basis.assign(1, 0);
    counts.assign(1, nshots);
    ncols = 1;
    norms.assign(1, 1.0);
}

void q1g_state::download(double* out, size_t len)
{
    if (len < 2 * ncols * N)
        throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "download buffer too small");
    settle_norms();
    if (sparse) {
        std::memset(out, 0, 2 * ncols * N * sizeof(double));
        for (uint64_t c = 0; c < ncols; ++c) out[2 * (c * N + basis[c])] = 1.0;
        return;
    }
    const uint64_t n = ncols * N;
    if (prec == kC128) {
        d2h(out, amps.p, n * 16, "download");
        sync();
    } else {
        std::vector<float> tmp(2 * n);
        d2h(tmp.data(), amps.p, n * 8, "download");
        sync();
        for (uint64_t e = 0; e < 2 * n; ++e) out[e] = tmp[e];
    }
}

// ---------------------------------------------------------------- plans

q1g_plan::~q1g_plan()
{
    if (staged) {
        cudaEventSynchronize(staged);
        cudaEventDestroy(staged);
    }
}

namespace q1g {


static std::vector<int> positions_of(const std::vector<int>& qubits, int nbits)
{
    std::vector<int> p;
    for (int q : qubits) p.push_back(nbits - 1 - q);
    std::sort(p.begin(), p.end());
    return p;
}

// The tile of a pass: the blocks' positions plus the lowest other positions,
// 12 in all, ascending.
static std::vector<int> tile_positions(const std::vector<const std::vector<int>*>& bits, int nbits)
{
    std::vector<int> T;
    for (auto* b : bits)
        for (int p : positions_of(*b, nbits))
            if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
    for (int p = 0; (int)T.size() < 12 && p < nbits; ++p)
        if (std::find(T.begin(), T.end(), p) == T.end()) T.push_back(p);
    std::sort(T.begin(), T.end());
    return T;
}

// Tile bits 0..L-1 are positions 0..L-1: the tile is 2^(12-L) contiguous runs.
static int tile_run_bits(const std::vector<int>& T)
{
    int L = 0;
    while (L < (int)T.size() && T[L] == L) ++L;
    return L;
}

// Shortest contiguous run a pass may copy in pieces (2^7 amplitudes = 1 KB):
// at most 32 runs per tile.  Shorter runs need the tile to be one
// tensor-map box, unpadded.
constexpr int kMinTcRunBits = 7;
// Tile positions at or above this one are 2 MB (a large page) or more apart
// in complex64; a pair's tile may have q1g_plan::tc_max_high of them (8 by
// default: at most 256 large pages per tile; a tile over 512 ran 2.4x
// slower, one over 256 as fast as any).
constexpr int kHighPosition = 18;
// Shortest contiguous run (as a power of two of amplitudes) of a three-block
// pass's tile: 8 amplitudes, 64 bytes.
constexpr int kMinTripleRunBits = 3;

static TcPass lower_tc_pass(const std::vector<const std::vector<cd>*>& mats,
                            const std::vector<const std::vector<int>*>& bits, int nbits, uint64_t ncols, int slack,
                            int pair_mode)
{
    const bool shuffle = pair_mode == 2;
    TcPass t;
    const std::vector<int> T = tile_positions(bits, nbits);
    auto tbit = [&](int pos) { return (int)(std::find(T.begin(), T.end(), pos) - T.begin()); };
    t.tilemap.nz = 12;
    for (int j = 0; j < 12; ++j) t.tilemap.zpos[j] = T[j];
    t.tilemap.setmask = 0;
    const int L = tile_run_bits(T);
    t.box = tc_tile_box(T.data(), nbits, ncols);
    if (L < kMinTcRunBits && !t.box.usable)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "tensor-core tile with runs shorter than 128 amplitudes");
    t.offs.run_bits = (uint32_t)L;
    t.offs.nruns = 1u << (12 - L);
    for (uint32_t r = 0; r < t.offs.nruns && r < 32; ++r) {
        uint64_t o = 0;
        for (int b = L; b < 12; ++b)
            if ((r >> (b - L)) & 1) o |= uint64_t(1) << T[b];
        t.offs.run_off[r] = o;
    }
    t.offs.nblocks = (uint32_t)mats.size();
    t.images.assign(mats.size() * kTcImageHalves, 0);
    for (size_t bi = 0; bi < mats.size(); ++bi) {
        // gate qubits: the block's own, padded from the tile's highest positions
        std::vector<int> gpos = positions_of(*bits[bi], nbits);
        for (int j = 11; (int)gpos.size() < 5; --j)
            if (std::find(gpos.begin(), gpos.end(), T[j]) == gpos.end()) gpos.push_back(T[j]);
        std::vector<int> q;
        for (int p : gpos) q.push_back(nbits - 1 - p);
        std::sort(q.begin(), q.end());   // ascending qubits: q[0] is the matrix MSB
        const auto m32 = embed_matrix(*mats[bi], *bits[bi], q);
        std::vector<double> md(2 * 32 * 32);
        for (size_t e = 0; e < m32.size(); ++e) {
            md[2 * e] = m32[e].real();
            md[2 * e + 1] = m32[e].imag();
        }
        build_tc_image(md.data(), t.images.data() + bi * kTcImageHalves,
                       bi + 1 == mats.size() ? kTcLastBScaleLog2 : 0);
        TcBlockGeom& G = t.offs.blk[bi];
        int r = 0;
        for (int j = 0; j < 12; ++j)
            if (std::find(gpos.begin(), gpos.end(), T[j]) == gpos.end()) G.jrow_bit[r++] = 1u << j;
        for (int g = 0; g < 32; ++g) {
            uint32_t jc = 0;
            for (int j = 0; j < 5; ++j)
                if ((g >> (4 - j)) & 1) jc |= 1u << tbit(nbits - 1 - q[j]);
            G.jgate[g] = jc;
        }
        G.vec2 = G.jgate[1] == 1u ? 1u : 0u;
    }
    t.offs.shuffle = 0;
    int reg1[5];
    if (mats.size() == 2 && shuffle && tc_shuffle_layout(t.offs.blk[0], t.offs.blk[1], t.offs.swap_lane, reg1)) {
        // the second block takes the first block's results in registers:
        // its image in their order, matrix index bit k = tile bit reg1[k]
        t.offs.shuffle = 1;
        std::vector<int> q2(5);
        for (int k = 0; k < 5; ++k) q2[4 - k] = nbits - 1 - T[reg1[k]];
        const auto m32 = embed_matrix(*mats[1], *bits[1], q2);
        std::vector<double> md(2 * 32 * 32);
        for (size_t e = 0; e < m32.size(); ++e) {
            md[2 * e] = m32[e].real();
            md[2 * e + 1] = m32[e].imag();
        }
        build_tc_image(md.data(), t.images.data() + kTcImageHalves, kTcLastBScaleLog2);
    }
    // pair modes 4 and 5: the four-group kernel, every A operand in shared
    // memory (5: three blocks per pass where they fit)
    const bool quad = pair_mode >= 4;
    auto finish = [&] {
        if (!quad) return;
        t.offs.groups = 4;
        t.offs.stage_bytes = (t.offs.stage_bytes + 1023u) & ~1023u;
        // the first block's split is dealt to the threads by a map of its
        // own, in a gate order that map chooses: its image in that order
        int gbit0[5];
        tc_split_map(t.offs, gbit0);
        std::vector<int> q0(5);
        for (int k = 0; k < 5; ++k) q0[4 - k] = nbits - 1 - T[gbit0[k]];
        const auto m32 = embed_matrix(*mats[0], *bits[0], q0);
        std::vector<double> md(2 * 32 * 32);
        for (size_t e = 0; e < m32.size(); ++e) {
            md[2 * e] = m32[e].real();
            md[2 * e + 1] = m32[e].imag();
        }
        build_tc_image(md.data(), t.images.data(), mats.size() == 1 ? kTcLastBScaleLog2 : 0);
    };
    auto rebuild_image = [&](size_t bi, const int* gb) {
        // block bi in the gate order a layout chose: matrix index bit k =
        // tile bit gb[k]
        std::vector<int> qk(5);
        for (int k = 0; k < 5; ++k) qk[4 - k] = nbits - 1 - T[gb[k]];
        const auto m32 = embed_matrix(*mats[bi], *bits[bi], qk);
        std::vector<double> md(2 * 32 * 32);
        for (size_t e = 0; e < m32.size(); ++e) {
            md[2 * e] = m32[e].real();
            md[2 * e + 1] = m32[e].imag();
        }
        build_tc_image(md.data(), t.images.data() + bi * kTcImageHalves,
                       bi + 1 == mats.size() ? kTcLastBScaleLog2 : 0);
    };
    int gbits[kTcMaxBlocks][5];
    // store boxes for the last block's write-back (an unpadded one-box tile)
    std::vector<TcStoreBox> stores;
    if (quad && mats.size() >= 2 && t.box.usable)
        stores = tc_store_boxes(T.data(), nbits, ncols, t.offs.blk[mats.size() - 1].jgate[31]);
    int store = -1;
    if (quad && mats.size() >= 2 &&
        tc_chain_layout(t.offs, t.box.usable != 0, slack, gbits, &t.cost, &t.ideal, &stores, &store)) {
        if (t.offs.st_box) t.sbox = stores[(size_t)store].box;
        // the later blocks read the operands the previous block's
        // write-back scattered, in the gate orders the layout chose
        for (size_t bi = 1; bi < mats.size(); ++bi) rebuild_image(bi, gbits[bi]);
        finish();
        return t;
    }
    if (mats.size() > 2) throw Error(Q1G_ERR_INVALID_ARGUMENT, "a three-block pass needs the four-group kernel");
    int gbit1[5];
    if (mats.size() == 2 && (pair_mode == 3 || quad) && tc_direct_layout(t.offs, t.box.usable != 0, slack, gbit1)) {
        // the second block reads the operands the first block's write-back
        // scattered: its image in the gate order that layout chose, matrix
        // index bit k = tile bit gbit1[k]
        std::vector<int> q2(5);
        for (int k = 0; k < 5; ++k) q2[4 - k] = nbits - 1 - T[gbit1[k]];
        const auto m32 = embed_matrix(*mats[1], *bits[1], q2);
        std::vector<double> md(2 * 32 * 32);
        for (size_t e = 0; e < m32.size(); ++e) {
            md[2 * e] = m32[e].real();
            md[2 * e + 1] = m32[e].imag();
        }
        build_tc_image(md.data(), t.images.data() + kTcImageHalves, kTcLastBScaleLog2);
        finish();
        return t;
    }
    tc_choose_padding(t.offs, t.box.usable != 0, slack);
    finish();
    return t;
}

// Whether blocks on these qubit sets could share a tensor-core pass: their
// positions fit one 12-position tile, at most max_high of its positions lie
// at 2 MB strides or more, and the tile has runs of >= 128 amplitudes or is
// one tensor-map box (the rule plan_run applies, before any padding choice).
static bool tc_pairable(const std::vector<const std::vector<int>*>& qs, int nbits, int max_high)
{
    std::vector<int> u;
    for (auto* q : qs)
        for (int x : *q)
            if (std::find(u.begin(), u.end(), x) == u.end()) u.push_back(x);
    if (u.size() > 12 || nbits < 12) return false;
    const auto T = tile_positions(qs, nbits);
    int high = 0;
    for (int p : T) high += p >= kHighPosition;
    return high <= max_high && (tile_run_bits(T) >= kMinTcRunBits || tc_tile_box(T.data(), nbits, 1).usable);
}

void order_blocks_for_tc_pairs(std::vector<FusedBlock>& blocks, int nbits, int max_high, int group)
{
    // Blocks on disjoint qubits commute.  Take the earliest block whose
    // predecessors (the last earlier block on each of its qubits) are all
    // taken, then, while the pass has room (group blocks), the earliest
    // ready block that can share its tensor-core pass, so that plan_run
    // finds them next to each other.
    const int m = (int)blocks.size();
    if (m < 3 || nbits < 12) return;
    auto candidate = [&](int i) {
        return !blocks[i].phase_run && !blocks[i].swap_run && blocks[i].qubits.size() >= 3 &&
               blocks[i].qubits.size() <= 5;
    };
    std::vector<std::vector<int>> succ(m);
    std::vector<int> indeg(m, 0), last(nbits, -1);
    for (int j = 0; j < m; ++j) {
        std::vector<int> preds;
        for (int q : blocks[j].qubits) {
            if (last[q] >= 0 && std::find(preds.begin(), preds.end(), last[q]) == preds.end()) preds.push_back(last[q]);
            last[q] = j;
        }
        for (int i : preds) succ[i].push_back(j);
        indeg[j] = (int)preds.size();
    }
    std::set<int> ready;
    for (int j = 0; j < m; ++j)
        if (indeg[j] == 0) ready.insert(j);
    std::vector<int> order;
    auto take = [&](int j) {
        ready.erase(j);
        order.push_back(j);
        for (int k : succ[j])
            if (--indeg[k] == 0) ready.insert(k);
    };
    while (!ready.empty()) {
        const int a = *ready.begin();
        take(a);
        if (!candidate(a)) continue;
        std::vector<const std::vector<int>*> pass = {&blocks[a].qubits};
        while ((int)pass.size() < group) {
            int next = -1;
            for (int b : ready) {
                if (!candidate(b)) continue;
                pass.push_back(&blocks[b].qubits);
                const bool ok = tc_pairable(pass, nbits, max_high);
                pass.pop_back();
                if (ok) {
                    next = b;
                    break;
                }
            }
            if (next < 0) break;
            pass.push_back(&blocks[next].qubits);
            take(next);
        }
    }
    std::vector<FusedBlock> out;
    out.reserve(m);
    for (int j : order) out.push_back(std::move(blocks[j]));
    blocks.swap(out);
}

// A swap-run block (fuse_runs): every gate must be the swap permutation;
// one permutation pass (swap_run.cu), or the swaps one by one when the
// state has fewer than 10 qubits.
template <typename Stage>
static void run_swap_block(q1g_state* s, const FusedBlock& b, const std::vector<SeqGate>& gates, Stage&& stage)
{
    const int n = s->nbits;
    std::vector<int> pa, pb;
    for (int g : b.gates) {
        const SeqGate& q = gates[g];
        if (q.bits.size() != 2) throw Error(Q1G_ERR_INVALID_ARGUMENT, "a gate marked swap acts on two qubits");
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                const bool one = (r == c && (r == 0 || r == 3)) || (r == 1 && c == 2) || (r == 2 && c == 1);
                if (q.mat[4 * r + c] != cd(one ? 1.0 : 0.0, 0.0))
                    throw Error(Q1G_ERR_INVALID_ARGUMENT, "a gate marked swap is not the swap");
            }
        pa.push_back(n - 1 - q.bits[0]);
        pb.push_back(n - 1 - q.bits[1]);
    }
    auto t = std::make_unique<SwapTile>();
    if (!swap_run_layout(*t, pa.data(), pb.data(), (int)pa.size(), n, (int)amp_bytes(s->prec))) {
        for (int g : b.gates) {
            const GateOp op = classify(gates[g].mat.data(), 2, gates[g].bits.data(), n);
            if (op.kind != GateOp::Noop) s->apply_op(op, s->amps.as<char>(), s->total());
        }
        return;
    }
    const void* dt = stage(t.get(), sizeof(SwapTile));
    const uint64_t total = s->total();
    s->launch("swap_run", 2.0 * total * s->bsz(), [&] {
        return launch_swap_run(s->amps.p, (int)amp_bytes(s->prec), total, dt, s->sm_count(), s->stream);
    });
}

// A phase-run block (fuse_runs): on complex64 states of up to 32
// qubits one pass of run_phase/phase_pair kernels with the block's phase
// function (and its trailing 1-qubit gate); otherwise its gates one by one.
// Each gate of the run must be diagonal with unit-modulus entries: its
// log-phases theta_s over its (at most two) qubits contribute, by the Moebius
// transform, a constant, one linear term per qubit and, for two qubits, the
// product term, which contains the run's pivot.
template <typename Stage>
static void run_phase_block(q1g_plan* p, q1g_state* s, const FusedBlock& b, const std::vector<SeqGate>& gates,
                            Stage&& stage)
{
    const int n = s->nbits;
    const size_t ndiag = b.gates.size() - (b.trailing_pair ? 1 : 0);
    if (s->prec != kC64 || n > 32) {
        for (int g : b.gates) {
            const GateOp op = classify(gates[g].mat.data(), (int)gates[g].bits.size(), gates[g].bits.data(), n);
            if (op.kind != GateOp::Noop) s->apply_op(op, s->amps.as<char>(), s->total());
        }
        return;
    }
    const int pivot_q = phase_run_pivot(b, p->gate_bits);
    const int pivot_pos = pivot_q >= 0 ? n - 1 - pivot_q : -1;
    std::vector<double> lin0(n, 0.0), lin1(n, 0.0);
    double c = 0.0;
    for (size_t j = 0; j < ndiag; ++j) {
        const SeqGate& g = gates[b.gates[j]];
        const size_t k = g.bits.size(), dim = size_t(1) << k;
        double th[4];
        for (size_t r = 0; r < dim; ++r)
            for (size_t col = 0; col < dim; ++col) {
                const cd v = g.mat[r * dim + col];
                if (r != col && v != cd(0.0, 0.0))
                    throw Error(Q1G_ERR_INVALID_ARGUMENT, "a gate marked diagonal has an off-diagonal entry");
                if (r == col) {
                    if (std::abs(std::abs(v) - 1.0) > 1e-9)
                        throw Error(Q1G_ERR_INVALID_ARGUMENT, "a gate marked diagonal is not a phase");
                    th[r] = std::arg(v);
                }
            }
        if (k == 1) {
            c += th[0];
            lin0[n - 1 - g.bits[0]] += th[1] - th[0];
        } else {
            // matrix index bit 1 = g.bits[0], bit 0 = g.bits[1]
            c += th[0];
            lin0[n - 1 - g.bits[0]] += th[2] - th[0];
            lin0[n - 1 - g.bits[1]] += th[1] - th[0];
            const double w = th[3] - th[2] - th[1] + th[0];
            if (g.bits[0] == pivot_q) lin1[n - 1 - g.bits[1]] += w;
            else if (g.bits[1] == pivot_q) lin1[n - 1 - g.bits[0]] += w;
            else throw Error(Q1G_ERR_INVALID_ARGUMENT, "phase run without a common qubit");
        }
    }
    std::vector<float2> tab(2048);
    phase_run_tables(n, c, lin0.data(), lin1.data(), tab.data());
    const void* dtab = stage(tab.data(), tab.size() * sizeof(float2));
    int q_pos = -1;
    double m2[8] = {1, 0, 0, 0, 0, 0, 1, 0};
    if (b.trailing_pair) {
        const SeqGate& t = gates[b.gates.back()];
        q_pos = n - 1 - t.bits[0];
        for (int e = 0; e < 4; ++e) {
            m2[2 * e] = t.mat[e].real();
            m2[2 * e + 1] = t.mat[e].imag();
        }
    }
    const uint64_t total = s->total();
    s->launch(b.trailing_pair ? "phase_pair_run_c64" : "phase_run_c64", 2.0 * total * s->bsz(), [&] {
        return launch_phase_run(s->amps.as<float2>(), total, n, pivot_pos, dtab, q_pos, m2, s->sm_count(), s->stream);
    });
}

// Positions a plan may leave out of its start-of-run subspace: the compact
// state is at most 1/8 of the full one.  Below kPrefixMinQubits a full pass
// costs microseconds, less than the compact plan's own launches and norm
// check (a 16-qubit brick of 20 layers with 8192 runs took 6.4 ms with the
// prefix against 4.3 ms without).
constexpr int kPrefixSpare = 3;
constexpr int kPrefixMinQubits = 24;

// A basis state stays a basis state on every position no gate has touched.
// So the plan's leading blocks, as long as together they touch at most
// nbits - kPrefixSpare positions, run on a compact state of those positions
// (the same blocks on renumbered qubits); the full state is then zeroed and
// the compact one scattered into it, which replaces the fill of the basis
// state.  Returns the number of blocks done.
static size_t run_subspace_prefix(q1g_plan* p, q1g_state* s, const double* mats, size_t n)
{
    const int nb = s->nbits;
    if (!p->prefix_known) {
        p->prefix_known = true;
        uint64_t mask = 0;
        size_t len = 0;
        for (const auto& b : p->blocks) {
            if (b.phase_run || b.swap_run) break;
            uint64_t m = mask;
            for (int q : b.qubits) m |= uint64_t(1) << (nb - 1 - q);
            if (__builtin_popcountll(m) > nb - kPrefixSpare) break;
            mask = m;
            ++len;
        }
        if (len >= 2 && nb >= kPrefixMinQubits) {
            const int na = __builtin_popcountll(mask);
            auto cq = [&](int q) {
                const int pos = nb - 1 - q;
                return na - 1 - __builtin_popcountll(mask & ((uint64_t(1) << pos) - 1));
            };
            auto tp = std::make_unique<q1g_plan>();
            tp->nbits = na;
            tp->width = p->width;
            tp->tensor_cores = p->tensor_cores;
            tp->tc_pairs = p->tc_pairs;
            tp->tc_max_high = p->tc_max_high;
            tp->tc_slack = p->tc_slack;
            tp->gate_bits = p->gate_bits;
            tp->mat_off = p->mat_off;
            tp->mat_doubles = p->mat_doubles;
            tp->kinds = p->kinds;
            for (size_t i = 0; i < len; ++i) {
                FusedBlock b = p->blocks[i];
                for (auto& q : b.qubits) q = cq(q);
                for (int g : b.gates)
                    for (size_t j = 0; j < p->gate_bits[g].size(); ++j) tp->gate_bits[g][j] = cq(p->gate_bits[g][j]);
                tp->blocks.push_back(b);
            }
            p->prefix_len = len;
            p->prefix_mask = mask;
            p->prefix_plan = std::move(tp);
        }
    }
    if (!p->prefix_plan) return 0;
    const uint64_t mask = p->prefix_mask;
    const int na = __builtin_popcountll(mask);
    if (!s->compact || s->compact->nbits != na || s->compact->prec != s->prec)
        s->compact = std::make_unique<q1g_state>(na, s->nshots, s->prec, s->stream);
    q1g_state* c = s->compact.get();
    c->stream = s->stream;
    c->fp64_exact = s->fp64_exact;
    c->prof = s->prof;
    c->nshots = s->nshots;
    const uint64_t b = s->basis[0];
    uint64_t cb = 0;
    SubspacePositions sp{};
    for (int pos = 0; pos < nb; ++pos)
        if ((mask >> pos) & 1) {
            if ((b >> pos) & 1) cb |= uint64_t(1) << sp.n;
            sp.pos[sp.n++] = pos;
        }
    c->sparse = true;
    c->basis.assign(1, cb);
    c->counts.assign(1, s->counts[0]);
    c->ncols = 1;
    c->norms.assign(1, s->norms[0]);
    plan_run(p->prefix_plan.get(), c, mats, n, false);
    c->ensure_dense();
    s->amps.ensure(s->N * s->bsz());
    s->launch("subspace_fill", double(s->N * s->bsz()), [&] {
        return launch_scatter_subspace(s->amps.p, c->amps.p, s->prec, nb, na, sp, b & ~mask, s->stream);
    });
    s->sparse = false;
    s->basis.clear();
    s->norm_pending = c->norm_pending;    // the compact plan's norm correction, if any, is still to come
    c->norm_pending = false;
    for (auto& pe : c->pending) s->pending.push_back(pe);
    c->pending.clear();
    return p->prefix_len;
}

void plan_run(q1g_plan* p, q1g_state* s, const double* mats, size_t n, bool subspace_prefix)
{
    if (n != p->mat_doubles)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "expected " + std::to_string(p->mat_doubles) + " matrix doubles");
    if (s->nbits != p->nbits)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "plan and state differ in qubit count");
    const size_t ng = p->gate_bits.size();
    std::vector<SeqGate> gates(ng);
    for (size_t g = 0; g < ng; ++g) {
        const size_t k = p->gate_bits[g].size();
        const size_t dim = size_t(1) << k;
        gates[g].bits = p->gate_bits[g];
        gates[g].mat.resize(dim * dim);
        const double* m = mats + p->mat_off[g];
        for (size_t e = 0; e < dim * dim; ++e) gates[g].mat[e] = cd(m[2 * e], m[2 * e + 1]);
    }
    const bool use_tc = s->prec == kC64 && s->nbits >= 12 && p->tensor_cores;
    const size_t nb = p->blocks.size();
    // Blocks are lowered one pass ahead of the launches, so the host work of
    // pass i+1 (block product, classification, tensor-core image) runs while
    // the device executes pass i.
    std::vector<GateOp> ops(nb);
    std::vector<std::vector<cd>> bmats(nb);
    std::vector<std::vector<int>> bbits(nb);
    std::vector<char> ready(nb, 0);
    auto prepare = [&](size_t bi) {
        if (ready[bi]) return;
        const auto& b = p->blocks[bi];
        if (b.gates.size() == 1) {
            bmats[bi] = gates[b.gates[0]].mat;
            bbits[bi] = gates[b.gates[0]].bits;
        } else {
            bmats[bi] = block_matrix(b, gates);
            bbits[bi] = b.qubits;
        }
        ops[bi] = classify(bmats[bi].data(), (int)bbits[bi].size(), bbits[bi].data(), s->nbits);
        ready[bi] = 1;
    };
    // The lowering of a tensor-core pass (tile geometry, padding and the f16
    // images) is kept with the plan, keyed by its first block and block count
    // and checked against the blocks' matrices and qubits and the state's
    // shape: a circuit run again builds no images (about 50 us per block on
    // the host, which small states do not hide behind their passes).
    auto lower_tc_cached = [&](size_t i, int nblk) -> TcPass {
        if (p->tc_memo.size() != kTcMaxBlocks * nb) p->tc_memo.assign(kTcMaxBlocks * nb, TcPassMemo{});
        TcPassMemo& e = p->tc_memo[kTcMaxBlocks * i + (size_t)(nblk - 1)];
        const int variant = 8 * p->tc_slack + p->tc_pairs;
        bool hit = e.nblocks == nblk && e.nbits == s->nbits && e.ncols == s->ncols && e.slack == variant;
        for (int j = 0; hit && j < nblk; ++j) hit = e.bits[j] == bbits[i + j] && e.mats[j] == bmats[i + j];
        if (!hit) {
            if (nblk == 3) {
                e.pass = lower_tc_pass({&bmats[i], &bmats[i + 1], &bmats[i + 2]},
                                       {&bbits[i], &bbits[i + 1], &bbits[i + 2]}, s->nbits, s->ncols, p->tc_slack,
                                       p->tc_pairs);
            } else if (nblk == 2) {
                e.pass = lower_tc_pass({&bmats[i], &bmats[i + 1]}, {&bbits[i], &bbits[i + 1]}, s->nbits, s->ncols,
                                       p->tc_slack, p->tc_pairs);
                if ((e.pass.offs.shuffle || e.pass.offs.direct) && e.pass.offs.pad_shift < 31) {
                    // the shuffled or direct row layout needs padding (bank
                    // conflicts); the staged one, free to order its rows,
                    // may not: one tensor-map copy per tile is kept if it can
                    TcPass staged =
                        lower_tc_pass({&bmats[i], &bmats[i + 1]}, {&bbits[i], &bbits[i + 1]}, s->nbits, s->ncols,
                                      p->tc_slack, 1);
                    if (staged.offs.pad_shift >= 31) e.pass = std::move(staged);
                }
            } else
                e.pass = lower_tc_pass({&bmats[i]}, {&bbits[i]}, s->nbits, s->ncols, p->tc_slack,
                                       p->tc_pairs >= 4 ? 4 : 1);
            e.nblocks = nblk;
            e.slack = variant;
            e.nbits = s->nbits;
            e.ncols = s->ncols;
            for (int j = 0; j < nblk; ++j) {
                e.bits[j] = bbits[i + j];
                e.mats[j] = bmats[i + j];
            }
        }
        return e.pass;
    };
    // tensor-core eligible: dense blocks of >= 3 target qubits
    auto eligible = [&](size_t bi) {
        if (p->blocks[bi].phase_run || p->blocks[bi].swap_run) return false;
        prepare(bi);
        return use_tc && ops[bi].kind == GateOp::Dense && ops[bi].t >= 3 && bbits[bi].size() <= 5 &&
               tc_block_bounded(bmats[bi].data(), 1 << bbits[bi].size());
    };
    double max_norm = 0.0;
    for (double v : s->norms) max_norm = std::max(max_norm, v);
    // Staging: every pass uploads its matrix or tensor-core image from its own
    // slice of one pinned buffer (at most 32 KB per block).
    if (p->staged) check_cuda(cudaEventSynchronize(p->staged), "plan staging wait");
    else check_cuda(cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming), "cudaEventCreate");
    p->hmats.ensure(std::max<size_t>(nb, 1) * 32768);
    p->dmats.ensure(std::max<size_t>(nb, 1) * 32768);
    size_t staged = 0;
    auto stage = [&](const void* src, size_t sz) -> const void* {
        char* h = p->hmats.as<char>() + staged;
        char* d = p->dmats.as<char>() + staged;
        std::memcpy(h, src, sz);
        s->h2d(d, h, sz, "upload plan matrix");
        staged += (sz + 255) & ~size_t(255);
        return d;
    };
    bool launched = false, any_tc = false;
    auto begin = [&] {
        if (!launched) s->ensure_dense();
        launched = true;
    };
    const size_t first = (subspace_prefix && s->sparse && s->ncols == 1 && s->basis.size() == 1)
                             ? run_subspace_prefix(p, s, mats, n)
                             : 0;
    for (size_t i = first; i < nb; ++i) {
        if (p->blocks[i].phase_run) {
            begin();
            run_phase_block(p, s, p->blocks[i], gates, stage);
            continue;
        }
        if (p->blocks[i].swap_run) {
            begin();
            run_swap_block(s, p->blocks[i], gates, stage);
            continue;
        }
        prepare(i);
        const GateOp& op = ops[i];
        if (op.kind == GateOp::Noop) continue;
        if (eligible(i)) {
            // consecutive blocks share a pass when their qubits fit one
            // 12-position tile with runs of >= 128 amplitudes or as one
            // tensor-map box: up to three in the four-group kernel's direct
            // chain in pair mode 5, else two
            TcPass t;
            int group = 1;
            // -1: blocks i .. i+k-1 do not fit one tile; else its run bits
            auto fits = [&](int k) {
                std::vector<const std::vector<int>*> bs;
                std::vector<int> u;
                for (int j = 0; j < k; ++j) {
                    bs.push_back(&bbits[i + j]);
                    for (int q : positions_of(bbits[i + j], s->nbits))
                        if (std::find(u.begin(), u.end(), q) == u.end()) u.push_back(q);
                }
                if (u.size() > 12) return -1;
                const auto Tk = tile_positions(bs, s->nbits);
                int high = 0;
                for (int q : Tk) high += q >= kHighPosition;
                const int L = tile_run_bits(Tk);
                if (high > p->tc_max_high) return -1;
                if (L < kMinTcRunBits && !tc_tile_box(Tk.data(), s->nbits, s->ncols).usable) return -1;
                return L;
            };
            if (p->tc_pairs == 5 && i + 2 < nb && eligible(i + 1) && eligible(i + 2)) {
                const int L3 = fits(3);
                if (L3 >= 0) {
                    t = lower_tc_cached(i, 3);
                    // short runs only as one unpadded tensor-map copy; a
                    // third block only where the tile's runs are at least
                    // 64 bytes (a copy of 16- or 32-byte runs wastes DRAM
                    // sectors: such passes ran at 19-46 % of DRAM rate) and
                    // the layout keeps the bank wavefronts within twice the
                    // minimum (a conflicted write-back costs more than the
                    // saved pass)
                    if ((L3 >= kMinTcRunBits || t.offs.pad_shift >= 31) && L3 >= kMinTripleRunBits &&
                        t.cost <= 2 * t.ideal)
                        group = 3;
                }
            }
            if (group == 1 && p->tc_pairs && i + 1 < nb && eligible(i + 1)) {
                const int L2 = fits(2);
                if (L2 >= 0) {
                    t = lower_tc_cached(i, 2);
                    if (L2 >= kMinTcRunBits || t.offs.pad_shift >= 31) group = 2;
                }
            }
            if (group == 1) t = lower_tc_cached(i, 1);
            begin();
            if (!any_tc) {
                s->errbuf.ensure(sizeof(int));
                check_cuda(cudaMemsetAsync(s->errbuf.p, 0, sizeof(int), s->stream), "clear error flag");
                any_tc = true;
            }
            tc_operand_scales(max_norm, t.offs);
            const void* img = stage(t.images.data(), t.images.size() * sizeof(uint16_t));
            const uint64_t total = s->total();
            s->launch("fused_tc_c64", 2.0 * total * s->bsz(), [&] {
                return launch_fused_tc(s->amps.as<float2>(), total >> 12, t.tilemap, t.offs, t.box, img,
                                       s->errbuf.as<int>(), s->sm_count(), s->stream, s->tc_wait_ns,
                                       t.offs.st_box ? &t.sbox : nullptr);
            });
            i += (size_t)(group - 1);   // the next blocks rode in this pass
        } else if (op.kind == GateOp::Dense &&
                   dense_tiled_applies(s->prec, s->nbits, op.t, op.map, s->fp64_exact)) {
            begin();
            const size_t d2 = op.dense.size();
            std::vector<double> v(2 * d2);
            for (size_t e = 0; e < d2; ++e) {
                v[2 * e] = op.dense[e].real();
                v[2 * e + 1] = op.dense[e].imag();
            }
            std::vector<unsigned char> img(dense_tiled_matrix_bytes(s->prec, op.t));
            dense_tiled_matrix(s->prec, op.t, v.data(), img.data());
            const void* dm = stage(img.data(), img.size());
            const uint64_t total = s->total();
            s->launch(s->prec == kC128 ? "dense_tiled_c128" : "dense_tiled_c64", 2.0 * s->bsz() * op.touched(total),
                      [&] {
                          return launch_dense_tiled(s->amps.p, s->prec, total, s->nbits, op.map, op.offs, op.t, dm,
                                                    s->sm_count(), s->stream);
                      });
        } else if (op.kind == GateOp::Dense) {
            begin();
            const size_t d2 = op.dense.size();
            const void* dm;
            if (s->prec == kC128) {
                std::vector<double> v(2 * d2);
                for (size_t e = 0; e < d2; ++e) {
                    v[2 * e] = op.dense[e].real();
                    v[2 * e + 1] = op.dense[e].imag();
                }
                dm = stage(v.data(), v.size() * sizeof(double));
            } else {
                std::vector<float> v(2 * d2);
                for (size_t e = 0; e < d2; ++e) {
                    v[2 * e] = (float)op.dense[e].real();
                    v[2 * e + 1] = (float)op.dense[e].imag();
                }
                dm = stage(v.data(), v.size() * sizeof(float));
            }
            const uint64_t total = s->total();
            s->launch(s->prec == kC128 ? "dense_c128" : "dense_c64", 2.0 * s->bsz() * op.touched(total), [&] {
                return launch_dense(s->amps.p, s->prec, total, op.map, op.offs, op.t, dm, s->stream);
            });
        } else {
            begin();
            s->apply_op(op, s->amps.as<char>(), s->total());
        }
    }
    if (staged) check_cuda(cudaEventRecord(p->staged, s->stream), "cudaEventRecord");
    p->last_h2d_bytes = staged;
    if (!launched) return;
    if (any_tc) {
        // the tensor-core passes' bounded waits: report an expiry now
        s->hstage.ensure(sizeof(int));
        int* h_flag = s->hstage.as<int>();
        s->d2h(h_flag, s->errbuf.p, sizeof(int), "read error flag");
        s->sync();
        if (*h_flag) throw Error(Q1G_ERR_TIMEOUT, "a tensor-core block kernel gave up waiting on its MMAs");
        s->norm_pending = true;
    }
}

}  // namespace q1g

std::vector<double> q1g_state::measure_norms()
{
    using namespace q1g;
    if (sparse) return std::vector<double>(ncols, 1.0);
    q1g_state* s = this;
    const uint64_t total = s->total();
    const uint64_t chunk = std::min<uint64_t>(s->N, 256);
    const uint64_t nch = s->N / chunk;
    const uint64_t ntmp = segment_sums_tmp_doubles(s->ncols, nch);
    s->dscratch.ensure((s->ncols * nch + 2 * s->ncols + ntmp) * sizeof(double));
    double* d_sums = s->dscratch.as<double>();
    double* d_norm = d_sums + s->ncols * nch;
    s->launch("column_norms", double(total * s->bsz()), [&] {
        return launch_chunk_sums_dense(s->amps.p, s->prec, total, chunk, d_sums, s->stream);
    });
    check_cuda(launch_segment_sums(d_sums, s->ncols, nch, d_norm, d_norm + 2 * s->ncols, s->stream),
               "segment_sums");
    s->hstage.ensure(s->ncols * sizeof(double));
    double* h_norm = s->hstage.as<double>();
    s->d2h(h_norm, d_norm, s->ncols * sizeof(double), "read norms");
    s->sync();
    return std::vector<double>(h_norm, h_norm + s->ncols);
}

void q1g_state::settle_norms()
{
    using namespace q1g;
    if (!norm_pending || sparse) {
        norm_pending = false;
        return;
    }
    q1g_state* s = this;
    {
        // per-column squared norms now, then rescale each column to the norm
        // it should have (the plans since the last settle were unitary)
        const std::vector<double> h_norm = s->measure_norms();
        const uint64_t total = s->total();
        std::vector<double> scale(s->ncols, 1.0);
        bool any_scale = false;
        for (uint64_t c = 0; c < s->ncols; ++c) {
            if (h_norm[c] > 0.0) scale[c] = std::sqrt(s->norms[c] / h_norm[c]);
            any_scale |= scale[c] != 1.0;
        }
        if (any_scale) {
            // measure_norms left its sums in dscratch: the scales go after them
            const uint64_t nch = s->N / std::min<uint64_t>(s->N, 256);
            double* d_scale = s->dscratch.as<double>() + s->ncols * nch + s->ncols;
            s->h2d(d_scale, scale.data(), s->ncols * sizeof(double), "upload scales");
            s->launch("renormalise", 2.0 * total * s->bsz(), [&] {
                return launch_scale_columns(s->amps.p, s->prec, s->N, s->ncols, d_scale, s->stream);
            });
            s->sync();
        }
    }
    norm_pending = false;
}
