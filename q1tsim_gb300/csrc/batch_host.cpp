// Host side of the batched executor: lowering of circuit programs, device
// buffers, and the CUDA graph that replays the persistent launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>

#include "batch.h"

using namespace q1g;

q1g_batch::~q1g_batch()
{
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

namespace q1g {

// Warp-tile layout of a dense op (warp_tile.h): complex64 tiles of 1024
// amplitudes, 16 per stage row.
void batch_tile_layout(BatchOp& op, const int* pos, int tb, int nbits)
{
    warp_tile_layout(op.tile, pos, tb, op.offs, nbits, 10, 4);
}

static BatchOp dense_op(const std::vector<cd>& m, const std::vector<int>& qubits, int nbits, int cond, int ccbit,
                        std::vector<float2>& pool)
{
    BatchOp op{};
    op.kind = kBatchDense;
    op.t = (int)qubits.size();
    op.cond = cond;
    op.ccbit = ccbit;
    op.map.nz = op.t;
    std::vector<int> pos(op.t);
    for (int j = 0; j < op.t; ++j) pos[j] = nbits - 1 - qubits[j];
    std::vector<int> sorted = pos;
    std::sort(sorted.begin(), sorted.end());
    for (int j = 0; j < op.t; ++j) op.map.zpos[j] = sorted[j];
    op.map.setmask = 0;
    for (int s = 0; s < (1 << op.t); ++s) {
        uint64_t o = 0;
        for (int j = 0; j < op.t; ++j)
            if ((s >> (op.t - 1 - j)) & 1) o |= uint64_t(1) << pos[j];
        op.offs[s] = o;
    }
    batch_tile_layout(op, pos.data(), op.t, nbits);
    op.mat = (uint32_t)pool.size();
    for (const cd& v : m) pool.push_back(make_float2((float)v.real(), (float)v.imag()));
    return op;
}

void batch_add_circuit(q1g_batch* b, size_t nr_bits, size_t nr_shots, uint64_t seed, size_t nops, const int* kinds,
                       const size_t* nbits_per_op, const size_t* bits_flat, const double* mats_flat,
                       const size_t* args)
{
    if (b->built) throw Error(Q1G_ERR_INVALID_ARGUMENT, "batch already ran: add circuits before the first run");
    if (nr_bits < 1 || nr_bits > 26)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "batched circuits take 1 to 26 qubits");
    const int n = (int)nr_bits;
    BatchCircuit C{};
    C.nbits = n;
    C.nshots = nr_shots;
    C.seed = seed;
    C.op_begin = (uint32_t)b->ops.size();
    std::vector<SeqGate> seg;
    auto flush = [&] {
        if (seg.empty()) return;
        std::vector<std::vector<int>> gb;
        for (auto& g : seg) gb.push_back(g.bits);
        for (const auto& blk : fuse(gb, n, b->width)) {
            const auto m = blk.gates.size() == 1 ? embed_matrix(seg[blk.gates[0]].mat, seg[blk.gates[0]].bits, blk.qubits)
                                                 : block_matrix(blk, seg);
            b->ops.push_back(dense_op(m, blk.qubits, n, -1, 0, b->mats));
        }
        seg.clear();
    };
    int nmeasure = 0;
    bool sampled = false;
    size_t bo = 0, mo = 0;
    for (size_t i = 0; i < nops; ++i) {
        const size_t k = nbits_per_op[i];
        const size_t* bits = bits_flat + bo;
        bo += k;
        if (sampled) throw Error(Q1G_ERR_INVALID_ARGUMENT, "measure_all must be the last op of a batched circuit");
        if (kinds[i] == Q1G_OP_GATE || kinds[i] == Q1G_OP_CONDITIONAL) {
            if (k < 1 || k > 4) throw Error(Q1G_ERR_INVALID_NR_BITS, "batched gates act on 1 to 4 qubits");
            const size_t dim = size_t(1) << k;
            SeqGate g;
            for (size_t j = 0; j < k; ++j) {
                if (bits[j] >= nr_bits) throw Error(Q1G_ERR_INVALID_QBIT, "Invalid qubit index " + std::to_string(bits[j]));
                g.bits.push_back((int)bits[j]);
            }
            g.mat.resize(dim * dim);
            for (size_t e = 0; e < dim * dim; ++e) g.mat[e] = cd(mats_flat[mo + 2 * e], mats_flat[mo + 2 * e + 1]);
            mo += 2 * dim * dim;
            if (kinds[i] == Q1G_OP_GATE) {
                seg.push_back(g);
            } else {
                flush();
                // every run of a column holds the same classical bits (set by
                // the measurements that split the columns, 0 before any), so
                // a gate conditioned on one bit applies to whole columns
                const size_t cbit = args[2 * i], value = args[2 * i + 1];
                if (cbit >= 64) throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit " + std::to_string(cbit), cbit);
                if (value > 1)
                    throw Error(Q1G_ERR_INVALID_ARGUMENT, "a batched conditional gate tests one classical bit for 0 or 1");
                std::vector<int> q = g.bits;
                std::sort(q.begin(), q.end());
                b->ops.push_back(dense_op(embed_matrix(g.mat, g.bits, q), q, n, (int)value, (int)cbit, b->mats));
            }
        } else if (kinds[i] == Q1G_OP_MEASURE) {
            flush();
            if ((1 << (nmeasure + 1)) > kBatchMaxCols)
                throw Error(Q1G_ERR_INVALID_ARGUMENT, "at most 4 mid-circuit measurements per batched circuit (" +
                                                          std::to_string(kBatchMaxCols) + " run columns)");
            const size_t q = args[2 * i], cbit = args[2 * i + 1];
            if (q >= nr_bits) throw Error(Q1G_ERR_INVALID_QBIT, "Invalid qubit index " + std::to_string(q), q);
            if (cbit >= 64) throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit " + std::to_string(cbit), cbit);
            BatchOp op{};
            op.kind = kBatchMeasure;
            op.pos = n - 1 - (int)q;
            op.cbit = (int)cbit;
            b->ops.push_back(op);
            ++nmeasure;
        } else if (kinds[i] == Q1G_OP_MEASURE_ALL) {
            flush();
            if (k != nr_bits)
                throw Error(Q1G_ERR_INVALID_NR_MEASUREMENT_BITS, "measure_all needs one classical bit per qubit");
            BatchOp op{};
            op.kind = kBatchSample;
            op.cpos = (uint32_t)(b->cbit_tables.size() / 64);
            std::vector<uint64_t> table(64, 0);
            for (size_t q = 0; q < k; ++q) {
                if (bits[q] >= 64) throw Error(Q1G_ERR_INVALID_CBIT, "Invalid classical bit " + std::to_string(bits[q]));
                table[n - 1 - q] = uint64_t(1) << bits[q];
                op.cmask |= uint64_t(1) << bits[q];
            }
            b->cbit_tables.insert(b->cbit_tables.end(), table.begin(), table.end());
            b->ops.push_back(op);
            sampled = true;
        } else {
            throw Error(Q1G_ERR_INVALID_ARGUMENT, "unknown batched op kind");
        }
    }
    flush();
    C.op_end = (uint32_t)b->ops.size();
    // every measurement at most doubles the columns, and a column holds at
    // least one run
    C.maxcols = (int)std::min<uint64_t>(uint64_t(1) << nmeasure, std::max<uint64_t>(nr_shots, 1));
    b->circuits.push_back(C);
}

static void upload(DevBuf& d, const void* h, size_t bytes, cudaStream_t st)
{
    d.ensure(std::max<size_t>(bytes, 16));
    if (bytes) check_cuda(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, st), "batch upload");
}

static void batch_build(q1g_batch* b)
{
    if (!b->stream) check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    // queue order: most work first (longest-processing-time order), so the
    // long circuits start early and the short ones fill in at the end.  The
    // work estimate counts amplitude reads and writes: every gate pass over
    // every column (their number at most doubling at each measurement), the
    // measurements, and the sampling's chunk sums and searched chunks.
    const size_t nc = b->circuits.size();
    std::vector<double> work(nc, 0.0);
    for (size_t i = 0; i < nc; ++i) {
        const BatchCircuit& C = b->circuits[i];
        const double N = std::ldexp(1.0, C.nbits);
        double w = N, cols = 1.0;
        for (uint32_t oi = C.op_begin; oi < C.op_end; ++oi) {
            const BatchOp& op = b->ops[oi];
            if (op.kind == kBatchDense) {
                w += 2.0 * N * (op.cond >= 0 ? 1.0 : cols);
            } else if (op.kind == kBatchMeasure) {
                w += 4.0 * N * cols;
                cols = std::min(2.0 * cols, (double)C.maxcols);
            } else {
                w += N * cols + (double)C.nshots * std::min(N, 256.0);
            }
        }
        work[i] = w;
    }
    std::vector<size_t> order(nc);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return work[x] > work[y]; });
    uint64_t res = 0;
    for (auto& C : b->circuits) {
        C.res_off = res;
        res += C.nshots;
    }
    b->total_runs = res;
    std::vector<BatchCircuit> queue;
    uint64_t off = 0, per_cta = 16;
    for (size_t i : order) {
        BatchCircuit C = b->circuits[i];
        C.state_off = off;
        off += (uint64_t)C.maxcols * (uint64_t(1) << C.nbits);
        const uint64_t n = uint64_t(1) << C.nbits;
        per_cta = std::max<uint64_t>(per_cta, n / std::min<uint64_t>(n, 256) + C.nshots + 2);
        queue.push_back(C);
    }
    b->arena_amps = off;
    b->scratch_per_cta = (per_cta + 31) & ~uint64_t(31);
    b->arena.ensure(std::max<uint64_t>(off, 1) * sizeof(float2));
    b->results.ensure(std::max<uint64_t>(res, 1) * sizeof(uint64_t));
    b->hresults.ensure(std::max<uint64_t>(res, 1) * sizeof(uint64_t));
    upload(b->dcircuits, queue.data(), queue.size() * sizeof(BatchCircuit), b->stream);
    upload(b->dops, b->ops.data(), b->ops.size() * sizeof(BatchOp), b->stream);
    upload(b->dmats, b->mats.data(), b->mats.size() * sizeof(float2), b->stream);
    upload(b->dtables, b->cbit_tables.data(), b->cbit_tables.size() * sizeof(uint64_t), b->stream);
    const int grid = std::min<int>(b->sms, (int)std::max<size_t>(nc, 1));
    b->scratch.ensure((size_t)grid * b->scratch_per_cta * sizeof(double));
    b->queue.ensure(sizeof(unsigned));
    b->traffic.ensure(sizeof(unsigned long long));
    b->htraffic.ensure(sizeof(unsigned long long));
    check_cuda(cudaStreamSynchronize(b->stream), "batch upload");

    BatchArgs a{};
    a.arena = b->arena.as<float2>();
    a.results = b->results.as<uint64_t>();
    a.circuits = b->dcircuits.as<BatchCircuit>();
    a.ncircuits = (int)nc;
    a.ops = b->dops.as<BatchOp>();
    a.mats = b->dmats.as<float2>();
    a.cbit_tables = b->dtables.as<uint64_t>();
    a.scratch = b->scratch.as<double>();
    a.scratch_per_cta = b->scratch_per_cta;
    a.queue = b->queue.as<unsigned>();
    a.traffic = b->traffic.as<unsigned long long>();
    check_cuda(setup_batch_kernel(), "batch kernel attributes");
    // one execution = reset queue and results, the persistent launch, results out
    check_cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = cudaMemsetAsync(b->queue.p, 0, sizeof(unsigned), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->traffic.p, 0, sizeof(unsigned long long), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->results.p, 0, std::max<uint64_t>(res, 1) * sizeof(uint64_t), b->stream);
    if (e == cudaSuccess) e = launch_batch(a, b->sms, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->hresults.p, b->results.p, res * sizeof(uint64_t), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->htraffic.p, b->traffic.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            b->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    check_cuda(e, "batch capture");
    check_cuda(e2, "end capture");
    b->graph = g;
    check_cuda(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate");
    check_cuda(cudaEventCreate(&b->ev0), "event");
    check_cuda(cudaEventCreate(&b->ev1), "event");
    b->built = true;
}

void batch_run(q1g_batch* b, uint64_t* results, size_t len)
{
    if (!b->built) batch_build(b);
    if (results && len < b->total_runs)
        throw Error(Q1G_ERR_NOT_ENOUGH_SPACE, "results buffer holds fewer words than the batch has runs");
    check_cuda(cudaEventRecord(b->ev0, b->stream), "event");
    check_cuda(cudaGraphLaunch(b->exec, b->stream), "graph launch");
    check_cuda(cudaEventRecord(b->ev1, b->stream), "event");
    check_cuda(cudaStreamSynchronize(b->stream), "batch run");
    float ms = 0.f;
    check_cuda(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "event time");
    b->last_ms = ms;
    b->last_traffic = *static_cast<const unsigned long long*>(b->htraffic.p);
    if (results) std::memcpy(results, b->hresults.p, b->total_runs * sizeof(uint64_t));
}

}  // namespace q1g
