// Batched executor: host state of a batch of independent circuits.
#pragma once

#include <vector>

#include "engine.h"

struct q1g_batch {
    int width = 4;                      // fusion width (<= 4)
    std::vector<q1g::BatchCircuit> circuits;   // in add order; res_off set at build
    std::vector<q1g::BatchOp> ops;
    std::vector<float2> mats;
    std::vector<uint64_t> cbit_tables;
    bool built = false;
    uint64_t total_runs = 0;
    uint64_t arena_amps = 0;
    uint64_t scratch_per_cta = 0;
    int sms = 0;
    q1g::DevBuf arena, results, dcircuits, dops, dmats, dtables, scratch, queue, traffic;
    q1g::HostBuf hresults, htraffic;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.f;
    uint64_t last_traffic = 0;          // algorithmic device-memory bytes of the last run
    ~q1g_batch();
};

namespace q1g {
void batch_add_circuit(q1g_batch* b, size_t nr_bits, size_t nr_shots, uint64_t seed, size_t nops, const int* kinds,
                       const size_t* nbits_per_op, const size_t* bits_flat, const double* mats_flat,
                       const size_t* args);
void batch_run(q1g_batch* b, uint64_t* results, size_t len);
// warp-tile layout of a dense op on nbits qubits, gate positions pos[0..tb)
void batch_tile_layout(BatchOp& op, const int* pos, int tb, int nbits);
}  // namespace q1g
