// Host-side gate lowering: matrix classification and the gate-fusion pass.
#pragma once

#include <stdint.h>

#include <complex>
#include <vector>

#include "kernels.h"

namespace q1g {

using cd = std::complex<double>;

// A gate (or fused block) lowered onto kernel arguments.
struct GateOp {
    enum Kind { Noop, Pair, Phase, Dense } kind = Noop;
    IndexMap map{};          // all gate positions zeroed, controls in setmask
    uint64_t o0 = 0, o1 = 0; // Pair: offsets of the two touched basis states
    double m2[8] = {0};      // Pair: 2x2 (re, im) row-major
    double ph[2] = {1, 0};   // Phase
    int t = 0;               // Dense: number of target qubits
    DenseOffsets offs{};     // Dense: offsets of the 2^t target states
    std::vector<cd> dense;   // Dense: 2^t x 2^t row-major
    int k = 0;               // gate qubits including controls
    // Amplitudes read and written per launch over `total` amplitudes.
    uint64_t touched(uint64_t total) const;
};

// Classify the 2^k x 2^k matrix `mat` acting on qubits `bits` (bits[0] is the
// most significant bit of the matrix index, src/gates.rs:40-53) of an
// nbits-qubit state: control qubits (identity whenever the bit is 0) move
// into the index map, basis states the gate leaves fixed are dropped, and
// what remains is a Phase (one state), a Pair (two) or a Dense update.
GateOp classify(const cd* mat, int k, const int* bits, int nbits);

// A gate of a sequence: qubits and matrix.
struct SeqGate {
    std::vector<int> bits;
    std::vector<cd> mat;   // 2^k x 2^k row-major
};

// Fusion: the gate list grouped into blocks of at most `width` qubits.  A
// block's qubits are ascending (first = most significant matrix bit) and its
// gates are the sequence indices it absorbed, in order.
struct FusedBlock {
    std::vector<int> qubits;
    std::vector<int> gates;
    // A run of diagonal gates applied as one phase function (fuse_runs), its
    // last gate a non-diagonal 1-qubit gate when trailing_pair is set.
    bool phase_run = false;
    bool trailing_pair = false;
    // A run of swaps on pairwise disjoint qubit pairs, one permutation pass.
    bool swap_run = false;
};

// Gate kinds a plan may be told about (q1g_plan_set_gate_kinds).
enum GateKind : unsigned char { kGateGeneral = 0, kGateDiagonal = 1, kGateSwap = 2 };

// Greedy fusion over open blocks on disjoint qubit sets: a gate joins the
// open blocks it touches when their union fits in `width` qubits; otherwise
// the largest subset that fits is kept and the other touched blocks are
// emitted first.  A final pass merges an emitted block into an earlier one
// when every block in between is disjoint from it.  Only the qubit lists are
// used, so the grouping can be computed once per circuit structure.
std::vector<FusedBlock> fuse_greedy(const std::vector<std::vector<int>>& gate_bits, int nbits, int width);

// Window fusion: blocks are chosen one at a time, each the qubit set of at
// most `width` qubits that absorbs the most gates whose predecessors are all
// done (every gate on its qubits whose own qubits lie in the set, in a valid
// order).  The candidate sets are the windows of `width` consecutive qubits
// and, for every ready gate, the set grown from its qubits by the ready gates
// adding the fewest new qubits.  A gate wider than `width` is a block alone.
std::vector<FusedBlock> fuse_windows(const std::vector<std::vector<int>>& gate_bits, int nbits, int width);

// The fusion of a gate sequence: of fuse_greedy and fuse_windows, the one
// with fewer blocks.
std::vector<FusedBlock> fuse(const std::vector<std::vector<int>>& gate_bits, int nbits, int width);

// Shortest run of consecutive diagonal gates taken as one phase pass.
constexpr int kMinPhaseRun = 3;

// fuse() with two kinds of runs taken out first (kinds[g] a GateKind):
// - a run of at least kMinPhaseRun consecutive diagonal gates, none on more
//   than two qubits and every two-qubit one sharing a common qubit (the
//   pivot), is one phase-run block; its phase is c + L0(x) + x_pivot L1(x)
//   with L0, L1 linear in the basis bits.  A non-diagonal 1-qubit gate
//   directly after the run joins it (applied after the phases in the same
//   pass);
// - a run of at least 2 consecutive swaps on pairwise disjoint qubit pairs is
//   one swap-run block (a permutation of the bit positions).
// The gates between runs are fused by fuse(); blocks never cross a run.
std::vector<FusedBlock> fuse_runs(const std::vector<std::vector<int>>& gate_bits,
                                  const std::vector<unsigned char>& kinds, int nbits, int width);

// Qubit shared by every two-qubit gate of a phase run (-1 when it has none).
int phase_run_pivot(const FusedBlock& b, const std::vector<std::vector<int>>& gate_bits);

// Matrix of a block: product of its gates' matrices embedded on its qubits.
std::vector<cd> block_matrix(const FusedBlock& b, const std::vector<SeqGate>& gates);

// Embed `mat` on `bits` into the 2^|qubits| space of `qubits`.
std::vector<cd> embed_matrix(const std::vector<cd>& mat, const std::vector<int>& bits,
                             const std::vector<int>& qubits);

}  // namespace q1g
