// Gate classification and fusion (host side).
#include "gate_plan.h"

#include <algorithm>
#include <stdexcept>

#include "engine.h"

namespace q1g {

uint64_t GateOp::touched(uint64_t total) const
{
    const uint64_t units = total >> map.nz;
    switch (kind) {
        case Pair: return 2 * units;
        case Phase: return units;
        case Dense: return (uint64_t(1) << t) * units;
        default: return 0;
    }
}

GateOp classify(const cd* mat, int k, const int* bits, int nbits)
{
    if (k < 0 || k > kMaxMapBits)
        throw Error(Q1G_ERR_INVALID_ARGUMENT, "gates on more than 12 qubits are not supported");
    const int dim = 1 << k;
    auto M = [&](int r, int c) { return mat[(size_t)r * dim + c]; };
    auto gbit = [&](int x, int m) { return (x >> (k - 1 - m)) & 1; };

    std::vector<int> ctrl, tgt;
    for (int m = 0; m < k; ++m) {
        bool is_ctrl = true;
        for (int r = 0; r < dim && is_ctrl; ++r)
            for (int c = 0; c < dim; ++c)
                if (gbit(r, m) == 0 || gbit(c, m) == 0) {
                    const cd expect = r == c ? cd(1.0, 0.0) : cd(0.0, 0.0);
                    if (M(r, c) != expect) {
                        is_ctrl = false;
                        break;
                    }
                }
        (is_ctrl ? ctrl : tgt).push_back(m);
    }
    const int t = (int)tgt.size();
    int cpat = 0;
    for (int m : ctrl) cpat |= 1 << (k - 1 - m);
    auto full_index = [&](int s) {
        int x = cpat;
        for (int j = 0; j < t; ++j)
            if ((s >> (t - 1 - j)) & 1) x |= 1 << (k - 1 - tgt[j]);
        return x;
    };
    auto pos = [&](int m) { return nbits - 1 - bits[m]; };
    auto offset = [&](int s) {
        uint64_t o = 0;
        for (int j = 0; j < t; ++j)
            if ((s >> (t - 1 - j)) & 1) o |= uint64_t(1) << pos(tgt[j]);
        return o;
    };

    GateOp op;
    op.k = k;
    op.map.nz = k;
    for (int m = 0; m < k; ++m) op.map.zpos[m] = pos(m);
    std::sort(op.map.zpos, op.map.zpos + k);
    op.map.setmask = 0;
    for (int m : ctrl) op.map.setmask |= uint64_t(1) << pos(m);

    const int tdim = 1 << t;
    std::vector<cd> G((size_t)tdim * tdim);
    for (int r = 0; r < tdim; ++r)
        for (int c = 0; c < tdim; ++c) G[(size_t)r * tdim + c] = M(full_index(r), full_index(c));

    std::vector<int> nonfixed;
    for (int s = 0; s < tdim; ++s) {
        bool fixed = G[(size_t)s * tdim + s] == cd(1.0, 0.0);
        for (int o = 0; o < tdim && fixed; ++o)
            if (o != s && (G[(size_t)s * tdim + o] != cd(0.0, 0.0) || G[(size_t)o * tdim + s] != cd(0.0, 0.0)))
                fixed = false;
        if (!fixed) nonfixed.push_back(s);
    }
    if (nonfixed.empty()) {
        op.kind = GateOp::Noop;
    } else if (nonfixed.size() == 1) {
        const int s = nonfixed[0];
        op.kind = GateOp::Phase;
        op.map.setmask |= offset(s);
        const cd g = G[(size_t)s * tdim + s];
        op.ph[0] = g.real();
        op.ph[1] = g.imag();
    } else if (nonfixed.size() == 2) {
        const int s0 = nonfixed[0], s1 = nonfixed[1];
        op.kind = GateOp::Pair;
        op.o0 = offset(s0);
        op.o1 = offset(s1);
        const cd e[4] = {G[(size_t)s0 * tdim + s0], G[(size_t)s0 * tdim + s1],
                         G[(size_t)s1 * tdim + s0], G[(size_t)s1 * tdim + s1]};
        for (int q = 0; q < 4; ++q) {
            op.m2[2 * q] = e[q].real();
            op.m2[2 * q + 1] = e[q].imag();
        }
    } else {
        if (t > 5)
            throw Error(Q1G_ERR_INVALID_ARGUMENT,
                        "a gate acting densely on more than 5 non-control qubits is not supported");
        op.kind = GateOp::Dense;
        op.t = t;
        for (int s = 0; s < tdim; ++s) op.offs.off[s] = offset(s);
        op.dense = G;
    }
    return op;
}

std::vector<cd> embed_matrix(const std::vector<cd>& mat, const std::vector<int>& bits,
                             const std::vector<int>& qubits)
{
    const int k = (int)bits.size();
    const int m = (int)qubits.size();
    const int dim = 1 << m;
    std::vector<int> bpos(k);  // position (within the block index) of gate bit j
    for (int j = 0; j < k; ++j) {
        auto it = std::find(qubits.begin(), qubits.end(), bits[j]);
        bpos[j] = m - 1 - (int)(it - qubits.begin());
    }
    int gmask = 0;
    for (int j = 0; j < k; ++j) gmask |= 1 << bpos[j];
    const int gdim = 1 << k;
    std::vector<cd> full((size_t)dim * dim, cd(0.0, 0.0));
    for (int col = 0; col < dim; ++col) {
        int gin = 0;
        for (int j = 0; j < k; ++j) gin |= ((col >> bpos[j]) & 1) << (k - 1 - j);
        const int base = col & ~gmask;
        for (int gout = 0; gout < gdim; ++gout) {
            int row = base;
            for (int j = 0; j < k; ++j) row |= ((gout >> (k - 1 - j)) & 1) << bpos[j];
            full[(size_t)row * dim + col] += mat[(size_t)gout * gdim + gin];
        }
    }
    return full;
}

std::vector<cd> block_matrix(const FusedBlock& b, const std::vector<SeqGate>& gates)
{
    // acc = G_last ... G_first, each gate applied to the rows of acc as a
    // k-qubit operator on its bits (32 * 2^k multiply-adds per column, not a
    // dense product with the embedded matrix).
    const int m = (int)b.qubits.size();
    const int dim = 1 << m;
    std::vector<double> acc(2 * (size_t)dim * dim, 0.0);   // row-major (re, im)
    for (int i = 0; i < dim; ++i) acc[2 * ((size_t)i * dim + i)] = 1.0;
    double vin[2 * 32], vout[2 * 32];
    int rowof[32];
    for (int gi : b.gates) {
        const auto& g = gates[gi];
        const int k = (int)g.bits.size();
        const int gdim = 1 << k;
        int bpos[5], gmask = 0;
        for (int j = 0; j < k; ++j) {
            auto it = std::find(b.qubits.begin(), b.qubits.end(), g.bits[j]);
            bpos[j] = m - 1 - (int)(it - b.qubits.begin());
            gmask |= 1 << bpos[j];
        }
        for (int gs = 0; gs < gdim; ++gs) {
            int r = 0;
            for (int j = 0; j < k; ++j) r |= ((gs >> (k - 1 - j)) & 1) << bpos[j];
            rowof[gs] = r;
        }
        const double* gm = reinterpret_cast<const double*>(g.mat.data());
        for (int base = 0; base < dim; ++base) {
            if (base & gmask) continue;
            for (int c = 0; c < dim; ++c) {
                for (int gs = 0; gs < gdim; ++gs) {
                    const double* a = &acc[2 * ((size_t)(base | rowof[gs]) * dim + c)];
                    vin[2 * gs] = a[0];
                    vin[2 * gs + 1] = a[1];
                }
                for (int go = 0; go < gdim; ++go) {
                    double re = 0.0, im = 0.0;
                    const double* row = gm + 2 * (size_t)go * gdim;
                    for (int gs = 0; gs < gdim; ++gs) {
                        re += row[2 * gs] * vin[2 * gs] - row[2 * gs + 1] * vin[2 * gs + 1];
                        im += row[2 * gs] * vin[2 * gs + 1] + row[2 * gs + 1] * vin[2 * gs];
                    }
                    vout[2 * go] = re;
                    vout[2 * go + 1] = im;
                }
                for (int go = 0; go < gdim; ++go) {
                    double* a = &acc[2 * ((size_t)(base | rowof[go]) * dim + c)];
                    a[0] = vout[2 * go];
                    a[1] = vout[2 * go + 1];
                }
            }
        }
    }
    std::vector<cd> out((size_t)dim * dim);
    for (size_t e = 0; e < out.size(); ++e) out[e] = cd(acc[2 * e], acc[2 * e + 1]);
    return out;
}

namespace {

std::vector<int> set_union(const std::vector<int>& a, const std::vector<int>& b)
{
    std::vector<int> u;
    std::set_union(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(u));
    return u;
}

bool intersects(const std::vector<int>& a, const std::vector<int>& b)
{
    size_t i = 0, j = 0;
    while (i < a.size() && j < b.size()) {
        if (a[i] == b[j]) return true;
        if (a[i] < b[j]) ++i; else ++j;
    }
    return false;
}

}  // namespace

std::vector<FusedBlock> fuse(const std::vector<std::vector<int>>& gate_bits, int nbits, int width)
{
    std::vector<FusedBlock> out;
    std::vector<FusedBlock> open;  // pairwise disjoint
    for (int gi = 0; gi < (int)gate_bits.size(); ++gi) {
        std::vector<int> q = gate_bits[gi];
        std::sort(q.begin(), q.end());
        std::vector<int> touched;
        for (int b = 0; b < (int)open.size(); ++b)
            if (intersects(open[b].qubits, q)) touched.push_back(b);
        if (width <= 0 || (int)q.size() > width) {
            for (int b : touched) out.push_back(open[b]);
            for (int j = (int)touched.size() - 1; j >= 0; --j) open.erase(open.begin() + touched[j]);
            out.push_back(FusedBlock{q, {gi}});
            continue;
        }
        // keep the largest touched blocks that still fit with the gate
        std::vector<int> order = touched;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return open[a].qubits.size() > open[b].qubits.size();
        });
        std::vector<int> u = q;
        std::vector<char> chosen(open.size(), 0);
        for (int b : order) {
            auto cand = set_union(u, open[b].qubits);
            if ((int)cand.size() <= width) {
                u = cand;
                chosen[b] = 1;
            }
        }
        FusedBlock merged;
        merged.qubits = u;
        std::vector<FusedBlock> keep;
        for (int b = 0; b < (int)open.size(); ++b) {
            const bool is_touched = std::find(touched.begin(), touched.end(), b) != touched.end();
            if (!is_touched) {
                keep.push_back(open[b]);
            } else if (chosen[b]) {
                merged.gates.insert(merged.gates.end(), open[b].gates.begin(), open[b].gates.end());
            } else {
                out.push_back(open[b]);  // must precede the gate
            }
        }
        merged.gates.push_back(gi);
        keep.push_back(merged);
        open.swap(keep);
    }
    for (auto& b : open) out.push_back(b);

    if (width <= 0) return out;
    // Move each block back past disjoint blocks and merge it into the first
    // earlier block whose union with it fits.
    std::vector<FusedBlock> res;
    for (auto& b : out) {
        bool merged = false;
        for (int e = (int)res.size() - 1; e >= 0; --e) {
            auto u = set_union(res[e].qubits, b.qubits);
            if ((int)u.size() <= width) {
                res[e].qubits = u;
                res[e].gates.insert(res[e].gates.end(), b.gates.begin(), b.gates.end());
                merged = true;
                break;
            }
            if (intersects(res[e].qubits, b.qubits)) break;
        }
        if (!merged) res.push_back(b);
    }
    (void)nbits;
    return res;
}

int phase_run_pivot(const FusedBlock& b, const std::vector<std::vector<int>>& gate_bits)
{
    std::vector<int> common;
    bool any = false;
    const size_t ndiag = b.gates.size() - (b.trailing_pair ? 1 : 0);
    for (size_t j = 0; j < ndiag; ++j) {
        const auto& q = gate_bits[b.gates[j]];
        if (q.size() != 2) continue;
        std::vector<int> s = q;
        std::sort(s.begin(), s.end());
        if (!any) {
            common = s;
            any = true;
        } else {
            std::vector<int> c;
            std::set_intersection(common.begin(), common.end(), s.begin(), s.end(), std::back_inserter(c));
            common.swap(c);
        }
    }
    if (!any) return -1;
    return common.empty() ? -2 : common[0];
}

std::vector<FusedBlock> fuse_runs(const std::vector<std::vector<int>>& gate_bits,
                                  const std::vector<unsigned char>& kinds, int nbits, int width)
{
    const int ng = (int)gate_bits.size();
    std::vector<FusedBlock> out;
    std::vector<int> pending;   // regular gates since the last run
    auto flush = [&] {
        if (pending.empty()) return;
        std::vector<std::vector<int>> sub;
        for (int g : pending) sub.push_back(gate_bits[g]);
        for (auto b : fuse(sub, nbits, width)) {
            for (auto& gi : b.gates) gi = pending[gi];
            out.push_back(b);
        }
        pending.clear();
    };
    auto emit = [&](FusedBlock& run) {
        for (int g : run.gates)
            for (int q : gate_bits[g])
                if (std::find(run.qubits.begin(), run.qubits.end(), q) == run.qubits.end()) run.qubits.push_back(q);
        std::sort(run.qubits.begin(), run.qubits.end());
        flush();
        out.push_back(run);
    };
    int i = 0;
    while (i < ng) {
        if (kinds[i] == kGateSwap && gate_bits[i].size() == 2) {
            // consecutive swaps while their qubit pairs stay disjoint
            std::vector<int> used;
            int j = i;
            while (j < ng && kinds[j] == kGateSwap && gate_bits[j].size() == 2 &&
                   gate_bits[j][0] != gate_bits[j][1] &&
                   std::find(used.begin(), used.end(), gate_bits[j][0]) == used.end() &&
                   std::find(used.begin(), used.end(), gate_bits[j][1]) == used.end()) {
                used.push_back(gate_bits[j][0]);
                used.push_back(gate_bits[j][1]);
                ++j;
            }
            if (j - i >= 2) {
                FusedBlock run;
                run.swap_run = true;
                for (int g = i; g < j; ++g) run.gates.push_back(g);
                emit(run);
                i = j;
            } else {
                pending.push_back(i++);
            }
            continue;
        }
        if (kinds[i] != kGateDiagonal) {
            pending.push_back(i++);
            continue;
        }
        int j = i;
        bool small = true;
        while (j < ng && kinds[j] == kGateDiagonal) {
            small = small && gate_bits[j].size() <= 2;
            ++j;
        }
        FusedBlock run;
        run.phase_run = true;
        for (int g = i; g < j; ++g) run.gates.push_back(g);
        if (j - i < kMinPhaseRun || !small || phase_run_pivot(run, gate_bits) == -2) {
            for (int g = i; g < j; ++g) pending.push_back(g);
            i = j;
            continue;
        }
        if (j < ng && gate_bits[j].size() == 1 && kinds[j] == kGateGeneral) {
            run.gates.push_back(j);
            run.trailing_pair = true;
            ++j;
        }
        emit(run);
        i = j;
    }
    flush();
    return out;
}

}  // namespace q1g
