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

std::vector<FusedBlock> fuse_greedy(const std::vector<std::vector<int>>& gate_bits, int nbits, int width)
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

std::vector<FusedBlock> fuse_windows(const std::vector<std::vector<int>>& gate_bits, int nbits, int width)
{
    const int ng = (int)gate_bits.size();
    std::vector<FusedBlock> out;
    if (ng == 0) return out;
    if (width <= 0) return fuse_greedy(gate_bits, nbits, width);
    // the gates of each qubit in order, and how far each qubit is done
    std::vector<std::vector<int>> perq(nbits);
    for (int g = 0; g < ng; ++g)
        for (int q : gate_bits[g]) perq[q].push_back(g);
    std::vector<int> ptr(nbits, 0);
    auto next_of = [&](const std::vector<int>& p, int q) { return p[q] < (int)perq[q].size() ? perq[q][p[q]] : -1; };
    auto ready = [&](const std::vector<int>& p, int g) {
        for (int q : gate_bits[g])
            if (next_of(p, q) != g) return false;
        return true;
    };
    // every gate whose qubits lie in `in` and whose predecessors are done,
    // taken in a valid order; p advances past them
    auto absorb = [&](const std::vector<char>& in, const std::vector<int>& qs, std::vector<int>& p,
                      std::vector<int>* taken) {
        int count = 0;
        for (bool progress = true; progress;) {
            progress = false;
            for (int q : qs) {
                for (;;) {
                    const int g = next_of(p, q);
                    if (g < 0 || !ready(p, g)) break;
                    bool inside = true;
                    for (int x : gate_bits[g]) inside = inside && in[x];
                    if (!inside) break;
                    for (int x : gate_bits[g]) ++p[x];
                    if (taken) taken->push_back(g);
                    ++count;
                    progress = true;
                }
            }
        }
        return count;
    };
    int remaining = ng;
    std::vector<char> in(nbits, 0);
    while (remaining > 0) {
        // a ready gate wider than a block goes alone
        int wide = -1;
        for (int q = 0; q < nbits && wide < 0; ++q) {
            const int g = next_of(ptr, q);
            if (g >= 0 && (int)gate_bits[g].size() > width && ready(ptr, g)) wide = g;
        }
        if (wide >= 0) {
            FusedBlock b;
            b.qubits = gate_bits[wide];
            std::sort(b.qubits.begin(), b.qubits.end());
            b.gates = {wide};
            for (int x : gate_bits[wide]) ++ptr[x];
            out.push_back(b);
            --remaining;
            continue;
        }
        // candidate qubit sets: every window of `width` consecutive qubits,
        // and for every ready gate the set grown from its qubits by the ready
        // gates that add the fewest new qubits
        std::vector<std::vector<int>> cands;
        for (int a = 0; a + width <= nbits; ++a) {
            std::vector<int> w;
            for (int q = a; q < a + width; ++q) w.push_back(q);
            cands.push_back(w);
        }
        if (nbits < width) {
            std::vector<int> w;
            for (int q = 0; q < nbits; ++q) w.push_back(q);
            cands.push_back(w);
        }
        for (int q0 = 0; q0 < nbits; ++q0) {
            const int g0 = next_of(ptr, q0);
            if (g0 < 0 || !ready(ptr, g0) || gate_bits[g0][0] != q0) continue;
            std::vector<int> s = gate_bits[g0];
            std::sort(s.begin(), s.end());
            std::vector<int> p = ptr;
            std::fill(in.begin(), in.end(), 0);
            for (int x : s) in[x] = 1;
            absorb(in, s, p, nullptr);
            for (;;) {
                int best = -1, best_new = width + 1;
                for (int q = 0; q < nbits; ++q) {
                    const int g = next_of(p, q);
                    if (g < 0 || !ready(p, g)) continue;
                    int add = 0;
                    for (int x : gate_bits[g]) add += in[x] ? 0 : 1;
                    if (add == 0 || (int)s.size() + add > width) continue;
                    if (add < best_new) {
                        best_new = add;
                        best = g;
                    }
                }
                if (best < 0) break;
                for (int x : gate_bits[best])
                    if (!in[x]) {
                        in[x] = 1;
                        s.push_back(x);
                    }
                std::sort(s.begin(), s.end());
                absorb(in, s, p, nullptr);
            }
            cands.push_back(s);
        }
        // the candidate that absorbs the most gates
        int best_count = -1;
        std::vector<int> best_set;
        for (const auto& c : cands) {
            std::fill(in.begin(), in.end(), 0);
            for (int x : c) in[x] = 1;
            std::vector<int> p = ptr;
            const int cnt = absorb(in, c, p, nullptr);
            if (cnt > best_count) {
                best_count = cnt;
                best_set = c;
            }
        }
        std::fill(in.begin(), in.end(), 0);
        for (int x : best_set) in[x] = 1;
        FusedBlock b;
        absorb(in, best_set, ptr, &b.gates);
        if (b.gates.empty()) throw std::logic_error("window fusion made no progress");
        for (int g : b.gates)
            for (int x : gate_bits[g])
                if (std::find(b.qubits.begin(), b.qubits.end(), x) == b.qubits.end()) b.qubits.push_back(x);
        std::sort(b.qubits.begin(), b.qubits.end());
        remaining -= (int)b.gates.size();
        out.push_back(b);
    }
    return out;
}

std::vector<FusedBlock> fuse(const std::vector<std::vector<int>>& gate_bits, int nbits, int width)
{
    auto greedy = fuse_greedy(gate_bits, nbits, width);
    if (width <= 1) return greedy;
    auto windows = fuse_windows(gate_bits, nbits, width);
    return windows.size() < greedy.size() ? windows : greedy;
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
