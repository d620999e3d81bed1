"""Autotuner for gate runs: fusion width, dense-block kernel and the
tensor-core tiling.

For one circuit structure (qubit count, precision and the qubits of each
gate), every candidate is lowered to a plan and timed on a scratch state of
the same shape; the fastest one is remembered for that structure.  A
candidate is a fusion width, whether complex64 dense blocks run on the
tensor cores or the CUDA cores, and for tensor-core plans the tiling of
their passes (q1g_plan_set_tc_tiling): whether two blocks may share a pass,
how many tile positions of a pair may lie at large-page strides, and how
many bank conflicts an unpadded one-box tile may take before it is padded.
Matrices do not affect the choice: the plan's passes and their cost depend
only on the structure.
"""
import time

from .vectorstate import Plan, VectorState

DEFAULT_TILING = Plan.DEFAULT_TC_TILING
# tensor-core tilings tried beside the default (four consumer groups, pairs
# whose second block reads operands the first stored) at the widest fusion
# width: three blocks per pass; two groups with pairs through the staged
# tile, through registers (warp shuffles) or through stored operands; no
# pairs; pairs over fewer large pages; a tighter conflict slack
TC_TILINGS = (DEFAULT_TILING, (5, 8, 4), (1, 8, 2), (2, 8, 2), (3, 8, 2), (0, 8, 2), (4, 5, 4), (4, 8, 2))

# (fusion width, dense complex64 blocks on tensor cores, tiling)
CANDIDATES_C64 = tuple((5, True, t) for t in TC_TILINGS) + (
    (4, True, DEFAULT_TILING), (3, True, DEFAULT_TILING),
    (4, False, DEFAULT_TILING), (3, False, DEFAULT_TILING), (2, False, DEFAULT_TILING), (0, False, DEFAULT_TILING))
CANDIDATES_C128 = tuple((w, False, DEFAULT_TILING) for w in (0, 1, 2, 3))

_cache = {}


def structure_key(nr_bits, precision, gate_bits):
    return (nr_bits, precision, hash(tuple(tuple(b) for b in gate_bits)))


def make_plan(nr_bits, gate_bits, width, tensor_cores, tiling, kinds=None):
    plan = Plan(nr_bits, gate_bits, width, tensor_cores=tensor_cores, kinds=kinds)
    if tiling != DEFAULT_TILING:
        plan.set_tc_tiling(*tiling)
    return plan


def tune(nr_bits, precision, gate_bits, mats_flat, reps=2, candidates=None, kinds=None):
    """Best (fusion_width, tensor_cores, tiling) for this structure, by
    device time.  kinds: per gate, Plan.KIND_* (phase and swap runs)."""
    key = structure_key(nr_bits, precision, gate_bits) + (tuple(int(k) for k in kinds or ()),)
    if key in _cache:
        return _cache[key]
    if candidates is None:
        candidates = CANDIDATES_C64 if precision == "c64" else CANDIDATES_C128
    scratch = VectorState(nr_bits, 1, precision)
    timings = []
    for width, tc, tiling in candidates:
        plan = make_plan(nr_bits, gate_bits, width, tc, tiling, kinds=kinds)
        scratch.reset_all()
        scratch.apply_plan(plan, mats_flat)          # warm-up: first touch, caches
        scratch.synchronize()
        best = float("inf")
        for _ in range(reps):
            scratch.reset_all()
            t0 = time.perf_counter()
            scratch.apply_plan(plan, mats_flat)
            scratch.synchronize()
            best = min(best, time.perf_counter() - t0)
        timings.append((best, width, tc, tiling, plan.nblocks))
    del scratch
    timings.sort(key=lambda x: x[0])
    choice = (timings[0][1], timings[0][2], timings[0][3])
    _cache[key] = choice
    tune.last_timings = [{"seconds": t, "fusion_width": w, "tensor_cores": c, "pairs": tl[0],
                          "max_high_positions": tl[1], "conflict_slack": tl[2], "blocks": nb}
                         for t, w, c, tl, nb in timings]
    return choice


tune.last_timings = []


def clear():
    _cache.clear()
