"""Autotuner for gate runs: fusion width and dense-block kernel.

For one circuit structure (qubit count, precision and the qubits of each
gate), every candidate (fusion width, tensor cores or CUDA cores) is lowered
to a plan and timed on a scratch state of the same shape. The fastest one is
remembered for that structure. Matrices do not affect the choice: the plan's
passes and their cost depend only on the structure.
"""
import time

import numpy as np

from .vectorstate import Plan, VectorState

# (fusion width, dense complex64 blocks on tensor cores)
CANDIDATES_C64 = ((5, True), (4, True), (3, True), (4, False), (3, False), (2, False), (0, False))
CANDIDATES_C128 = ((0, False), (1, False), (2, False), (3, False))

_cache = {}


def structure_key(nr_bits, precision, gate_bits):
    return (nr_bits, precision, hash(tuple(tuple(b) for b in gate_bits)))


def tune(nr_bits, precision, gate_bits, mats_flat, reps=2, candidates=None, kinds=None):
    """Best (fusion_width, tensor_cores) for this structure, by device time.
    kinds: per gate, Plan.KIND_* (phase and swap runs)."""
    key = structure_key(nr_bits, precision, gate_bits) + (tuple(int(k) for k in kinds or ()),)
    if key in _cache:
        return _cache[key]
    if candidates is None:
        candidates = CANDIDATES_C64 if precision == "c64" else CANDIDATES_C128
    scratch = VectorState(nr_bits, 1, precision)
    timings = []
    for width, tc in candidates:
        plan = Plan(nr_bits, gate_bits, width, tensor_cores=tc, kinds=kinds)
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
        timings.append((best, width, tc, plan.nblocks))
    del scratch
    timings.sort()
    choice = (timings[0][1], timings[0][2])
    _cache[key] = choice
    tune.last_timings = [{"seconds": t, "fusion_width": w, "tensor_cores": c, "passes": nb}
                         for t, w, c, nb in timings]
    return choice


tune.last_timings = []


def clear():
    _cache.clear()
