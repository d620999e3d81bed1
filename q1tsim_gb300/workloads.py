"""Seeded synthetic circuits of the benchmark configurations.

Every generator returns a `Circuit` built through the public API (gates by
object, as a q1tsim user would add them) so the same circuit can run on the
GPU state, in a batch, through the serving loop, or on the CPU oracle.
"""
import math

import numpy as np

from . import gates as G
from .circuit import Circuit


def brick(n, depth, seed, precision="c64", fusion_width=5, measure=True):
    """U3 on every qubit, then CX on (2i, 2i+1) in even layers and
    (2i+1, 2i+2) in odd layers; angles uniform in [0, 2pi) from the seed."""
    rng = np.random.default_rng(seed)
    c = Circuit(n, n, precision=precision, fusion_width=fusion_width)
    for layer in range(depth):
        for q in range(n):
            c.add_gate(G.U3(*rng.uniform(0.0, 2 * math.pi, 3)), [q])
        for q in range(0 if layer % 2 == 0 else 1, n - 1, 2):
            c.add_gate(G.CX(), [q, q + 1])
    if measure:
        c.measure_all(list(range(n)))
    return c


def qft(n, precision="c64", fusion_width=5, measure=True):
    """Quantum Fourier transform: H, controlled phases CP(pi/2^k) = CU1, then
    the final swaps (q1tsim names the controlled phase CU1)."""
    c = Circuit(n, n, precision=precision, fusion_width=fusion_width)
    for j in range(n):
        c.add_gate(G.H(), [j])
        for k in range(j + 1, n):
            c.add_gate(G.CU1(math.pi / 2 ** (k - j)), [k, j])
    for j in range(n // 2):
        c.add_gate(G.Swap(), [j, n - 1 - j])
    if measure:
        c.measure_all(list(range(n)))
    return c


def ghz(n, precision="c64", fusion_width=5, measure=True):
    """H on qubit 0 and a CX chain."""
    c = Circuit(n, n, precision=precision, fusion_width=fusion_width)
    c.add_gate(G.H(), [0])
    for q in range(n - 1):
        c.add_gate(G.CX(), [q, q + 1])
    if measure:
        c.measure_all(list(range(n)))
    return c


def mid_measure_circuit(n, depth, seed, nmeasure=1):
    """Layers of seeded U3 / CX / CZ gates with `nmeasure` mid-circuit Z
    measurements: measurement j on a random qubit into classical bit j,
    followed by an X on that qubit conditioned on the result (from the second
    on, every other one conditioned on the previous bit being 0 instead);
    then measure_all into classical bits nmeasure .. nmeasure+n-1."""
    rng = np.random.default_rng(seed)
    c = Circuit(n, n + nmeasure, precision="c64", fusion_width=4)
    mid = int(rng.integers(1, depth))
    mq = int(rng.integers(n))
    extra = [(int(rng.integers(1, depth + 1)), int(rng.integers(n))) for _ in range(nmeasure - 1)]
    meas = sorted([(mid, mq)] + extra, key=lambda x: x[0])
    for layer in range(depth):
        for q in range(n):
            c.add_gate(G.U3(*rng.uniform(0.0, 2 * math.pi, 3)), [q])
        start = layer % 2
        for q in range(start, n - 1, 2):
            c.add_gate(G.CX() if rng.random() < 0.5 else G.CZ(), [q, q + 1])
        for j, (at, q) in enumerate(meas):
            if at == layer + 1:
                c.measure(q, j)
                if j > 0 and j % 2 == 0:
                    c.add_conditional_gate([j - 1], 0, G.X(), [q])
                else:
                    c.add_conditional_gate([j], 1, G.X(), [q])
    c.measure_all(list(range(nmeasure, n + nmeasure)))
    return c


def batch_workload(ncircuits, seed, qmin=8, qmax=20, dmin=10, dmax=40):
    """Circuits with qubit count uniform in [qmin, qmax] and depth uniform in
    [dmin, dmax], each with a mid-circuit measurement and conditional X."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(ncircuits):
        n = int(rng.integers(qmin, qmax + 1))
        d = int(rng.integers(dmin, dmax + 1))
        out.append(mid_measure_circuit(n, d, int(rng.integers(2 ** 63))))
    return out
