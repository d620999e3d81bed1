"""Continuous-batching request loop over the GPU engine.

Requests (circuits with a shot count and a seed) arrive over time. A request
is admitted as soon as a slot is free and its device memory fits in the HBM
budget, so work of requests that arrive while others run overlaps on the
device. Each slot owns a CUDA stream (a VectorState per qubit count, reused)
and runs the request's lowered plan, its measurement and the result
download. Admission is FIFO: the oldest waiting request is admitted first,
and a request that does not fit waits for memory to be freed.

This has no reference counterpart. The reference runs one circuit at a time
(src/circuit.rs:562-641); each request here computes exactly what
`Circuit.execute(shots, Rng(seed))` computes for it alone.
"""
import collections
import threading
import time

import numpy as np

from .vectorstate import Rng, VectorState


class Request:
    """A circuit to run `shots` times with Rng(seed).  init_seed: start from
    a random normalised state drawn on the device (re, im i.i.d. N(0,1),
    VectorState.fill_random_normal) instead of |0...0>."""
    __slots__ = ("rid", "circuit", "shots", "seed", "init_seed", "arrival", "admitted", "done", "result", "error")

    def __init__(self, rid, circuit, shots, seed, arrival=0.0, init_seed=None):
        self.rid = rid
        self.circuit = circuit
        self.shots = shots
        self.seed = seed
        self.init_seed = init_seed
        self.arrival = arrival
        self.admitted = None
        self.done = None
        self.result = None
        self.error = None

    def state_bytes(self):
        amp = 16 if self.circuit.precision == "c128" else 8
        # the state plus sampling scratch (chunk sums, uniforms, outcomes)
        return (amp << self.circuit.nr_qbits) + 48 * self.shots + (8 << max(self.circuit.nr_qbits - 8, 0))

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


def prepare_state(req, st):
    """The request's initial state in `st`: |0...0> or its random state (one
    column: a reused state may hold the basis columns a previous request's
    measure_all left)."""
    st.reset_all()
    if req.init_seed is not None:
        st.fill_random_normal(req.init_seed)


def run_alone(req):
    """What the request computes when nothing else runs: Circuit.execute
    from its initial state."""
    c = req.circuit
    st = VectorState(c.nr_qbits, req.shots, c.precision)
    prepare_state(req, st)
    c.execute_with(req.shots, Rng(req.seed), st)
    return c.cstate().copy()


class Server:
    """Admits requests by HBM budget into `slots` concurrent device workers."""

    # 16 slots by default: a slot's thread spends much of each request on the
    # host (plan lowering, waits on its own stream), so more slots keep the
    # device busier; on the serving mix 8 / 12 / 16 slots gave 970 / 1069 /
    # 1126 circuits/s
    def __init__(self, hbm_budget_bytes, slots=16):
        self.budget = int(hbm_budget_bytes)
        self.slots = int(slots)
        self.used = 0
        self.pending = collections.deque()
        self.cv = threading.Condition()
        self.closing = False
        self.completed = []
        self.peak_used = 0
        self.peak_inflight = 0
        self.inflight = 0
        self.threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        self._stream_of = {}
        for t in self.threads:
            t.start()

    # ------------------------------------------------------------ client
    def submit(self, req):
        if req.state_bytes() > self.budget:
            raise ValueError(f"request {req.rid} needs {req.state_bytes()} bytes, above the HBM budget")
        with self.cv:
            self.pending.append(req)
            self.cv.notify_all()

    def close(self):
        with self.cv:
            self.closing = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()

    # ------------------------------------------------------------ worker
    def _admit(self):
        """Oldest pending request that fits, or None (FIFO head only)."""
        if self.pending and self.used + self.pending[0].state_bytes() <= self.budget:
            req = self.pending.popleft()
            self.used += req.state_bytes()
            self.peak_used = max(self.peak_used, self.used)
            self.inflight += 1
            self.peak_inflight = max(self.peak_inflight, self.inflight)
            return req
        return None

    def _worker(self, slot):
        import torch
        stream = torch.cuda.Stream()
        states = {}
        while True:
            with self.cv:
                req = self._admit()
                while req is None:
                    if self.closing and not self.pending:
                        return
                    self.cv.wait(timeout=0.05)
                    req = self._admit()
            req.admitted = time.perf_counter()
            try:
                c = req.circuit
                key = (c.nr_qbits, req.shots, c.precision)
                st = states.get(key)
                if st is None:
                    # kept for later requests of the same shape: allocating
                    # (and freeing, which synchronises the device) per request
                    # would stall the other slots
                    st = VectorState(c.nr_qbits, req.shots, c.precision)
                    st.set_stream(stream.cuda_stream)
                    states[key] = st
                prepare_state(req, st)
                c.execute_with(req.shots, Rng(req.seed), st)
                req.result = c.cstate().copy()
            except Exception as e:    # reported with the request
                req.error = repr(e)
            req.done = time.perf_counter()
            with self.cv:
                self.used -= req.state_bytes()
                self.inflight -= 1
                self.completed.append(req)
                self.cv.notify_all()


def serve(requests, rate_hz, hbm_budget_bytes, slots=16, seed=0):
    """Replay `requests` as a Poisson stream of mean rate `rate_hz` and serve
    them.  Returns (requests in completion order, wall seconds, server)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests))
    srv = Server(hbm_budget_bytes, slots)
    t0 = time.perf_counter()
    at = t0
    for req, gap in zip(requests, gaps):
        at += gap
        delay = at - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        req.arrival = at
        srv.submit(req)
    srv.close()
    wall = time.perf_counter() - t0
    return srv.completed, wall, srv


def latency_stats(done):
    lat = np.array([r.latency for r in done if r.error is None])
    if len(lat) == 0:
        return {}
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "completed": int(len(lat)),
            "errors": int(sum(1 for r in done if r.error is not None))}


def mixed_requests(count, seed, qmin=10, qmax=26, dmin=5, dmax=50, shots=4096):
    """Seeded mix of GHZ, QFT-on-a-random-state and random U3/CX brick
    circuits, complex64 fused."""
    from . import workloads
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(qmin, qmax + 1))
        kind = int(rng.integers(3))
        init_seed = None
        if kind == 0:
            c = workloads.ghz(n)
        elif kind == 1:
            # the QFT of a random state whose amplitudes are i.i.d. N(0,1),
            # drawn on the device from init_seed
            c = workloads.qft(n)
            init_seed = int(rng.integers(2 ** 62))
        else:
            c = workloads.brick(n, int(rng.integers(dmin, dmax + 1)), int(rng.integers(2 ** 62)))
        out.append(Request(i, c.freeze(), shots, int(rng.integers(2 ** 62)), init_seed=init_seed))
    return out


def device_seconds(requests):
    """Device time of each request run alone (the sum of its kernels'
    CUDA-event times): the bound on how many requests per second the device
    can serve, whatever the batching."""
    total = 0.0
    states = {}
    for req in requests:
        c = req.circuit
        key = (c.nr_qbits, req.shots, c.precision)
        st = states.get(key)
        if st is None:
            st = states[key] = VectorState(c.nr_qbits, req.shots, c.precision)
        st.profile(True)
        st.profile_report(reset=True)
        prepare_state(req, st)
        c.execute_with(req.shots, Rng(req.seed), st)
        total += sum(v["ms"] for v in st.profile_report(reset=True).values()) / 1e3
        st.profile(False)
    return total
