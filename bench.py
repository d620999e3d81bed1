"""Benchmark: 30-qubit random U3/CX brick circuit, gates/s and shots/s.

Workload (one step): |0...0> on 30 qubits, 24 brick layers -- U3(theta, phi,
lambda) on every qubit with angles uniform in [0, 2pi) from the seed, then CX
on (2i, 2i+1) in even layers and (2i+1, 2i+2) in odd layers (1068 gates) --
in complex64 with gates fused into blocks of <= 5 qubits, then 1,000,000
Z-basis shots sampled from the final state.  The same circuit in plain
complex128 mode (one gate per pass) is timed once beside it, and the fused
complex64 result is compared with it on the device (1 - fidelity, max |d amp|,
outcome TV).

`value` = circuit gates / device time of the fused gate passes (state resident
in HBM, 8 GiB > L2, so no flush is needed); `e2e` = the same metric through
the public Circuit API with host matrices in and the classical results out.

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "30q random-circuit gates/s & %HBM peak, FP32-fused vs FP64 plain; shots/s"


def brick_gates(n, depth, seed):
    """(name, params, bits) of the U3/CX brick circuit."""
    rng = np.random.default_rng(seed)
    out = []
    for layer in range(depth):
        for q in range(n):
            out.append(("U3", [float(v) for v in rng.uniform(0.0, 2 * math.pi, 3)], [q]))
        for q in range(0 if layer % 2 == 0 else 1, n - 1, 2):
            out.append(("CX", [], [q, q + 1]))
    return out


def world_aggregate(local_ms, local_units, dist, device):
    """(max over ranks of the elapsed ms, sum over ranks of the units done).
    Replicas do not exchange data; only these two numbers are reduced."""
    import torch
    ms = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(ms, op=dist.ReduceOp.MAX)
        dist.all_reduce(units, op=dist.ReduceOp.SUM)
    return float(ms[0]), float(units[0])


def dram_traffic(kernel, qubits):
    """DRAM bytes per launch of `kernel` at `qubits` from the ncu summaries in
    profiles/dram_traffic.txt (None when no capture covers it)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and int(parts[1]) == qubits:
                return float(parts[2])
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_cpu():
    """The host's CPU model and its total cores (lscpu, else platform)."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":", 1)[0].strip() == "Model name":
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"model": model or platform.processor() or platform.machine(), "total_cores": os.cpu_count(),
            "arch": platform.machine()}


def oracle_gate_times(n_sample, seed):
    """Seconds per U3 and per CX of the oracle (single-threaded complex128
    restatement of the reference's algorithm) at n_sample qubits, each the
    mean over gates spread across the qubit positions (the reference's cost
    depends on the position: a 1-qubit gate loops over 2^q row blocks).
    One untimed gate touches the state first."""
    from oracle import oracle as orc
    from q1tsim_gb300 import gates as G
    rng = np.random.default_rng(seed)
    s = orc.OracleState.new(n_sample, 1)
    s.apply_gate(G.H().matrix(), [0])
    n = n_sample
    u3 = []
    for q in (0, n // 2, n - 1):
        m = G.U3(*rng.uniform(0.0, 2 * math.pi, 3)).matrix()
        t0 = time.perf_counter()
        s.apply_gate(m, [q])
        u3.append(time.perf_counter() - t0)
    cx = []
    for q in (0, n - 2):
        t0 = time.perf_counter()
        s.apply_gate(G.CX().matrix(), [q, q + 1])
        cx.append(time.perf_counter() - t0)
    return sum(u3) / len(u3), sum(cx) / len(cx), sum(u3) + sum(cx)


def oracle_rate(n_sample, n_full, depth, seed):
    """The oracle's gates/s on the brick circuit at n_full qubits, estimated
    from its per-gate-type times at n_sample qubits: (U3 count x U3 time + CX
    count x CX time) x 2^(n_full - n_sample), since every gate touches all
    2^n amplitudes."""
    t_u3, t_cx, spent = oracle_gate_times(n_sample, seed)
    gl = brick_gates(n_full, depth, seed)
    n_u3 = sum(1 for nm, _, _ in gl if nm == "U3")
    n_cx = len(gl) - n_u3
    t_full = (n_u3 * t_u3 + n_cx * t_cx) * 2.0 ** (n_full - n_sample)
    return len(gl) / t_full, t_u3, t_cx, spent


def cpu_baseline(n_sample, seed, n_full, depth, n_cached=22):
    """The oracle on a state larger than the host's caches (n_sample
    qubits, complex128), with the same estimate from a state that fits in
    them (n_cached qubits) beside it."""
    rate, t_u3, t_cx, spent = oracle_rate(n_sample, n_full, depth, seed)
    rate_c, t_u3c, t_cxc, _ = oracle_rate(n_cached, n_full, depth, seed)
    return {"value": rate, "unit": "gates/s", "cores": 1, "kind": "port", "host": host_cpu(),
            "sample": f"oracle (reference algorithm, 1 thread; the reference is single-threaded) at "
                      f"{n_sample} qubits ({(16 << n_sample) / 2 ** 30:g} GiB complex128): 3 U3 and 2 CX at "
                      f"spread positions, {t_u3:.3f} s per U3 and {t_cx:.3f} s per CX ({spent:.1f} s), "
                      f"weighted by the circuit's U3/CX counts and scaled by 2^({n_sample}-{n_full})",
            "in_cache": {"qubits": n_cached, "value": rate_c, "s_per_u3": t_u3c, "s_per_cx": t_cxc,
                         "note": f"{(16 << n_cached) / 2 ** 20:g} MiB state, within the host's caches"}}


def qft_leg(args):
    """QFT on a random normalised 28-qubit state (re, im i.i.d.
    N(0,1) from the seed, drawn on the device), complex64 fused against
    complex128 plain."""
    import torch
    from q1tsim_gb300 import Plan, VectorState, workloads
    n = args.qft_qubits
    qc = workloads.qft(n, measure=False)
    bits = [op[2] for op in qc.ops]
    kinds = [op[1].plan_kind() for op in qc.ops]   # controlled-phase ladders, final swaps
    mats = np.concatenate([np.ascontiguousarray(op[1].matrix()).ravel() for op in qc.ops]).view(np.float64)
    out = {"workload": f"QFT ({len(bits)} gates: H, CU1(pi/2^k), Swap) on a random N(0,1) {n}-qubit state",
           "gates": len(bits)}
    def random_state(prec):
        s = VectorState(n, 1, prec)
        s.fill_random_normal(args.seed + 5)
        return s

    for prec, width in (("c128", 0), ("c64", args.fusion)):
        plan = Plan(n, bits, width, kinds=kinds if width else None)
        st = random_state(prec)
        st.apply_plan(plan, mats)      # warm-up
        # the best of three runs, each from the drawn state
        dt = float("inf")
        for _ in range(3):
            st.fill_random_normal(args.seed + 5)
            st.synchronize()
            t0 = time.perf_counter()
            st.apply_plan(plan, mats)
            st.synchronize()
            dt = min(dt, time.perf_counter() - t0)
        out[prec] = {"ms": dt * 1e3, "passes": plan.nblocks, "gates_per_s": len(bits) / dt}
        out["_" + prec] = st
    acc = out.pop("_c128").compare(out.pop("_c64"))
    out["accuracy_c64_vs_c128"] = acc
    torch.cuda.empty_cache()
    return out


def brick32_leg(args):
    """32-qubit U3/CX brick, depth 24, complex64 with fused
    5-qubit tensor-core blocks (f16 hi/lo halves), then 10^6 Z-basis shots; 1 - F and
    outcome TV against a complex128 run of the same circuit on the GPU
    (32 GiB + 64 GiB of HBM; the complex128 run alone takes about 20 s)."""
    import torch
    from q1tsim_gb300 import Plan, Rng, VectorState
    from q1tsim_gb300 import gates as G
    n = 32
    gl = brick_gates(n, 24, args.seed + 11)
    gates = [(G.by_name(nm, p), b) for nm, p, b in gl]
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    out = {"workload": f"random U3/CX brick circuit, {n} qubits, depth 24 ({len(gates)} gates), complex64 fused "
                       f"k<={args.fusion}, then 1000000 Z shots; complex128 run on the GPU as the reference",
           "gates": len(gates)}
    fused = VectorState(n, 1, "c64")
    plan = Plan(n, bits, args.fusion)
    fused.apply_plan(plan, mats)            # warm-up
    fused.reset_all()
    fused.synchronize()
    t0 = time.perf_counter()
    fused.apply_plan(plan, mats)
    fused.synchronize()
    dt = time.perf_counter() - t0
    res = np.zeros(1_000_000, dtype=np.uint64)
    fused.peek_all_into(list(range(n)), res, rng=Rng(args.seed + 13))
    fused.synchronize()
    t1 = time.perf_counter()
    fused.peek_all_into(list(range(n)), res, rng=Rng(args.seed + 14))
    fused.synchronize()
    st = time.perf_counter() - t1
    out["c64"] = {"ms": dt * 1e3, "passes": plan.nblocks, "gates_per_s": len(gates) / dt,
                  "shots_per_s": 1e6 / st}
    plain = VectorState(n, 1, "c128")
    pplan = Plan(n, bits, 0)
    plain.synchronize()
    t0 = time.perf_counter()
    plain.apply_plan(pplan, mats)
    plain.synchronize()
    dt = time.perf_counter() - t0
    out["c128"] = {"ms": dt * 1e3, "passes": pplan.nblocks, "gates_per_s": len(gates) / dt}
    out["accuracy_c64_vs_c128"] = plain.compare(fused)
    del plain, fused
    torch.cuda.empty_cache()
    return out


def brick16_leg(args):
    """16-qubit U3/CX brick, 20 layers, measure_all over 8192
    runs, histogram -- on the GPU (complex128 plain and complex64 fused) and
    in full on the CPU oracle."""
    from oracle import oracle as orc
    from q1tsim_gb300 import Rng, workloads
    res = {"workload": "16-qubit U3/CX brick, 20 layers (470 gates), measure_all over 8192 runs, histogram"}
    for prec, width in (("c128", 0), ("c64", args.fusion)):
        c = workloads.brick(16, 20, args.seed + 3, precision=prec, fusion_width=width)
        c.execute(8192, Rng(1))
        t0 = time.perf_counter()
        for k in range(5):
            c.execute(8192, Rng(k))
            h = c.histogram()
        res[prec] = {"ms": (time.perf_counter() - t0) / 5 * 1e3, "distinct_outcomes": len(h)}
    c = workloads.brick(16, 20, args.seed + 3, precision="c128", fusion_width=0)
    t0 = time.perf_counter()
    c.execute_with(8192, Rng(1), orc.OracleState.new(16, 8192))
    c.histogram()
    cpu_ms = (time.perf_counter() - t0) * 1e3
    res["cpu_baseline"] = {"ms": cpu_ms, "cores": 1, "kind": "port",
                           "sample": "the full workload on the oracle (reference algorithm, 1 thread)"}
    res["speedup_c128_vs_cpu"] = cpu_ms / res["c128"]["ms"]
    return res


def batch_leg(args):
    """Independent circuits (8-20 qubits, depth 10-40, U3/CX/CZ,
    one mid-circuit measurement + conditional X, 1024 runs each) in one
    persistent launch replayed from a CUDA graph."""
    from q1tsim_gb300 import workloads
    from q1tsim_gb300.batch import Batch
    t0 = time.perf_counter()
    circuits = workloads.batch_workload(args.batch_circuits, args.seed + 11)
    b = Batch(4)
    for i, c in enumerate(circuits):
        b.add(c, 1024, args.seed + i)
    setup_s = time.perf_counter() - t0
    b.run()   # builds the device program and the graph
    dev_ms, wall_ms = [], []
    for _ in range(max(args.steps, 3)):
        w0 = time.perf_counter()
        b.run()
        wall_ms.append((time.perf_counter() - w0) * 1e3)
        dev_ms.append(b.info()["last_ms"])
    ngates = sum(1 for c in circuits for op in c.ops if op[0] in ("gate", "cgate"))
    ms = statistics.median(dev_ms)
    info = b.info()
    peak, peak_kind = peaks()
    # algorithmic bytes counted by the kernel itself (amplitude passes and
    # classical words) over the device time of the launch
    achieved = info["traffic_bytes"] / (ms / 1e3) / 1e9
    # CPU: the oracle runs the first circuits one by one
    from oracle import oracle as orc
    from q1tsim_gb300.vectorstate import Rng
    sample = circuits[:12]
    c0 = time.perf_counter()
    for i, c in enumerate(sample):
        c.execute_with(1024, Rng(args.seed + i), orc.OracleState.new(c.nr_qbits, 1024))
    cpu_s = time.perf_counter() - c0
    work = lambda cs: sum((2 ** c.nr_qbits) * sum(1 for op in c.ops if op[0] in ("gate", "cgate")) for c in cs)
    cpu_total_s = cpu_s * work(circuits) / work(sample)
    return {"workload": f"{len(circuits)} circuits, 8-20 qubits, depth 10-40 U3/CX/CZ, mid-circuit measure + "
                        "conditional X, 1024 runs each, complex64, fusion k<=4",
            "circuits": len(circuits), "gates": ngates, "device_ms": ms, "e2e_ms": statistics.median(wall_ms),
            "circuits_per_s": len(circuits) / (ms / 1e3), "gates_per_s": ngates / (ms / 1e3),
            "e2e_circuits_per_s": len(circuits) / (statistics.median(wall_ms) / 1e3),
            "arena_gib": info["arena_bytes"] / 2 ** 30, "lowered_ops": info["ops"],
            "roofline": {"bound": "hbm", "kernel": "k_batch", "traffic_gb": info["traffic_bytes"] / 1e9,
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak},
            "launches_per_run": 1, "setup_s": setup_s,
            "cpu_baseline": {"value": len(circuits) / cpu_total_s, "unit": "circuits/s", "cores": 1, "kind": "port",
                             "sample": f"oracle on the first {len(sample)} circuits in {cpu_s:.2f} s, scaled to "
                                       "the batch by sum(gates x 2^n)"}}


def serving_leg(args):
    """A Poisson stream of GHZ, QFT-on-a-random-N(0,1)-state and brick
    circuits, 10-26 qubits, depth 5-50, 4096 shots, complex64 fused, admitted
    by HBM budget into concurrent slots: at the offered 2000 circuits/s and
    at 1000/s, with the device-time bound of the same requests beside them."""
    from q1tsim_gb300.serving import device_seconds, latency_stats, mixed_requests, serve
    reqs = mixed_requests(args.serve_requests, args.seed + 23)
    dev_s = device_seconds(reqs)
    out = {"requests": len(reqs), "slots": 16, "hbm_budget_gib": 64,
           "device_seconds": dev_s, "device_bound_circuits_per_s": len(reqs) / dev_s,
           "workload": "Poisson mix of GHZ, QFT on a random state (re, im i.i.d. N(0,1), drawn on the device) "
                       "and U3/CX brick circuits, 10-26 qubits, depth 5-50, 4096 shots, complex64 fused"}
    for rate in (2000.0, 1000.0):
        reqs = mixed_requests(args.serve_requests, args.seed + 23)
        done, wall, srv = serve(reqs, rate_hz=rate, hbm_budget_bytes=64 << 30, slots=16, seed=args.seed)
        st = latency_stats(done)
        first = min(r.arrival for r in done)
        last = max(r.done for r in done)
        st.update({"offered_rate_hz": rate, "circuits_per_s": len(done) / (last - first),
                   "peak_inflight": srv.peak_inflight, "peak_budget_gib": srv.peak_used / 2 ** 30})
        out[f"at_{int(rate)}_per_s"] = st
    return out


def workload_config(args):
    """The headline workload, named the same way on both arms: the circuit
    and the shots (how an arm computes it goes in further keys)."""
    ngates = len(brick_gates(args.qubits, args.depth, args.seed))
    return {"workload": f"random U3/CX brick circuit, {args.qubits} qubits, depth {args.depth} ({ngates} gates), "
                        f"then {args.shots} Z shots",
            "qubits": args.qubits, "depth": args.depth, "gates": ngates, "shots": args.shots}


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU algorithm (the oracle port: the Rust
    reference cannot be built on this image) on the host cores.  Each step
    times a bounded sample at args.cpu_qubits qubits (a state larger than the
    host's caches) and scales it to the full circuit."""
    if rank != 0:
        return
    n_s = args.cpu_qubits
    for _ in range(args.warmup):
        oracle_rate(n_s, args.qubits, args.depth, args.seed)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rates.append(oracle_rate(n_s, args.qubits, args.depth, args.seed)[0])
    dt = time.perf_counter() - t0
    rate = statistics.median(rates)
    sample = (f"oracle (reference algorithm, 1 thread; the reference is single-threaded) per step: 3 U3 and "
              f"2 CX at spread positions on a {n_s}-qubit complex128 state ({(16 << n_s) / 2 ** 30:g} GiB); "
              f"gates/s of the {args.qubits}-qubit circuit from its U3/CX counts, scaled by "
              f"2^({n_s}-{args.qubits}); median over steps")
    line = {"metric": METRIC, "impl": "reference", "value": rate, "unit": "gates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(workload_config(args), computation="complex128, gate by gate"),
            "cpu_baseline": {"value": rate, "unit": "gates/s", "cores": 1, "kind": "port", "sample": sample,
                             "host": host_cpu()},
            "e2e": {"value": rate, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def plain_kernel_leg(n, bits, mats, stream, barrier, ngates=120):
    """The first `ngates` gates of the circuit, one pass per gate, in
    complex64, complex128 (double-float arithmetic, the default) and
    complex128 with FP64 arithmetic: per kernel, launches, time per launch and
    achieved HBM bandwidth (bytes of the amplitudes each launch touches, read
    and written) against the measured peak."""
    from q1tsim_gb300 import Plan, VectorState
    peak, peak_kind = peaks()
    sub = bits[:ngates]
    ndbl = sum(2 * (1 << len(b)) ** 2 for b in sub)
    out = {"gates": len(sub), "peak_gbs": peak, "peak_kind": peak_kind}
    for label, prec, exact in (("c64", "c64", False), ("c128", "c128", False), ("c128_fp64", "c128", True)):
        st = VectorState(n, 1, prec)
        st.set_stream(stream.cuda_stream)
        if exact:
            st.set_fp64_exact()
        plan = Plan(n, sub, 0)
        st.apply_plan(plan, mats[:ndbl])      # warm-up: allocation, first touch
        barrier()
        st.profile(True)
        st.profile_report(reset=True)
        st.apply_plan(plan, mats[:ndbl])
        prof = st.profile_report(reset=True)
        st.profile(False)
        ks = {}
        for k, v in prof.items():
            if not k.startswith(("pair", "phase", "dense")):
                continue
            gbs = v["bytes"] / (v["ms"] / 1e3) / 1e9
            ks[k] = {"launches": v["launches"], "ms_per_launch": round(v["ms"] / v["launches"], 4),
                     "gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
        out[label] = ks
        del st
        barrier()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=24)
    ap.add_argument("--shots", type=int, default=1_000_000)
    ap.add_argument("--fusion", type=int, default=5)
    ap.add_argument("--seed", type=int, default=20240601)
    ap.add_argument("--no-plain", action="store_true", help="skip the complex128 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-qubits", type=int, default=26)
    ap.add_argument("--batch-circuits", type=int, default=4096)
    ap.add_argument("--serve-requests", type=int, default=1000)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-circuits leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-qft", action="store_true", help="skip the 28-qubit QFT accuracy leg")
    ap.add_argument("--no-brick16", action="store_true", help="skip the 16-qubit CPU-runnable leg")
    ap.add_argument("--qft-qubits", type=int, default=28)
    ap.add_argument("--no-brick32", action="store_true", help="skip the 32-qubit complex64 vs complex128 leg")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from q1tsim_gb300 import Circuit, Plan, Rng, VectorState
    from q1tsim_gb300 import gates as G

    n, shots = args.qubits, args.shots
    gl = brick_gates(n, args.depth, args.seed + rank)
    gates = [(G.by_name(nm, p), b) for nm, p, b in gl]
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    ngates = len(gates)

    stream = torch.cuda.Stream()
    fused = VectorState(n, shots, "c64")
    fused.set_stream(stream.cuda_stream)
    plan = Plan(n, bits, args.fusion)
    res = np.zeros(shots, dtype=np.uint64)
    cbits = list(range(n))

    def gate_step():
        fused.reset_all()
        fused.apply_plan(plan, mats)

    def shot_step():
        fused.peek_all_into(cbits, res, rng=Rng(args.seed + 7))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 1)):
        gate_step()
        shot_step()
    barrier()

    # ---- gates: K device-resident circuit runs, CUDA events on the stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for _ in range(args.steps):
                gate_step()
            ev1.record(stream)
        barrier()
    gate_ms = ev0.elapsed_time(ev1)
    # ---- shots: K samplings of 1e6 shots from the resident state
    barrier()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    t_host = time.perf_counter()
    for _ in range(args.steps):
        shot_step()
    s1.record(stream)
    barrier()
    shot_wall = time.perf_counter() - t_host
    shot_ms = s0.elapsed_time(s1)

    gate_ms_max, gates_all = world_aggregate(gate_ms, args.steps * ngates, dist, "cuda")
    shot_ms_max, shots_all = world_aggregate(shot_wall * 1e3, args.steps * shots, dist, "cuda")
    value = gates_all / (gate_ms_max / 1e3)
    shots_per_s = shots_all / (shot_ms_max / 1e3)

    # ---- per-kernel profile of one step (CUDA events around every launch)
    fused.profile(True)
    fused.profile_report(reset=True)
    gate_step()
    shot_step()
    prof = fused.profile_report(reset=True)
    fused.profile(False)
    launches_per_step = sum(v["launches"] for v in prof.values())
    gate_kernels = {k: v for k, v in prof.items() if k.startswith(("dense", "pair", "phase", "fused"))}
    dom_name = max(gate_kernels, key=lambda k: gate_kernels[k]["ms"])
    dom = gate_kernels[dom_name]
    achieved = (dom["bytes"] / dom["launches"]) / (dom["ms"] / dom["launches"] / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = dram_traffic(dom_name, n)
    # fused blocks of >= 3 qubits run on the tensor cores, one or two per launch
    tc_blocks = sum(1 for qb, _ in plan.blocks() if len(qb) >= 3)

    # ---- plain complex128 run of the same circuit, and the accuracy of c64
    plain_info, accuracy = None, None
    if not args.no_plain:
        plain = VectorState(n, shots, "c128")
        plain.set_stream(stream.cuda_stream)
        pplan = Plan(n, bits, 0)
        plain.apply_plan(pplan, mats)   # warm-up (allocation + first touch)
        plain.reset_all()
        barrier()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        plain.apply_plan(pplan, mats)
        p1.record(stream)
        barrier()
        plain_ms = p0.elapsed_time(p1)
        gate_step()
        accuracy = plain.compare(fused)
        plain_info = {"gates_per_s": ngates / (plain_ms / 1e3), "ms_per_circuit": plain_ms,
                      "fused_speedup": (ngates / (gate_ms_max / args.steps / 1e3)) / (ngates / (plain_ms / 1e3))}
        # complex128 fused into 3-qubit blocks (double-float warp tiles)
        f128 = VectorState(n, shots, "c128")
        f128.set_stream(stream.cuda_stream)
        fplan = Plan(n, bits, 3)
        f128.apply_plan(fplan, mats)   # warm-up
        f128.reset_all()
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        f128.apply_plan(fplan, mats)
        f1.record(stream)
        barrier()
        f128_ms = f0.elapsed_time(f1)
        acc128 = plain.compare(f128)
        plain_info["fused_c128"] = {"fusion_width": 3, "blocks": fplan.nblocks, "ms_per_circuit": f128_ms,
                                    "gates_per_s": ngates / (f128_ms / 1e3), "speedup_vs_plain": plain_ms / f128_ms,
                                    "max_abs_diff_vs_plain": acc128["max_abs_diff"],
                                    "infidelity_vs_plain": acc128["infidelity"]}
        del f128
        del plain

    # ---- plain (unfused) gate kernels: the first layers, per-kernel profile
    plain_kernels = None if args.no_plain else plain_kernel_leg(n, bits, mats, stream, barrier)

    # ---- end to end through the public Circuit API (host in, results out)
    circ = Circuit(n, n, precision="c64", fusion_width=args.fusion)
    for g, b in gates:
        circ.add_gate(g, b)
    circ.measure_all(cbits)
    del fused
    circ.execute(shots, Rng(args.seed))
    barrier()
    circ.q_state.transfer_bytes(reset=True)
    t0 = time.perf_counter()
    for k in range(args.steps):
        circ.execute(shots, Rng(args.seed + k))
        _ = circ.cstate()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_ms_max, e2e_gates = world_aggregate(e2e_s * 1e3, args.steps * ngates, dist, "cuda")
    e2e_value = e2e_gates / (e2e_ms_max / 1e3)
    # bytes the engine itself copied over the host link during the timed
    # executions (matrices, tables, uniforms in; outcomes, words, flags out)
    h2d_all, d2h_all = circ.q_state.transfer_bytes()
    h2d, d2h = h2d_all // args.steps, d2h_all // args.steps

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_qubits, args.seed, n, args.depth)
    del circ
    batched = None if args.no_batch else batch_leg(args)
    serving = None if args.no_serve else serving_leg(args)
    qft = None if args.no_qft else qft_leg(args)
    brick16 = None if args.no_brick16 else brick16_leg(args)
    brick32 = None if args.no_brick32 else brick32_leg(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": gate_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {**workload_config(args), "computation": f"complex64 fused k<={args.fusion}",
                       "fusion_width": args.fusion, "fused_blocks": plan.nblocks,
                       "tensor_core_passes": dom["launches"] if dom_name == "fused_tc_c64" else None,
                       "parallelism": f"replicas{world}",
                       "l2": (f"state {(8 << n) / 2 ** 30:g} GiB > L2 (129 MB), no flush needed" if (8 << n) > 129e6
                              else "state smaller than L2")},
            "shots_per_s": shots_per_s, "shot_sampling_ms": shot_ms / args.steps,
            "plain_c128": plain_info, "accuracy_c64_vs_c128": accuracy,
            "plain_kernels": plain_kernels,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "launch_ms": dom["ms"] / dom["launches"],
                         "bytes_per_launch": dom["bytes"] / dom["launches"],
                         "blocks_per_launch": (round(tc_blocks / dom["launches"], 3)
                                               if dom_name.startswith("fused") else 1)},
            "kernels_per_step": {k: {"launches": v["launches"], "ms": round(v["ms"], 4)} for k, v in prof.items()},
            "gpu_launches": launches_per_step * args.steps,
            "e2e": {"value": e2e_value, "unit": "gates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "batched": batched,
            "serving": serving,
            "qft_random_state": qft,
            "cpu_runnable_16q": brick16,
            "brick_32q": brick32,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
