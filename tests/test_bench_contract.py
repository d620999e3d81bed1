"""The bench's JSON contract on the CPU. The reference arm prints one line
with the metric, its unit and direction, `impl: reference`, a cpu_baseline
describing the run and an e2e object without host-device bytes; ranks other
than 0 of a multi-process launch exit 0 without work or output. The clock
record and the DRAM-traffic lookup the GPU arm adds parse as intended."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--qubits", "14", "--depth", "2",
        "--steps", "1", "--warmup", "0"]


def _env(**extra):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env.update(extra)
    return env


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run(ARGS, capture_output=True, text=True, timeout=600, env=_env(), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "gates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["config"]["qubits"] == 14 and d["config"]["depth"] == 2
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = subprocess.run(ARGS, capture_output=True, text=True, timeout=120,
                       env=_env(RANK="1", WORLD_SIZE="2", LOCAL_RANK="1"), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


def test_clock_summary_reads_median_and_reasons():
    """nvidia-smi lines (clocks.sm, clocks.max.sm, power, active mask, then the
    four reasons) become the JSON line's clocks object; unparsable lines are
    skipped."""
    s = _bench().ClockSampler(0)
    s.lines = ["2070, 2070, 910.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "2055, 2070, 1399.8, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "[N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "2040, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "garbage"]
    assert s.summary() == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_dram_traffic_table_lookup():
    b = _bench()
    assert b.dram_traffic("fused_tc_c64", 30) == 16313143296.0
    assert b.dram_traffic("fused_tc_c64", 26) == 1019571456.0
    assert b.dram_traffic("fused_tc_c64", 17) is None
    assert b.dram_traffic("no_such_kernel", 30) is None
