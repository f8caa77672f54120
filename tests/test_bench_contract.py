"""CPU checks of bench.py's reporting helpers: the per-launch DRAM traffic table
(profiles/eval_traffic.json) is well formed and is looked up by workload and colouring,
the roofline block computes its fraction from the instrumented pass's bytes and
event time against the measured copy bandwidth, and the reference arm prints the
contract's line without ever mapping the CUDA library."""
import importlib.util
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    saved = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = saved
    return mod


def test_traffic_table_well_formed():
    with open(os.path.join(ROOT, "profiles", "eval_traffic.json")) as f:
        table = json.load(f)
    workloads = [k for k in table if not k.startswith("_")]
    assert {"torus_1024x512_qem", "heightfield_4096_aniso", "batch_256_qem"} <= set(workloads)
    for w in workloads:
        for coloring, entry in table[w].items():
            assert coloring in ("jp", "order", "squeeze")
            assert isinstance(entry["bytes_per_launch"], int) and entry["bytes_per_launch"] > 0
            assert 0.3 < entry["traffic_over_algorithmic"] < 3.0
            assert entry["how"]


def test_traffic_lookup_by_colouring(bench):
    b, how = bench.eval_traffic("torus_1024x512_qem", "order")
    assert b > 0 and "sampled sweeps" in how
    assert bench.eval_traffic("torus_1024x512_qem", "jp") == (None, None)
    assert bench.eval_traffic("no_such_workload", "jp") == (None, None)


def test_roofline_block_fraction(bench):
    tot = {"eval_bytes": 6.0e9, "eval_ms": 2.0, "eval_launches": 10}
    r = bench.roofline_block(False, tot, "heightfield_4096_aniso", "jp")
    peak = r["peak"]
    assert r["kernel"] == "eval_kernel" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(3000.0)          # 6 GB in 2 ms
    assert r["frac"] == pytest.approx(3000.0 / peak)
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(6.0e8)
    assert r["avg_launch_us"] == pytest.approx(200.0)
    assert r["traffic"] is not None
    # the persistent kernel is a different launch unit: no traffic figure for it
    tot_p = dict(tot, sweep_kernel_ms=4.0, sweep_kernel_launches=3)
    rp = bench.roofline_block(True, tot_p, "heightfield_4096_aniso", "jp")
    assert rp["kernel"] == "sweep_run_kernel" and rp["traffic"] is None
    assert rp["achieved"] == pytest.approx(1500.0)


RUNNER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "icosphere_l5_iso", "--steps", "2", "--warmup", "1"]
runpy.run_path("bench.py", run_name="__main__")
with open("/proc/self/maps") as f:
    libs = sorted({l.split()[-1] for l in f if ".so" in l})
print("MAPPED " + " ".join(libs))
"""


def test_reference_arm_line_and_no_cuda_library():
    """The reference arm on a small workload: one JSON line with the contract's keys, a
    cpu_baseline describing this run, an e2e block with no copies, a connected clustering
    -- and the process never maps the CUDA library (the arm runs the oracle's threaded
    restatement only)."""
    import subprocess
    r = subprocess.run([sys.executable, "-c", RUNNER], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1
    assert d["unit"] == "items/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "icosphere_l5_iso"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["energy"]["all_clusters_connected"] is True
    mapped = [l for l in r.stdout.splitlines() if l.startswith("MAPPED ")][0]
    assert "libacvd_gb300" not in mapped, mapped
