"""bench.py's output contract on CPU: the reference arm's JSON line (the
float64 oracle timed on the host cores) and the clock sampler's choice of
samples."""
import importlib.util
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench_module():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_sampler_keeps_timed_region_samples():
    b = _bench_module()

    class _Proc:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            pass

    idle = ["0", "1100", "2070", "150", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]
    load = ["0", "2070", "2070", "900", "0x4", "Not Active", "Not Active", "Not Active", "Active"]
    c = b.ClockSampler(0)
    c.proc = _Proc()
    c.t_mark = 10.0
    c.samples = [(9.0, idle), (10.2, load), (10.25, load)]
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["samples"] == 2
    assert out["reasons"] == ["sw_power_cap"]
    # a region shorter than the interval keeps whatever was sampled
    c = b.ClockSampler(0)
    c.proc = _Proc()
    c.t_mark = 20.0
    c.samples = [(9.0, idle)]
    assert c.stop()["sm_mhz"] == 1100.0


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "leapfrog steps/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "logistic_regression_N1000_d25_rmhmc_fisher_4096chains"
