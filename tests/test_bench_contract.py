"""The benchmark's reference arm runs on the host cores only, so its one-line JSON
contract is checked here: the keys and types every line carries, the reference arm's
own fields, and that a rank other than 0 prints nothing."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "3", "--warmup", "3"], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return [ln for ln in out.stdout.splitlines() if ln.strip()]


def test_reference_arm_prints_one_contract_line():
    lines = _run({"RANK": "0", "WORLD_SIZE": "1", "LOCAL_RANK": "0"})
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key, typ in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int),
                     ("steps", int), ("warmup", int), ("ms_per_step", float),
                     ("higher_is_better", bool), ("scaling", str), ("dtype", str),
                     ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(d[key], typ), key
    assert d["impl"] == "reference" and d["vs_baseline"] is None
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert abs(d["ms_per_step"] - 1e3 / d["value"]) < 1e-9 * d["ms_per_step"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"] and "workload" in d["config"]
    assert d["e2e"] == {"value": d["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    assert _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_compute_roofline_arithmetic(monkeypatch):
    """The compute roofline of the bench line: the flop census per step over the step
    time against the measured FP32 and special-function peaks (replaced here by fixed
    numbers; nothing touches a device)."""
    import types

    import bench  # the repository root is on the path (conftest)
    from oxdna import runtime
    monkeypatch.setattr(runtime, "device_peaks", lambda stream=None: (60_000.0, 8_000.0))
    r = bench.compute_roofline(0.016, types.SimpleNamespace(cuda_stream=None))
    census = json.load(open(bench.FLOP_COUNTS))["workloads"]["8000nt"]
    assert r["flops_per_step"] == census["flops_per_step"] > 0
    assert abs(r["achieved"] - census["flops_per_step"] / 0.016e-3 / 1e12) < 1e-12
    assert r["peak"] == 60.0 and r["unit"] == "TFLOP/s"
    assert abs(r["frac"] - r["achieved"] / 60.0) < 1e-15
    sp = r["special"]
    assert sp["ops_per_step"] == sum(census["special_per_step"].values())
    assert abs(sp["frac"] - sp["achieved"] / 8_000.0) < 1e-15
    assert 0.0 < r["frac"] < 1.0 and 0.0 < sp["frac"] < 1.0


def test_clock_sampler_summarises_the_timed_window():
    """The clock record covers the sample taken just before the timed region and those
    inside it (a process-start sample long before it and samples after it are left out);
    throttle reasons are read from the flags; without nvidia-smi the record says
    'unsampled' instead of failing."""
    sys.path.insert(0, ROOT)
    import bench
    c = bench.ClockSampler(0)
    row = lambda mhz, hw="Not Active", pc="Not Active": ["0", str(mhz), "2070", "900", "0x0", hw,  # noqa: E731
                                                          "Not Active", "Not Active", pc]
    c.rows = [(1.0, row(1200)), (9.5, row(2070)), (10.1, row(2070, pc="Active")), (10.3, row(2070)),
              (20.0, row(800, hw="Active"))]
    c._t0, c._t1 = 10.0, 10.5
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    none = bench.ClockSampler(0)
    none._t0, none._t1 = 1.0, 2.0
    assert none.summary()["reasons"] == ["unsampled"]


def test_clock_sampler_reads_its_file_after_the_region():
    """The sampler's output lines (nvidia-smi's local timestamp first) parse into the
    sample time and the clock fields; an incomplete line is skipped and a timestamp that
    does not parse gives no time. Where nvidia-smi cannot be started, the region still
    runs and the record says 'unsampled'."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    t, f = bench.ClockSampler.parse("2026/12/04 23:01:02.250, 0, 2070, 2070, 901.5, 0x0000000000000000, "
                                    "Not Active, Not Active, Not Active, Not Active\n")
    assert abs(t - (time.mktime(time.strptime("2026/12/04 23:01:02", "%Y/%m/%d %H:%M:%S")) + 0.25)) < 1e-9
    assert f[:3] == ["0", "2070", "2070"] and len(f) == 9
    assert bench.ClockSampler.parse("2026/12/04 23:01:02.250, 0, 20") is None
    assert bench.ClockSampler.parse("garbled, 0, 2070, 2070, 900, 0x0, Active")[0] is None
    env_path = os.environ.get("PATH", "")
    os.environ["PATH"] = ""
    try:
        with bench.ClockSampler(0) as c:
            pass
    finally:
        os.environ["PATH"] = env_path
    assert c.summary()["reasons"] == ["unsampled"]
