"""CPU checks of bench.py's output contract: the reference arm (the
reference's own module, or the oracle port where that is not built, timed on
host cores) prints one JSON line with the keys a benchmark harness reads, on
the same metric as the GPU arm, and a rank other than 0 of a multi-process
launch exits 0 without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _reference_arm(env_extra, timeout):
    env = dict(os.environ, **env_extra)
    # a 64^3 grid with the job's queries per cell keeps this CPU test short
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                           "--grid", "64"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def _json_lines(stdout):
    return [json.loads(l) for l in stdout.splitlines() if l.startswith("{")]


def test_reference_arm_prints_the_driver_line():
    sys.path.insert(0, ROOT)
    import bench
    r = _reference_arm({}, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "queries/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_do_no_work():
    r = _reference_arm({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"}, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert _json_lines(r.stdout) == []
