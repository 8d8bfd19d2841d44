"""bench.py's reference arm on the CPU: one JSON line in the contract's shape
(the same metric and unit as the GPU arm, impl "reference", a cpu_baseline
describing the run, an e2e object with zero copies); ranks other than 0 of a
multi-rank launch exit 0 without output."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                           "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)


def test_reference_arm_line():
    p = _run({})
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("elasticity hex8 128^3")


def test_reference_arm_other_ranks_are_silent():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0 and not p.stdout.strip()


def test_e2e_summary_takes_the_median_window():
    # seven windows of five steps, two of them slowed by other traffic on the host link: the median window sets
    # the value, every window is listed, the link-only copy is the median of its samples
    import bench
    steps, elements, h2d, d2h = 5, 2_097_152, 51_520_536, 4_160_317_536
    win = [0.1105, 0.1105, 0.2930, 0.1104, 0.1105, 0.2956, 0.1106]
    links = [0.0215, 0.0780, 0.0216]
    d = bench.e2e_summary(win, links, steps, elements, h2d, d2h)
    assert d["value"] == elements * steps / 0.1105 and d["unit"] == bench.UNIT
    assert d["windows"] == 7 and d["steps"] == 5 and d["statistic"] == "median of 7 windows of 5 steps"
    assert d["window_ms_per_step"] == [22.1, 22.1, 58.6, 22.08, 22.1, 59.12, 22.12]
    assert d["h2d_bytes_per_step"] == h2d and d["d2h_bytes_per_step"] == d2h
    assert abs(d["link_d2h_gbs"] - d2h / 0.0216 / 1e9) < 1e-9
    assert abs(d["link_bound_frac"] - 0.0216 / (0.1105 / 5)) < 1e-12
