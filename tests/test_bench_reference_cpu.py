"""bench.py's reference arm: the CPU restatement of the path timed on the host
cores, one bounded sample per step.  On a reduced workload (20k points, 100
keypoints, 2,000 RANSAC trials; ~10 s on 8 cores) the arm prints exactly one
JSON line with the keys of the benchmark contract, its `value` is the pair
fraction the step covered over the step's measured time, and ranks other
than 0 exit without work or output."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(args, env=None):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          timeout=600, env=env, cwd=ROOT)


def _json_lines(out):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def test_reference_arm_prints_one_contract_line(oracle):  # the fixture builds the oracle the arm runs
    r = _bench(["--impl", "reference", "--steps", "1", "--warmup", "0", "--points", "20000", "--keypoints", "100",
                "--ransac-iters", "2000"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "pair registrations/s" and d["unit"] == "pairs/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["cpu_baseline"]["cores"] >= 1 and "sample" in d["cpu_baseline"]
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # a step is the measured sample: the rate is its pair fraction over its time
    step_s = d["ms_per_step"] / 1000.0
    assert 0 < step_s < 600
    assert abs(d["value"] - d["pair_fraction_per_step"] / step_s) <= 1e-9 * d["value"]


def test_reference_arm_other_ranks_exit_without_output():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = _bench(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"], env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert _json_lines(r.stdout) == []
