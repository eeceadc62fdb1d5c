"""CPU checks of bench.py's command-line contract: the reference arm's JSON
line (the CPU oracle on a bounded sample), its silence on ranks other than 0,
and the timed start step both arms share."""
import argparse
import importlib.util
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("fs3d_bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_bench(*argv, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *argv], capture_output=True, text=True,
                          env=e, timeout=600)


def test_timed_start_step_is_shared_and_moves_with_the_warmup():
    bench = load_bench()
    ns = lambda **kw: argparse.Namespace(**{"warmup": 3, "segment": 64, "timed_from": 640, "no_autotune": False,
                                            **kw})
    # three warm-up segments, six trial segments and one plain segment fit before step 640
    assert bench.untimed_segments(ns()) == 10
    assert bench.untimed_segments(ns(warmup=1)) == 10  # at least three warm-up segments
    assert bench.untimed_segments(ns(warmup=6)) == 6 + bench.TUNE_SEGMENTS + 1
    assert bench.untimed_segments(ns(warmup=6, no_autotune=True)) == 10
    assert bench.untimed_segments(ns(timed_from=1280)) == 20


def test_reference_arm_prints_one_contract_line():
    r = run_bench("--impl", "reference", "--steps", "2", "--warmup", "3", "--cpu-budget", "1")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "dtype",
              "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["config"]["timed_from_step"] == 640
    assert d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["unit"] == d["unit"]


def test_reference_arm_is_silent_on_other_ranks():
    r = run_bench("--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--cpu-budget", "1",
                  env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
