"""The oracle once more, built at -O0 with gcc's undefined-behaviour checks
(every report aborts): its own tests, golden vectors included, must pass
unchanged, so no result of the checker depends on the optimiser or on
undefined behaviour (signed overflow, shifts past the width, misaligned or
out-of-bounds access that the checks see)."""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_suite_under_ubsan_at_O0(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    so = tmp_path / "liboracle_ubsan.so"
    r = subprocess.run(["gcc", "-O0", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
                        "-fsanitize=undefined", "-fno-sanitize-recover=undefined", "-shared", "-o", str(so),
                        os.path.join(ROOT, "oracle", "fs3d_oracle.c"), "-lm"], capture_output=True, text=True)
    if r.returncode != 0 and "ubsan" in r.stderr:
        pytest.skip("gcc's undefined-behaviour runtime is not installed")
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, FS3D_ORACLE_SO=str(so), UBSAN_OPTIONS="print_stacktrace=1")
    # -s: a report ends the process at once, before pytest would print what it captured
    t = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-s", "-p", "no:cacheprovider",
                        os.path.join(ROOT, "tests", "test_oracle.py")],
                       capture_output=True, text=True, env=env, cwd=ROOT, timeout=900)
    out = t.stdout + t.stderr
    assert t.returncode == 0 and "runtime error" not in out, out[-3000:]
