"""The oracle once more, built at -O0 with gcc's undefined-behaviour checks
and, where its runtime is installed, its address checks (every report
aborts): its own tests, golden vectors included, must pass unchanged, so no
result of the checker depends on the optimiser, on undefined behaviour
(signed overflow, shifts past the width) or on a read or write outside a
buffer."""
import os
import shutil
import subprocess
import sys

import pytest

from sanitize_util import report_found, sanitize_flags

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_suite_under_sanitizers_at_O0(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    flags, env_add, _ = sanitize_flags()
    so = tmp_path / "liboracle_checked.so"
    r = subprocess.run(["gcc", "-O0", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", *flags,
                        "-shared", "-o", str(so), os.path.join(ROOT, "oracle", "fs3d_oracle.c"), "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0 and "san" in r.stderr:
        pytest.skip("gcc's sanitizer runtime is not installed")
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, FS3D_ORACLE_SO=str(so), **env_add)
    # -s: a report ends the process at once, before pytest would print what it captured
    t = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-s", "-p", "no:cacheprovider",
                        os.path.join(ROOT, "tests", "test_oracle.py")],
                       capture_output=True, text=True, env=env, cwd=ROOT, timeout=900)
    out = t.stdout + t.stderr
    assert t.returncode == 0 and not report_found(out), out[-3000:]
