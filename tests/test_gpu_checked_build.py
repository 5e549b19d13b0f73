"""The bounds-checked library (GKRT_CHECKED: every node, triangle and instance index tested
against its array before the access) passes the traversal parity suites unchanged, with no
bounds error recorded: a sanitizer-style run, since compute-sanitizer is not available."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECKED = os.path.join(ROOT, "gknextengine_gb300", "_lib", "libgkrt_checked.so")


def test_checked_build_runs_the_parity_suites():
    if not os.path.exists(CHECKED):
        pytest.fail("libgkrt_checked.so missing: __graft_entry__.build() builds it")
    env = dict(os.environ, GKRT_LIBRARY=CHECKED)
    probe = ("from gknextengine_gb300 import native; L = native.load(); "
             "assert L._name.endswith('libgkrt_checked.so'), L._name; print('checked')")
    r = subprocess.run([sys.executable, "-c", probe], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "checked" in r.stdout, r.stderr[-2000:]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
                        "tests/test_gpu_parity.py", "tests/test_gpu_wide_bvh.py", "tests/test_gpu_refit.py",
                        "tests/test_gpu_nee.py"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-2000:])
    assert " passed" in r.stdout
