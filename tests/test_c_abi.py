"""The C ABI from a C program (tests/c/gkrt_c_abi.c, compiled with gcc against include/gkrt.h
and linked with libgkrt.so): host-only calls on CPU, one rt pass with ids read back on GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gknextengine_gb300", "_lib")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    if not os.path.exists(os.path.join(LIBDIR, "libgkrt.so")):
        pytest.skip("libgkrt.so not built")
    out = str(tmp_path_factory.mktemp("cabi") / "gkrt_c_abi")
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "gkrt_c_abi.c"), "-L", LIBDIR, "-lgkrt", f"-Wl,-rpath,{LIBDIR}", "-lm",
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_c_client_host_calls(exe):
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


@pytest.mark.gpu
def test_c_client_rt_pass(exe):
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
