"""The C ABI from plain C: include/rrtl_cuda.h compiles as strict C99 and a
C client linked against librrtl_gb300.so makes the host-only calls (no
device), as a caller binding the library over FFI would."""
import os
import shutil
import subprocess

import pytest

from rrtl_gb300 import build
from rrtl_gb300.workloads import counter

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c99_client_links_and_runs(tmp_path):
    lib = build.build()
    exe = tmp_path / "capi_client"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_client", "capi_client.c"), "-o", str(exe), lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    js = tmp_path / "counter.json"
    js.write_text(counter().to_json())
    r = subprocess.run([str(exe), str(js), "Counter"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "c client ok" in r.stdout
