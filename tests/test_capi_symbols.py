"""The C-ABI library loads on a host without a GPU and exports every entry
point include/rrtl_cuda.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from rrtl_gb300 import build, sim

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rrtl_cuda.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:rrtl_status|const char\*)\s+(rrtl_[a-z_0-9]+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    assert set(names) == set(sim.EXPORTS)


def test_last_error_is_empty_after_a_successful_call():
    from rrtl_gb300.workloads import counter

    build.build()
    sim.word_jit_emit(counter(), "Counter")  # no device needed
    assert sim.lib().rrtl_last_error() == b""


def test_null_arguments_fail_with_codes_not_crashes():
    build.build()
    L = sim.lib()
    assert L.rrtl_ctx_create(0, None) == 1  # RRTL_E_ARG: out is null
    assert b"E_ARG" in L.rrtl_last_error()
    assert L.rrtl_batch_eval(None) == 1


def test_every_entry_point_rejects_null_arguments():
    """Each rrtl_status call made with every argument NULL (or 0) returns
    RRTL_E_ARG before touching a device; destroying NULL is a no-op."""
    lib = ctypes.CDLL(build.build())  # fresh function objects, no argtypes
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = re.findall(r"^rrtl_status\s+(rrtl_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", text, re.M)
    assert len(protos) >= 50
    for name, params in protos:
        n = len([p for p in params.split(",") if p.strip() and p.strip() != "void"])
        st = getattr(lib, name)(*([None] * n))
        if name.endswith("_destroy"):
            assert st == 0, name
        else:
            assert st == 1, (name, st, sim.lib().rrtl_last_error())


def test_last_error_is_per_thread():
    """A failure on one thread leaves another thread's message untouched."""
    import threading

    build.build()
    L = sim.lib()
    assert L.rrtl_batch_eval(None) == 1
    before = L.rrtl_last_error()
    seen = {}

    def other():
        seen["start"] = L.rrtl_last_error()
        L.rrtl_ctx_create(0, None)
        seen["after"] = L.rrtl_last_error()

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen["start"] == b"" and b"out is null" in seen["after"]
    assert L.rrtl_last_error() == before


def test_without_a_device_the_context_fails_with_a_code():
    """On a host without a usable GPU the engine refuses at context creation
    with RRTL_E_DEVICE and the CUDA error text; it has no CPU fallback."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    build.build()
    L = sim.lib()
    out = ctypes.c_void_p()
    assert L.rrtl_ctx_create(0, ctypes.byref(out)) == 4  # RRTL_E_DEVICE
    assert L.rrtl_last_error().startswith(b"E_DEVICE") and out.value is None
    with pytest.raises(sim.RrtlError) as e:
        sim.Context(0)
    assert e.value.status == 4


def test_a_missing_library_fails_loudly(monkeypatch, tmp_path):
    """The Python mirror has no fallback: without the built library every
    entry raises."""
    monkeypatch.setattr(sim, "LIB_PATH", str(tmp_path / "librrtl_gb300.so"))
    monkeypatch.setattr(sim, "_lib", None)
    with pytest.raises(RuntimeError, match="is missing"):
        sim.lib()
    with pytest.raises(RuntimeError, match="is missing"):
        sim.bitslice_json("{}", "Top")
