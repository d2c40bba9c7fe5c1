"""The gate lowering run on the CPU exactly as the fused kernels consume it
(tests/native/gate_program_emu.cpp): staged piece blobs, slot rows and the
register commit list. The emulator checks the invariants the kernels rely
on without checking them (every group of a piece evaluated once through the
warp headers, no slot reuse clobbering a live net, no cell reading its own
piece's writes, records and commit rows holding their nets), and its
per-cycle output hash must equal the bit-parallel oracle's, for both piece
blobs the library builds (CTA barrier: lead warp 0.7, run cost 4; split
barrier: 0.85, 2) and several piece sizes and tile widths."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

from .helpers import crc32_netlist_json, oracle_bp_run

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = [os.path.join(HERE, "native", "gate_program_emu.cpp")] + [
    os.path.join(ROOT, "rrtl_gb300", "csrc", f) for f in ("gateprog.cpp", "design.cpp", "lower.cpp")]
LIB = os.path.join(HERE, "native", "_build", "libgate_emu.so")


@pytest.fixture(scope="module")
def emu():
    deps = SRC + [os.path.join(ROOT, "rrtl_gb300", "csrc", h) for h in
                  ("gateprog.h", "design.h", "lower.h", "json.h", "gate_dev.h", "stim.h")]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(p) for p in deps):
        from rrtl_gb300 import build as b

        cuda_home = os.path.dirname(os.path.dirname(b._nvcc()))
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{cuda_home}/include", "-o", LIB + ".tmp"]
                       + SRC, check=True)
        os.replace(LIB + ".tmp", LIB)
    L = ctypes.CDLL(LIB)
    P = ctypes.POINTER
    L.emu_gate_run.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.c_uint32, ctypes.c_double, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, P(ctypes.c_uint32),
                               P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32, P(ctypes.c_uint32),
                               P(ctypes.c_uint64), ctypes.c_char_p, ctypes.c_size_t]
    return L


def _emulate(L, js, top, od, stim, rec, lanes, cycles, seed, W, piece_groups, lead, run_cost, warps=16, lane_base=0):
    u32 = lambda a: np.ascontiguousarray(a, dtype=np.uint32)
    sig = u32([od.signal(n) for n, _, _ in stim])
    kind = u32([k for _, k, _ in stim])
    param = np.ascontiguousarray([p for _, _, p in stim], dtype=np.uint64)
    rsig = u32([od.signal(r) for r in rec])
    out = np.zeros(cycles, dtype=np.uint64)
    err = ctypes.create_string_buffer(512)
    P = ctypes.POINTER
    raw = js.encode()
    rc = L.emu_gate_run(raw, len(raw), top.encode(), W, piece_groups, warps, lead, run_cost, lanes, cycles, seed,
                        lane_base, len(stim), sig.ctypes.data_as(P(ctypes.c_uint32)),
                        kind.ctypes.data_as(P(ctypes.c_uint32)), param.ctypes.data_as(P(ctypes.c_uint64)), len(rec),
                        rsig.ctypes.data_as(P(ctypes.c_uint32)), out.ctypes.data_as(P(ctypes.c_uint64)), err, len(err))
    assert rc == 0, err.value.decode()
    return out


@pytest.fixture(scope="module")
def netlist():
    d, meta = gate_netlist(n_gates=6000, n_ff=256, n_pi=24, n_po=24, depth=14, seed=31)
    js = d.to_json()
    return js, meta, ob.OracleDesign(js, meta.top)


@pytest.mark.parametrize("W,piece_groups", [(8, 512), (8, 24), (4, 64), (2, 16), (1, 8)])
@pytest.mark.parametrize("lead,run_cost", [(0.7, 4.0), (0.85, 2.0)])
def test_emulated_program_equals_the_oracle(emu, netlist, W, piece_groups, lead, run_cost):
    js, meta, od = netlist
    stim, rec = netlist_run_spec(meta)
    lanes, cycles, seed = 300, 12, 41
    h = _emulate(emu, js, meta.top, od, stim, rec, lanes, cycles, seed, W, piece_groups, lead, run_cost)
    ref = oracle_bp_run(od, lanes, cycles, seed, [(od.signal(n), k, p) for n, k, p in stim],
                        [od.signal(r) for r in rec], 2)
    assert np.array_equal(h, ref["hash"])


def test_emulated_crc32_and_lane_base(emu):
    d = crc32_netlist_json()
    js = d.to_json()
    od = ob.OracleDesign(js, "crc32")
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)] + [(f"din_{i}", sim.STIM_RANDOM, i)
                                                                       for i in range(8)]
    rec = [f"crc_{i}" for i in range(32)]
    for lane_base in (0, 4096):
        h = _emulate(emu, js, "crc32", od, stim, rec, 100, 20, 7, 8, 512, 0.85, 2.0, lane_base=lane_base)
        ref = oracle_bp_run(od, 100, 20, 7, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec],
                            2, lane_base=lane_base)
        assert np.array_equal(h, ref["hash"]), lane_base
