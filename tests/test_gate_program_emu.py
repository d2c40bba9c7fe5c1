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


def _register_mix():
    """1-bit registers with every commit form: reset high/low to 0/1, no
    reset, D taken straight from another register (a copy cell keeps D and Q
    apart), an output driven by a register, a constant-driven register."""
    from rrtl_gb300.builder import Design, lit_u, mux, uint

    d = Design()
    m = d.module("Mix")
    clk, rst, rstn = m.input("clk", uint(1)), m.input("rst", uint(1)), m.input("rstn", uint(1))
    a, b, c = m.input("a", uint(1)), m.input("b", uint(1)), m.input("c", uint(1))
    regs = [m.reg(f"r{i}", uint(1)) for i in range(8)]
    for r in regs:
        m.clock(r, clk)
    m.next(regs[0], a ^ regs[7])
    m.reset(regs[0], rst, 1)
    m.next(regs[1], regs[0])  # D is another register
    m.reset_low(regs[1], rstn, 0)
    m.next(regs[2], mux(b, regs[1], ~regs[2]))
    m.reset_low(regs[2], rstn, 1)
    m.next(regs[3], (regs[2] & c) | regs[0])
    m.next(regs[4], regs[3] ^ regs[1] ^ a)
    m.reset(regs[4], rst, 0)
    m.next(regs[5], lit_u(1, 1))  # constant D
    m.next(regs[6], regs[5] & ~regs[4])
    m.next(regs[7], regs[6] | (b & c))
    outs = []
    for i, r in enumerate((regs[1], regs[4], regs[7])):
        o = m.output(f"o{i}", uint(1))
        m.assign(o, r)
        outs.append(f"o{i}")
    w = m.wire("w", uint(1))
    m.assign(w, regs[2] ^ regs[6])
    o = m.output("o3", uint(1))
    m.assign(o, w & a)
    outs.append("o3")
    return d, "Mix", outs


@pytest.mark.parametrize("W", [8, 4, 1])
def test_emulated_register_commit_forms(emu, W):
    d, top, outs = _register_mix()
    js = d.to_json()
    od = ob.OracleDesign(js, top)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 3), ("rstn", sim.STIM_RANDOM, 9),
            ("a", sim.STIM_RANDOM, 1), ("b", sim.STIM_RANDOM, 2), ("c", sim.STIM_RANDOM, 3)]
    h = _emulate(emu, js, top, od, stim, outs, 70, 40, 13, W, 8, 0.85, 2.0)
    ref = oracle_bp_run(od, 70, 40, 13, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in outs], 2)
    assert np.array_equal(h, ref["hash"])
