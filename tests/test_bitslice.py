"""Bit-slice lowering on the CPU: the plane design of a multi-bit design,
run on the packed oracle, equals the original design on the packed oracle
per lane and cycle (the reference checks its bit-slice engine against its
SIMD engine the same way, crates/rrtl-sim-ir/src/bitslice.rs:727-778), and
designs outside the scope are rejected."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.builder import Design, lit_u, mux, uint
from rrtl_gb300.workloads import Rng, counter

from .designs import random_word_design


def _limbs(vals, w):
    n = max(1, (w + 31) // 32)
    return np.array([[(v >> (32 * l)) & 0xFFFFFFFF for v in vals] for l in range(n)], dtype=np.uint32)


def _value(limbs, lane):
    return sum(int(limbs[l, lane]) << (32 * l) for l in range(limbs.shape[0]))


def compare_on_oracle(js, top, inputs, observe, lanes=9, cycles=30, seed=1):
    """inputs / observe: [(name, width)]; random inputs every cycle."""
    orig = ob.OracleDesign(js, top)
    planes = ob.OracleDesign(sim.bitslice_json(js, top), top)
    po, pb = ob.PackedSim(orig, lanes), ob.PackedSim(planes, lanes)
    rng = Rng(seed)
    for c in range(cycles):
        for name, w in inputs:
            vals = [rng.next() & ((1 << w) - 1) if w < 64 else rng.next() for _ in range(lanes)]
            if name == "rst":
                vals = [1 if c < 2 else 0] * lanes
            # tick settles first, so the inputs need no settle of their own
            po.set_signal(orig.signal(name), _limbs(vals, w), settle=False)
            for p in range(w):
                pb.set_signal(planes.signal(f"{name}[{p}]"), np.array([[(v >> p) & 1 for v in vals]], np.uint32),
                              settle=False)
        po.tick()
        pb.tick()
        for name, w in observe:
            a = po.get_signal(orig.signal(name))
            got = [0] * lanes
            for p in range(w):
                bits = pb.get_signal(planes.signal(f"{name}[{p}]"))[0]
                for l in range(lanes):
                    got[l] |= int(bits[l] & 1) << p
            assert got == [_value(a, l) for l in range(lanes)], (c, name)


@pytest.mark.parametrize("seed", range(16))
def test_random_designs_plane_by_plane(seed):
    d, meta = random_word_design(300 + seed, n_wires=14, depth=3, n_mems=0, async_resets=False, no_mul=True)
    inputs = [("clk", 1), ("rst", 1)] + list(meta["inputs"])
    observe = list(meta["outputs"]) + list(meta["regs"])
    compare_on_oracle(d.to_json(), meta["top"], inputs, observe, seed=seed)


def test_counter_and_adder_chain():
    compare_on_oracle(counter().to_json(), "Counter", [("clk", 1), ("rst", 1), ("en", 1)], [("count", 8), ("out", 8)])
    d = Design()
    m = d.module("Acc")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    a = m.input("a", uint(100))
    b = m.input("b", uint(100))
    acc = m.reg("acc", uint(100))
    m.clock(acc, clk)
    m.reset(acc, rst, 12345)
    m.next(acc, mux(a.lt_expr(b), acc + a - b, (acc ^ b) + lit_u(7, 100)))
    o = m.output("o", uint(1))
    m.assign(o, acc.eq_expr(a))
    compare_on_oracle(d.to_json(), "Acc", [("clk", 1), ("rst", 1), ("a", 100), ("b", 100)], [("acc", 100), ("o", 1)])
    from rrtl_gb300.workloads import narrow_alu

    compare_on_oracle(narrow_alu(16).to_json(), "Alu", [("clk", 1), ("rst", 1), ("din", 16), ("sel", 2)],
                      [("acc", 16), ("out", 16), ("flag", 1), ("b", 16)])


def test_out_of_scope_designs_are_rejected():
    for kw in ({"n_mems": 1, "async_resets": False, "no_mul": True}, {"n_mems": 0, "async_resets": True, "no_mul": True}):
        for seed in range(20):
            d, meta = random_word_design(seed, n_mems=kw["n_mems"], async_resets=kw["async_resets"], no_mul=True)
            js = d.to_json()
            if kw["n_mems"] or '"Async"' in js:
                with pytest.raises(sim.RrtlError) as e:
                    sim.bitslice_json(js, meta["top"])
                assert e.value.code == "E_BITSLICE"
                break
    d = Design()
    m = d.module("M")
    clk = m.input("clk", uint(1))
    x = m.input("x", uint(8))
    r = m.reg("r", uint(8))
    m.clock(r, clk)
    m.next(r, r * x)
    with pytest.raises(sim.RrtlError) as e:
        sim.bitslice_json(d.to_json(), "M")
    assert e.value.code == "E_BITSLICE"
