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


def _ctl_design():
    """The design of the reference's bit-slice test (crates/rrtl-sim-ir/src/bitslice.rs:727-745)."""
    d = Design()
    m = d.module("Ctl")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    sel = m.input("sel", uint(1))
    a = m.input("a", uint(8))
    b = m.input("b", uint(8))
    acc = m.reg("acc", uint(8))
    m.clock(acc, clk)
    m.reset(acc, rst, 0)
    m.next(acc, mux(sel, acc + a, acc ^ b))
    o = m.output("o", uint(8))
    m.assign(o, acc)
    o2 = m.output("o2", uint(1))
    m.assign(o2, acc.eq_expr(a))
    return d


def test_reference_bitslice_test_on_the_restated_engine():
    """The reference's bitslice_matches_simd_cpu (bitslice.rs:727-778): 100
    lanes, 30 cycles, seeded stimulus s = c*2654435761 + l + len(name)*7, rst
    on the first two cycles; the restated BitSliceSimulator equals the packed
    oracle on o and o2, and the plane design (the product's lowering) run on
    the packed oracle equals both."""
    js = _ctl_design().to_json()
    od = ob.OracleDesign(js, "Ctl")
    pd = ob.OracleDesign(sim.bitslice_json(js, "Ctl"), "Ctl")
    lanes = 100
    bs, ps, pp = ob.BitSlice(od, lanes), ob.PackedSim(od, lanes), ob.PackedSim(pd, lanes)
    ps.set_signal(od.signal("clk"), np.ones((1, lanes), np.uint32), settle=False)
    bs.set_signal(od.signal("clk"), np.ones((1, lanes), np.uint32))
    for c in range(30):
        for name, mask in (("rst", 1), ("sel", 1), ("a", 0xFF), ("b", 0xFF)):
            if name == "rst":
                vals = [1 if c < 2 else 0] * lanes
            else:
                vals = [((c * 2654435761 + l + len(name) * 7) & 0xFFFFFFFFFFFFFFFF) & mask for l in range(lanes)]
            arr = np.array([vals], dtype=np.uint32)
            ps.set_signal(od.signal(name), arr, settle=False)
            bs.set_signal(od.signal(name), arr)
            w = 8 if mask == 0xFF else 1
            for p in range(w):
                pp.set_signal(pd.signal(f"{name}[{p}]"), np.array([[(v >> p) & 1 for v in vals]], np.uint32),
                              settle=False)
        ps.tick()
        bs.tick()
        pp.tick()
        for name, w in (("o", 8), ("o2", 1)):
            ref = ps.get_signal(od.signal(name))[0]
            assert np.array_equal(bs.get_signal(od.signal(name))[0], ref), (c, name)
            planes = sum(pp.get_signal(pd.signal(f"{name}[{p}]"))[0].astype(np.uint64) << np.uint64(p) for p in range(w))
            assert np.array_equal(planes, ref.astype(np.uint64)), (c, name)


def test_restated_bitslice_settles_a_block_against_its_start_state():
    """The reference's BitSliceSimulator evaluates a whole settle block
    against the state at the block's start and stores afterwards
    (crates/rrtl-sim-ir/src/bitslice.rs:121-127, 295-316), so a wire that
    reads another wire of the same settle sees its earlier value; a tick
    settles twice, so a three-level chain is still short one level after it.
    The restatement keeps that; PackedSimulator and the product's plane
    lowering settle completely."""
    d = Design()
    m = d.module("Chain")
    clk = m.input("clk", uint(1))
    a = m.input("a", uint(8))
    w1 = m.wire("w1", uint(8))
    w2 = m.wire("w2", uint(8))
    m.assign(w1, a + lit_u(1, 8))
    m.assign(w2, w1 + lit_u(1, 8))
    o = m.output("o", uint(8))
    m.assign(o, w2 + lit_u(1, 8))
    js = d.to_json()
    od = ob.OracleDesign(js, "Chain")
    pd = ob.OracleDesign(sim.bitslice_json(js, "Chain"), "Chain")
    bs, ps, pp = ob.BitSlice(od, 4), ob.PackedSim(od, 4), ob.PackedSim(pd, 4)
    av = [5, 6, 7, 8]
    bs.set_signal(od.signal("a"), np.array([av], np.uint32))
    ps.set_signal(od.signal("a"), np.array([av], np.uint32), settle=False)
    for p in range(8):
        pp.set_signal(pd.signal(f"a[{p}]"), np.array([[(v >> p) & 1 for v in av]], np.uint32), settle=False)
    bs.tick()
    ps.tick()
    pp.tick()
    assert ps.get_signal(od.signal("o"))[0].tolist() == [8, 9, 10, 11]
    assert bs.get_signal(od.signal("o"))[0].tolist() == [2, 2, 2, 2]
    planes = sum(pp.get_signal(pd.signal(f"o[{p}]"))[0].astype(np.int64) << p for p in range(8))
    assert planes.tolist() == [8, 9, 10, 11]
