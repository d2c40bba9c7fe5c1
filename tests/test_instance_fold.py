"""Instance folding on the CPU: the structural analysis (the reference's own
accept/reject cases, crates/rrtl-sim-ir/src/instance_fold.rs:99-156, plus
the other rules), and the semantic claim checked with the oracle: the child
module over N x L lanes equals the flattened wrapper over L lanes, instance
by instance and cycle by cycle."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.builder import Design, lit_u, uint
from rrtl_gb300.workloads import Rng, replicated_datapath


def _child(d):
    m = d.module("M")
    clk = m.input("clk", uint(1))
    din = m.input("din", uint(32))
    acc = m.reg("acc", uint(32))
    m.clock(acc, clk)
    m.next(acc, acc * lit_u(3, 32) + din)
    o = m.output("o", uint(32))
    m.assign(o, acc)


def _plan_error(d, top="Top"):
    with pytest.raises(sim.RrtlError) as e:
        sim.instance_fold_plan(d, top)
    assert e.value.code == "E_INSTANCE_FOLD"
    return str(e.value)


def test_detects_independent_instances():
    d = Design()
    _child(d)
    m = d.module("Top")
    clk = m.input("clk", uint(1))
    for i in range(4):
        din = m.input(f"din{i}", uint(32))
        o = m.output(f"o{i}", uint(32))
        m.instance(f"u{i}", "M", [("clk", clk), ("din", din), ("o", o)])
    plan = sim.instance_fold_plan(d, "Top")
    assert plan["child"] == "M" and plan["instances"] == ["u0", "u1", "u2", "u3"]
    assert ["clk", 2, "clk", "in"] in plan["connections"] and ["o3", 3, "o", "out"] in plan["connections"]


def test_rejects_inter_instance_dataflow():
    d = Design()
    _child(d)
    m = d.module("Top")
    clk = m.input("clk", uint(1))
    din = m.input("din", uint(32))
    mid = m.wire("mid", uint(32))
    o = m.output("o", uint(32))
    m.instance("u0", "M", [("clk", clk), ("din", din), ("o", mid)])
    m.instance("u1", "M", [("clk", clk), ("din", mid), ("o", o)])
    assert "feeds" in _plan_error(d)


def test_rejects_shared_driver_top_logic_and_mixed_modules():
    d = Design()
    _child(d)
    m = d.module("Top")
    clk = m.input("clk", uint(1))
    din = m.input("din", uint(32))
    o = m.output("o", uint(32))
    m.instance("u0", "M", [("clk", clk), ("din", din), ("o", o)])
    m.instance("u1", "M", [("clk", clk), ("din", din), ("o", o)])
    assert "two instance outputs" in _plan_error(d)

    d = replicated_datapath(3)
    t = [m for m in d._modules if m.name == "Top"][0]
    from rrtl_gb300.builder import ModuleBuilder

    tb = ModuleBuilder(d, t)
    w = tb.wire("extra", uint(32))
    tb.assign(w, lit_u(5, 32))
    assert "logic of its own" in _plan_error(d)

    d = Design()
    _child(d)
    m2 = d.module("M2")
    clk2 = m2.input("clk", uint(1))
    din2 = m2.input("din", uint(32))
    o2 = m2.output("o", uint(32))
    m2.assign(o2, din2)
    m = d.module("Top")
    clk = m.input("clk", uint(1))
    a, b = m.input("a", uint(32)), m.input("b", uint(32))
    oa, ob_ = m.output("oa", uint(32)), m.output("ob", uint(32))
    m.instance("u0", "M", [("clk", clk), ("din", a), ("o", oa)])
    m.instance("u1", "M2", [("clk", clk), ("din", b), ("o", ob_)])
    assert "different modules" in _plan_error(d)

    d = Design()
    _child(d)
    m = d.module("Top")
    clk = m.input("clk", uint(1))
    din = m.input("din", uint(32))
    o = m.output("o", uint(32))
    m.instance("u0", "M", [("clk", clk), ("din", din), ("o", o)])
    assert "fewer than two" in _plan_error(d)


def test_fold_equals_flattened_on_the_oracle():
    """The packed oracle on the flattened wrapper (L lanes) and on the child
    (N x L lanes, inputs demultiplexed by lane block) agree on every
    instance output for 25 cycles."""
    n, base, cycles = 5, 7, 25
    d = replicated_datapath(n)
    js = d.to_json()
    plan = sim.instance_fold_plan(d, "Top")
    flat = ob.OracleDesign(js, "Top")
    child = ob.OracleDesign(js, plan["child"])
    pf = ob.PackedSim(flat, base)
    pc = ob.PackedSim(child, n * base)
    rng = Rng(9)
    for c in range(cycles):
        rst = 1 if c < 2 else 0
        pf.set_signal(flat.signal("clk"), np.ones((1, base), np.uint32))
        pf.set_signal(flat.signal("rst"), np.full((1, base), rst, np.uint32))
        pc.set_signal(child.signal("clk"), np.ones((1, n * base), np.uint32))
        pc.set_signal(child.signal("rst"), np.full((1, n * base), rst, np.uint32))
        allin = np.zeros((1, n * base), np.uint32)
        for i in range(n):
            v = np.array([[rng.next() & 0xFFFFFFFF for _ in range(base)]], np.uint32)
            pf.set_signal(flat.signal(f"din{i}"), v)
            allin[:, i * base:(i + 1) * base] = v
        pc.set_signal(child.signal("din"), allin)
        pf.tick()
        pc.tick()
        o = pc.get_signal(child.signal("o"))
        for i in range(n):
            assert np.array_equal(pf.get_signal(flat.signal(f"o{i}")), o[:, i * base:(i + 1) * base]), (c, i)


def _limbs(vals, w):
    n = max(1, (w + 31) // 32)
    return np.array([[(v >> (32 * l)) & 0xFFFFFFFF for v in vals] for l in range(n)], dtype=np.uint32)


@pytest.mark.parametrize("seed", range(6))
def test_random_children_with_shared_and_private_inputs_fold(seed):
    """Random child modules (registers with every reset kind, a memory,
    inputs and outputs of many widths) wrapped N = 3 times, each child input
    tied either to one shared wrapper input or to a private one per
    instance: the product's fold plan, used to demultiplex lane blocks, makes
    the child over N x L lanes equal the flattened wrapper on the oracle."""
    from .designs import random_word_design

    n, base, cycles = 3, 5, 12
    d, meta = random_word_design(seed, n_wires=10, depth=3, n_mems=1, top="Cell")
    rng = Rng(seed * 7 + 1)
    m = d.module("Wrap")
    clk, rst = m.input("clk", uint(1)), m.input("rst", uint(1))
    shared, wrap_in = {}, []
    for name, w in meta["inputs"]:
        if rng.below(3) == 0:
            shared[name] = m.input(f"sh_{name}", uint(w))
            wrap_in.append((f"sh_{name}", w))
    for i in range(n):
        conns = [("clk", clk), ("rst", rst)]
        for name, w in meta["inputs"]:
            if name in shared:
                conns.append((name, shared[name]))
            else:
                wrap_in.append((f"{name}_{i}", w))
                conns.append((name, m.input(f"{name}_{i}", uint(w))))
        conns += [(name, m.output(f"{name}_{i}", uint(w))) for name, w in meta["outputs"]]
        m.instance(f"u{i}", "Cell", conns)
    js = d.to_json()
    plan = sim.instance_fold_plan(js, "Wrap")
    assert plan["child"] == "Cell" and len(plan["instances"]) == n
    drives = {}
    for tsig, inst, port, direction in plan["connections"]:
        if direction == "in":
            drives.setdefault(port, {})[inst] = tsig
    flat, child = ob.OracleDesign(js, "Wrap"), ob.OracleDesign(js, "Cell")
    pf, pc = ob.PackedSim(flat, base), ob.PackedSim(child, n * base)
    compared = 0
    for c in range(cycles):
        vals = {"clk": [1] * base, "rst": [1 if c < 2 else 0] * base}
        for name, w in wrap_in:
            vals[name] = [rng.next() & ((1 << w) - 1) if w < 64 else rng.next() for _ in range(base)]
        for name, w in [("clk", 1), ("rst", 1)] + wrap_in:
            pf.set_signal(flat.signal(name), _limbs(vals[name], w), settle=False)
        for port, w in [("clk", 1), ("rst", 1)] + list(meta["inputs"]):
            lanes = sum((vals[drives[port][i]] for i in range(n)), [])
            pc.set_signal(child.signal(port), _limbs(lanes, w), settle=False)
        pf.tick()
        pc.tick()
        for name, w in meta["outputs"]:
            co = pc.get_signal(child.signal(name))
            for i in range(n):
                assert np.array_equal(pf.get_signal(flat.signal(f"{name}_{i}")), co[:, i * base:(i + 1) * base]), \
                    (c, name, i)
                compared += 1
    assert compared >= cycles * n
