"""Design loading and lowering checks on the CPU (no GPU)."""
import json

import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300.builder import Design, lit_u, mux, uint, sint
from rrtl_gb300.workloads import Rng, counter, gate_netlist, pipelined_cpu

from .designs import random_word_design


@pytest.mark.parametrize("seed", range(40))
def test_scalar_simulator_matches_packed_lowering(oracle_lib, seed):
    """The scalar Simulator runs the unlowered design; PackedSim runs the
    packed/machine lowering. Every op result goes through a wire so the scalar
    simulator's unmasked intermediates cannot differ by construction."""
    d, meta = random_word_design(seed, wire_every_node=True, async_resets=False)
    od = ob.OracleDesign(d.to_json(), meta["top"])
    lanes = 3
    ps = ob.PackedSim(od, lanes)
    sc = [ob.ScalarSim(od) for _ in range(lanes)]
    rng = Rng(seed + 100)
    nonzero = 0
    for cyc in range(10):
        for name, w in meta["inputs"] + [("rst", 1), ("clk", 1)]:
            if name == "clk":
                vals = [1] * lanes
            elif name == "rst":
                vals = [int(cyc < 1 and l % 2 == 0) for l in range(lanes)]
            else:
                vals = [rng.next() & ((1 << w) - 1) for _ in range(lanes)]
            limbs = max(1, (w + 31) // 32)
            arr = np.array([[(v >> (32 * k)) & 0xFFFFFFFF for v in vals] for k in range(limbs)], dtype=np.uint32)
            ps.set_signal(od.signal(name), arr)
            for l in range(lanes):
                sc[l].set(name, vals[l])
        ps.tick()
        for s in sc:
            s.tick()
        for name, w in meta["outputs"] + meta["regs"]:
            got = ps.get_signal(od.signal(name))
            for l in range(lanes):
                pv = sum(int(got[k][l]) << (32 * k) for k in range(got.shape[0]))
                assert pv == sc[l].get(name), (seed, cyc, name, l)
                nonzero += pv != 0
    assert nonzero > 0


def test_packed_layout_matches_reference_rules(oracle_lib):
    """Signals get ceil(width/32) limbs (min 1) at increasing offsets
    (crates/rrtl-sim-ir/src/lib.rs:12698-12722); memories do not take signal words."""
    d = Design()
    m = d.module("L")
    a = m.input("a", uint(1))
    b = m.input("b", uint(33))
    c = m.wire("c", uint(64))
    mm = m.mem("mm", 3, uint(40), 8)
    m.assign(c, b.zext(64))
    od = ob.OracleDesign(d.to_json(), "L")
    assert od.num_signals == 3
    assert od.total_signal_words == 1 + 2 + 2
    assert od.total_memory_words == 8 * 2


def test_type_errors_carry_reference_codes(oracle_lib):
    d = Design()
    m = d.module("T")
    a = m.input("a", uint(4))
    b = m.input("b", uint(5))
    w = m.wire("w", uint(4))
    m.assign(w, a & b)
    with pytest.raises(ob.OracleError, match="E_EXPR_TYPE"):
        ob.OracleDesign(d.to_json(), "T")
    d = Design()
    m = d.module("T")
    a = m.input("a", uint(4))
    w = m.wire("w", uint(4))
    m.assign(w, mux(a, a, a))
    with pytest.raises(ob.OracleError, match="E_MUX_COND_WIDTH"):
        ob.OracleDesign(d.to_json(), "T")
    d = Design()
    m = d.module("T")
    a = m.input("a", uint(4))
    w = m.wire("w", uint(4))
    m.assign(w, a.slice(2, 4))
    with pytest.raises(ob.OracleError, match="E_SLICE_RANGE"):
        ob.OracleDesign(d.to_json(), "T")
    with pytest.raises(ob.OracleError, match="E_SIM_IR_MODULE"):
        ob.OracleDesign(d.to_json(), "Missing")
    with pytest.raises(ob.OracleError, match="E_DESIGN_JSON"):
        ob.OracleDesign('{"modules": [', "T")


def test_hierarchy_flattening_matches_scalar(oracle_lib):
    """Instances flatten into port assignments (crates/rrtl-sim-ir/src/lib.rs:12307-12503)."""
    d = Design()
    c = d.module("Inc")
    x = c.input("x", uint(8))
    y = c.output("y", uint(8))
    c.assign(y, x + lit_u(1, 8))
    t = d.module("Top")
    clk = t.input("clk", uint(1))
    r = t.reg("r", uint(8))
    t.clock(r, clk)
    n = t.wire("n", uint(8))
    t.instance("u0", "Inc", [("x", r), ("y", n)])
    t.next(r, n)
    od = ob.OracleDesign(d.to_json(), "Top")
    p = ob.PackedSim(od, 2)
    s = ob.ScalarSim(od)
    for _ in range(5):
        p.tick()
        s.tick()
    assert list(p.get_signal(od.signal("r"))[0]) == [5, 5] == [s.get("r")] * 2


def test_workload_generators_are_deterministic():
    d1, m1 = gate_netlist(n_gates=500, n_ff=32, n_pi=8, n_po=8, depth=5, seed=4)
    d2, m2 = gate_netlist(n_gates=500, n_ff=32, n_pi=8, n_po=8, depth=5, seed=4)
    assert d1.to_json() == d2.to_json()
    assert counter().to_json() == counter().to_json()
    assert pipelined_cpu().to_json() == pipelined_cpu().to_json()
    obj = json.loads(d1.to_json())
    assert obj["modules"][0]["name"] == "netlist"


def test_gate_netlist_shape(oracle_lib):
    d, meta = gate_netlist(n_gates=4000, n_ff=128, n_pi=16, n_po=16, depth=20, seed=1)
    od = ob.OracleDesign(d.to_json(), meta.top)
    # 20 gate levels plus the output buffers
    assert od.num_levels == 21
    assert sum(1 for i in range(od.num_signals) if od.kind(i) == 3) == 128


def test_lut_class_list_is_the_permutation_representatives():
    """rrtl_gb300/csrc/lut_classes.h lists exactly the truth tables that are
    the smallest of their six input orders (the kernel's specialised loops)."""
    import os
    import re

    def perm_lut(l, p):
        out = 0
        for idx in range(8):
            nv = [(idx >> 2) & 1, (idx >> 1) & 1, idx & 1]
            ov = [0, 0, 0]
            for k in range(3):
                ov[p[k]] = nv[k]
            if (l >> ((ov[0] << 2) | (ov[1] << 1) | ov[2])) & 1:
                out |= 1 << idx
        return out

    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    canon = sorted(l for l in range(256) if min(perm_lut(l, p) for p in perms) == l)
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "rrtl_gb300", "csrc", "lut_classes.h")).read()
    listed = sorted(int(x) for x in re.findall(r"X\((\d+)\)", hdr.split("#define RRTL_LUT_CLASSES(X)")[1]))
    assert listed == canon and len(canon) == 80


def test_levelization_of_a_200k_deep_wire_chain(oracle_lib):
    """A comb chain 200,000 assignments deep levelizes without recursing that
    deep on the host stack: level k holds wire k, and the chain's output is
    the input plus the chain length (mod 2^16) after one settle."""
    n = 200_000
    d = Design()
    m = d.module("Chain")
    a = m.input("a", uint(16))
    y = m.output("y", uint(16))
    prev = a.value()
    for i in range(n):
        w = m.wire(f"w{i}", uint(16))
        m.assign(w, (prev + lit_u(1, 16)).trunc(16))
        prev = w.value()
    m.assign(y, prev)
    od = ob.OracleDesign(d.to_json(), "Chain")
    assert od.num_levels == n + 1
    ps = ob.PackedSim(od, 2)
    ps.set_signal(od.signal("a"), np.array([[7, 65535]], dtype=np.uint32))
    got = ps.get_signal(od.signal("y"))
    assert list(got[0]) == [(7 + n) & 0xFFFF, (65535 + n) & 0xFFFF]
