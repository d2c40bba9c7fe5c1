"""Edge cases of the batch API on the GPU: zero-cycle runs, runs with no
stimulus or no records, designs without registers or without combinational
logic, ragged lane counts at the tile edges, and the lane limit."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.builder import Design, mux, uint
from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

from .helpers import oracle_bp_run

pytestmark = pytest.mark.gpu


def _comb_only():
    d = Design()
    m = d.module("Comb")
    a, b, c = (m.input(n, uint(1)) for n in "abc")
    y = m.output("y", uint(1))
    m.assign(y, mux(a, b, c) ^ (a & b))
    return d


def _regs_only():
    d = Design()
    m = d.module("Shift")
    clk = m.input("clk", uint(1))
    din = m.input("din", uint(1))
    q = [m.reg(f"q{i}", uint(1)) for i in range(4)]
    for i, r in enumerate(q):
        m.clock(r, clk)
        m.next(r, din.value() if i == 0 else q[i - 1].value())
    o = m.output("o", uint(1))
    m.assign(o, q[-1])
    return d


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN])
def test_zero_cycles_empty_stim_and_no_records(engine, path):
    d, meta = gate_netlist(n_gates=800, n_ff=40, n_pi=8, n_po=8, depth=6, seed=71)
    js = d.to_json()
    cd = sim.CompiledDesign(js, meta.top)
    od = ob.OracleDesign(js, meta.top)
    g = sim.GpuBatchSimulator(cd, lanes=77)
    g.set_path(path)
    r = g.run(0, mode=0)  # settle only
    assert r["trace"] is None and r["hash"] is None
    g.run(5)  # no stimulus, no records: inputs hold, registers advance
    ref = oracle_bp_run(od, 77, 5, 0, [], [], 0)
    ref["sim"].settle()
    for q in meta.regs + meta.outputs:
        assert np.array_equal(g.get_signal_bits(q), ref["sim"].get_bits(od.signal(q))), q


@pytest.mark.parametrize("lanes", [31, 32, 255, 256, 257, 8 * 32 * 4 + 1])
def test_combinational_only_design(engine, lanes):
    d = _comb_only()
    g = sim.GpuBatchSimulator(d, "Comb", lanes=lanes)
    rng = np.random.default_rng(lanes)
    vals = {n: rng.integers(0, 2, lanes) for n in "abc"}
    for n, v in vals.items():
        g.set_input(n, v)
    g.eval_combinational()
    a, b, c = vals["a"], vals["b"], vals["c"]
    assert np.array_equal(g.get_signal("y"), np.where(a == 1, b, c) ^ (a & b))
    g.eval_combinational_many(2)  # settling again changes nothing
    assert np.array_equal(g.get_signal("y"), np.where(a == 1, b, c) ^ (a & b))


def test_register_only_design_shifts(engine):
    g = sim.GpuBatchSimulator(_regs_only(), "Shift", lanes=40)
    bits = [1, 0, 1, 1, 0, 0]
    seen = []
    for b in bits:
        g.set_input("din", [b] * 40)
        g.tick()
        seen.append(int(g.get_signal("o")[0]))
    assert seen == [0, 0, 0, 1, 0, 1]


def test_lane_limit_and_zero_lanes(engine):
    d = _comb_only()
    cd = sim.CompiledDesign(d, "Comb")
    for bad in (0, (1 << 30) + 1):
        with pytest.raises(sim.RrtlError) as e:
            sim.GpuBatchSimulator(cd, lanes=bad)
        assert e.value.code == "E_GPU_LANES"
