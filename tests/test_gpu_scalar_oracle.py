"""The GPU engines against the scalar Simulator restated (crates/rrtl-core/src/lib.rs:5849-6470).

The scalar simulator runs the unlowered design: it evaluates the design's
expression trees directly and never links the product's lowering
(lower.cpp), so these checks are independent of the packed/machine lowering
that the packed and bit-parallel oracles share with the engines. Every op
result of the random designs goes through a wire, so the scalar simulator's
unmasked intermediates (crates/rrtl-core/src/lib.rs:6401-6469) cannot differ
by construction. Outputs and registers are compared per lane after every
tick; inputs differ per lane.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, gate_netlist

from .designs import random_word_design

pytestmark = pytest.mark.gpu


def _limbs(vals, w):
    n = max(1, (w + 31) // 32)
    return np.array([[(v >> (32 * k)) & 0xFFFFFFFF for v in vals] for k in range(n)], dtype=np.uint32)


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_WORD_INTERP])
@pytest.mark.parametrize("seed", range(10))
def test_word_engine_matches_scalar_simulator(engine, seed, path):
    d, meta = random_word_design(700 + seed, wire_every_node=True, async_resets=False, n_mems=2)
    js = d.to_json()
    od = ob.OracleDesign(js, meta["top"])
    lanes = 6
    g = sim.GpuBatchSimulator(js, meta["top"], lanes)
    g.set_path(path)
    sc = [ob.ScalarSim(od) for _ in range(lanes)]
    rng = Rng(seed + 31)
    checked = 0
    for cyc in range(10):
        for name, w in meta["inputs"] + [("rst", 1), ("clk", 1)]:
            if name == "clk":
                vals = [1] * lanes
            elif name == "rst":
                vals = [int(cyc < 1 and l % 2 == 0) for l in range(lanes)]
            else:
                vals = [rng.next() & ((1 << w) - 1) for _ in range(lanes)]
            g.set_input_limbs(name, _limbs(vals, w))
            for l in range(lanes):
                sc[l].set(name, vals[l])
        g.tick()
        for s in sc:
            s.tick()
        for name, w in meta["outputs"] + meta["regs"]:
            got = g.get_signal_limbs(name)
            for l in range(lanes):
                v = sum(int(got[k][l]) << (32 * k) for k in range(got.shape[0]))
                assert v == sc[l].get(name), (seed, cyc, name, l)
                checked += v != 0
    assert checked > 0


@pytest.mark.parametrize("words", [0, 8, 4, -1])  # automatic, fused widths, plain path
def test_gate_engine_matches_scalar_simulator(engine, words):
    d, meta = gate_netlist(n_gates=2500, n_ff=96, n_pi=16, n_po=24, depth=12, seed=23)
    js = d.to_json()
    od = ob.OracleDesign(js, meta.top)
    lanes = 40
    g = sim.GpuBatchSimulator(js, meta.top, lanes)
    if words < 0:
        g.set_path(sim.PATH_PLAIN)
    else:
        g.set_tile_words(words)
    sc = [ob.ScalarSim(od) for _ in range(lanes)]
    rng = Rng(97)
    for cyc in range(8):
        ins = {meta.clk: [1] * lanes, meta.rst: [int(cyc == 0)] * lanes}
        for p in meta.inputs:
            ins[p] = [rng.below(2) for _ in range(lanes)]
        for name, vals in ins.items():
            g.set_input_limbs(name, _limbs(vals, 1))
            for l in range(lanes):
                sc[l].set(name, vals[l], settle=False)
        for s in sc:
            s.eval()
        g.tick()
        for s in sc:
            s.tick()
        for name in meta.outputs + meta.regs[::3]:
            got = g.get_signal_bits(name)
            want = [sc[l].get(name) for l in range(lanes)]
            assert [int(got[l // 32] >> (l % 32)) & 1 for l in range(lanes)] == want, (cyc, name)
