"""GPU parity of the lane-per-thread word engine against the packed oracle."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.builder import Design, lit_u, mux, uint
from rrtl_gb300.workloads import counter

from .helpers import oracle_packed_run

pytestmark = pytest.mark.gpu


def test_counter_known_answer(engine):
    """crates/rrtl-gpu-sim/src/lib.rs:5763-5787: rst=[1,0,0,0], en=[1,0,1,1]; tick; rst=0; tick -> [1,0,2,2]."""
    d = Design()
    m = d.module("Counter")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    en = m.input("en", uint(1))
    count = m.reg("count", uint(8))
    m.clock(count, clk)
    m.reset(count, rst, 0)
    m.next(count, mux(en, count + lit_u(1, 8), count))
    g = sim.GpuBatchSimulator(d, "Counter", 4)
    assert g.design.info.engine == sim.ENGINE_WORD
    g.set_input("rst", [1, 0, 0, 0])
    g.set_input("en", [1, 0, 1, 1])
    g.tick()
    g.set_input("rst", [0, 0, 0, 0])
    g.tick()
    assert list(g.get_signal("count")) == [1, 0, 2, 2]


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN])
def test_counter_1024_lanes_10k_cycles(engine, path):
    """Counter, 1,024 lanes x 10,000 cycles, rst on cycle 0, en ~ Bernoulli(0.5): full out trace."""
    d = counter()
    g = sim.GpuBatchSimulator(d, "Counter", 1024)
    g.set_path(path)
    cycles = 10_000
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 0)]
    res = g.run(cycles, seed=1, stim=stim, record=["out"], mode=sim.REC_TRACE | sim.REC_HASH)
    tr = res["trace"][:, 0, :]
    # closed form of the design: count' = rst ? 0 : count + en (mod 256); out samples count before the edge
    from rrtl_gb300.workloads import stim_word

    lanes = np.arange(1024)
    cnt = np.zeros(1024, dtype=np.int64)
    for c in range(cycles):
        assert np.array_equal(tr[c], cnt), c
        words = np.array([stim_word(1, 0, c, w) for w in range(32)], dtype=np.uint64)
        en = (words[lanes // 32] >> (lanes % 32).astype(np.uint64)) & 1
        cnt = np.zeros(1024, dtype=np.int64) if c < 1 else (cnt + en.astype(np.int64)) % 256
    od = ob.OracleDesign(d.to_json(), "Counter")
    small = 96
    gs = sim.GpuBatchSimulator(d, "Counter", small)
    r2 = gs.run(400, seed=1, stim=stim, record=["out"], mode=sim.REC_TRACE | sim.REC_HASH)
    ref = oracle_packed_run(od, small, 400, 1, [(od.signal(n), k, p) for n, k, p in stim], [od.signal("out")], 3)
    assert np.array_equal(r2["trace"], ref["trace"])
    assert np.array_equal(r2["hash"], ref["hash"])
