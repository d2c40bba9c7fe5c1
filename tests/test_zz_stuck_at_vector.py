"""The reference's ATPG known answer on the product's gate engine: its
symbolic test for crc_5 stuck-at-0 (din = 0x01, initial state 0), confirmed
concretely with lane 0 golden and lane 1 faulted, gives golden 0x690ce0ee
and faulty 0x690ce0ce after one clock
(crates/rrtl-sim-ir/examples/symbolic_exec.rs:192-212;
docs/rrtl-optimizations.md:1931-1934). Collected last so a failure here comes
after every other test."""
import numpy as np
import pytest

from rrtl_gb300 import sim

from .helpers import crc32_netlist_json

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN])
def test_crc5_stuck_at_0_vector(engine, path):
    cd = sim.CompiledDesign(crc32_netlist_json(), "crc32")
    g = sim.GpuBatchSimulator(cd, lanes=2)  # state starts at 0
    g.set_path(path)
    g.set_faults([(1, "crc_5", 0)])
    din = 0x01
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_CONST, 0)]
    stim += [(f"din_{i}", sim.STIM_CONST, (din >> i) & 1) for i in range(8)]
    rec = [f"crc_{i}" for i in range(32)]
    # a cycle records before its clock edge: row 1 is the state after one edge
    tr = g.run(2, stim=stim, record=rec, mode=sim.REC_TRACE)["trace"]
    assert tr.shape == (2, 32, 1)
    row = [[sum(((int(tr[c, i, 0]) >> l) & 1) << i for i in range(32)) for l in range(2)] for c in range(2)]
    assert row == [[0, 0], [0x690CE0EE, 0x690CE0CE]]
