"""The AOT bit-parallel CPU baseline (emitted C) agrees with the bit-parallel
interpreter on per-cycle output hashes (both restate the reference's
bit-parallel engines, crates/rrtl-sim-ir/src/bitparallel.rs)."""
import numpy as np

from oracle import binding as ob
from rrtl_gb300.workloads import gate_netlist, netlist_run_spec


def test_aot_hash_equals_interpreter(oracle_lib):
    d, meta = gate_netlist(n_gates=1200, n_ff=64, n_pi=12, n_po=16, depth=10, seed=13)
    od = ob.OracleDesign(d.to_json(), meta.top)
    stim, rec = netlist_run_spec(meta)
    si = [(od.signal(n), k, p) for n, k, p in stim]
    ri = [od.signal(r) for r in rec]
    aot = ob.BitParallelAot(od, si, ri, opt="-O1")
    lanes, cycles = 640, 15
    h = aot.run(lanes, cycles, 21, threads=3)
    ref = np.zeros(cycles, dtype=np.uint64)
    ob.bp_run_parallel(od, lanes, ob.make_run(cycles, 21, si, ri, 2, out_hash=ref), 4)
    assert np.array_equal(h, ref)
