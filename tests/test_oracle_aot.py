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


def test_aot_final_state_and_lane_base_match_interpreter(oracle_lib):
    """The AOT engine's final register state equals the interpreter's, and a
    run at lane_base L reproduces lanes [L, 2L) of a 2L-lane run (stimulus is
    keyed on global lanes), with RANDOM and RANDOM_UNIFORM inputs."""
    d, meta = gate_netlist(n_gates=900, n_ff=48, n_pi=10, n_po=12, depth=8, seed=14)
    od = ob.OracleDesign(d.to_json(), meta.top)
    for uniform in (False, True):
        stim, rec = netlist_run_spec(meta, uniform=uniform)
        si = [(od.signal(n), k, p) for n, k, p in stim]
        ri = [od.signal(r) for r in rec]
        regs = [od.signal(q) for q in meta.regs]
        aot = ob.BitParallelAot(od, si, ri, opt="-O1")
        h_all, q_all = aot.run(256, 9, 5, threads=2, signals=regs)
        h_lo, q_lo = aot.run(128, 9, 5, threads=2, signals=regs)
        h_hi, q_hi = aot.run(128, 9, 5, threads=2, signals=regs, lane_base=128)
        assert np.array_equal(h_lo + h_hi, h_all)
        assert np.array_equal(np.concatenate([q_lo, q_hi], axis=1), q_all)
        bp = ob.BitParallel(od, 256)
        hb = np.zeros(9, dtype=np.uint64)
        bp.run(ob.make_run(9, 5, si, ri, 2, out_hash=hb))
        assert np.array_equal(hb, h_all)
        for k, s in enumerate(regs):
            assert np.array_equal(bp.get_bits(s), q_all[k])
