"""Fault-simulation protocol on the CPU oracle.

The reference drives the golden lane and every faulted lane with one input
sequence (set_signal_all, crates/rrtl-sim-ir/examples/fault_sim.rs:66-76) and
reports, per faulted lane, the first cycle its observed outputs differ from
lane 0's (:86-93). RANDOM_UNIFORM stimulus gives every lane that sequence;
the engines compare each lane with lane 0 of its 32-lane word, which is
fault-free and therefore equal to the reference's golden lane.
"""
import numpy as np

from oracle import binding as ob
from rrtl_gb300.workloads import Rng, gate_netlist, job_faults, netlist_run_spec


def _netlist():
    d, meta = gate_netlist(n_gates=5000, n_ff=192, n_pi=24, n_po=24, depth=20, seed=61)
    return meta, ob.OracleDesign(d.to_json(), meta.top)


def _detect(od, meta, lanes, cycles, uniform, faults=(), mode=4 | 2 | 1):
    stim, rec = netlist_run_spec(meta, uniform=uniform)
    words = (lanes + 31) // 32
    bp = ob.BitParallel(od, lanes)
    for lane, sig, v in faults:
        bp.set_force(od.signal(sig), lane, v)
    det = np.zeros(lanes, dtype=np.uint32)
    tr = np.zeros((cycles, len(rec), words), dtype=np.uint32)
    h = np.zeros(cycles, dtype=np.uint64)
    bp.run(ob.make_run(cycles, 9, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec], mode,
                       out_trace=tr, out_hash=h, detect=det))
    return det, tr


def test_fault_free_lanes_never_detect_with_uniform_stimulus(oracle_lib):
    meta, od = _netlist()
    det, _ = _detect(od, meta, 256, 40, uniform=True)
    assert (det == 0xFFFFFFFF).all()
    # per-lane random stimulus makes lanes differ without any fault: detection is then meaningless
    det_rand, _ = _detect(od, meta, 256, 40, uniform=False)
    assert (det_rand != 0xFFFFFFFF).sum() > 200


def test_uniform_fault_job_matches_the_reference_protocol(oracle_lib):
    """Per faulted lane, the detection cycle equals the first cycle its
    recorded outputs differ from global lane 0 (the reference's golden lane),
    computed from the trace."""
    meta, od = _netlist()
    lanes, cycles = 320, 48
    faults = job_faults(meta, lanes, seed=5)
    det, tr = _detect(od, meta, lanes, cycles, uniform=True, faults=faults)
    bits = (tr[:, :, np.arange(lanes) // 32] >> (np.arange(lanes) % 32)) & 1  # [cycle][rec][lane]
    differs = (bits != bits[:, :, :1]).any(axis=1)  # [cycle][lane] vs global lane 0
    want = np.where(differs.any(axis=0), differs.argmax(axis=0), 0xFFFFFFFF).astype(np.uint32)
    assert np.array_equal(det, want)
    assert (det[::32] == 0xFFFFFFFF).all()  # lane 0 of every word is fault-free
    n_det = int((det != 0xFFFFFFFF).sum())
    assert 0 < n_det < lanes - lanes // 32  # some faults are detected, some stay latent
