"""Instance folding on the GPU: the child module over N x L lanes equals the
flattened wrapper over L lanes, per instance, per cycle (the reference's
fold_matches_naive check, crates/rrtl-gpu-sim/src/instance_fold.rs:100-192,
on the GPU engines)."""
import numpy as np
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, replicated_datapath

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,base", [(4, 3), (16, 100), (64, 64)])
def test_folded_run_equals_flattened(engine, n, base):
    cycles = 40
    d = replicated_datapath(n)
    js = d.to_json()
    rng = np.random.default_rng(n * 1000 + base)
    din = rng.integers(0, 2**32, size=(cycles, n, base), dtype=np.uint64).astype(np.uint32)
    flat = sim.GpuBatchSimulator(js, "Top", base)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim_flat = stim + [(f"din{i}", sim.STIM_TRACE, i) for i in range(n)]
    rf = flat.run(cycles, stim=stim_flat, record=[f"o{i}" for i in range(n)], mode=sim.REC_TRACE, input_trace=din)
    fold = sim.InstanceFoldSimulator(js, "Top", base)
    assert fold.num_instances == n and fold.total_lanes == n * base
    # lane block i of the child's din column is instance i's stream
    din_fold = din.reshape(cycles, 1, n * base)
    rc = fold.sim.run(cycles, stim=stim + [("din", sim.STIM_TRACE, 0)], record=["o"], mode=sim.REC_TRACE,
                      input_trace=din_fold)
    got = rc["trace"][:, 0, :].reshape(cycles, n, base)
    assert np.array_equal(got, rf["trace"])
    assert got[-1].any()


def test_fold_port_demux_stepwise(engine):
    """set_top_input / get_top_output address the wrapper's signals per
    instance block; ticking both simulators cycle by cycle agrees."""
    n, base = 6, 33
    d = replicated_datapath(n)
    js = d.to_json()
    flat = sim.GpuBatchSimulator(js, "Top", base)
    fold = sim.InstanceFoldSimulator(js, "Top", base)
    assert fold.port_offset("din") == fold.sim.design.signal("din")[0]
    assert fold.port_offset("no_such_port") is None
    assert fold.port_offset("acc") is None  # a register, not a port
    rng = Rng(4)
    for c in range(12):
        for name, v in (("clk", 1), ("rst", 1 if c == 0 else 0)):
            flat.set_input(name, [v] * base)
            fold.set_top_input(name, np.full((1, base), v, np.uint32))
        for i in range(n):
            v = np.array([[rng.next() & 0xFFFFFFFF for _ in range(base)]], np.uint32)
            flat.set_input_limbs(f"din{i}", v)
            fold.set_top_input(f"din{i}", v)
        flat.tick()
        fold.tick()
        fold.synchronize()
        for i in range(n):
            assert np.array_equal(fold.get_top_output(f"o{i}"), flat.get_signal_limbs(f"o{i}")), (c, i)
