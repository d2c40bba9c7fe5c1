"""The lane-shard runtime (rrtl_runtime_*) against one batch of all its lanes:
the reference's DistributedRuntime gives shards to workers
(crates/rrtl-runtime/src/lib.rs:6785-7760); here the shards' runs (one job
queue launch for the gate engine, consecutive runs for the word engine) must
give exactly the whole run's per-cycle hashes, traces and detection vectors,
with faults and input traces given on global lanes."""
import numpy as np
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import cpu_rom_hashed, gate_netlist, job_faults, netlist_run_spec, pipelined_cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def netlist(engine):
    d, meta = gate_netlist(n_gates=3000, n_ff=128, n_pi=16, n_po=20, depth=12, seed=33)
    return meta, sim.CompiledDesign(d.to_json(), meta.top)


@pytest.mark.parametrize("shards", [1, 3, 5])
def test_gate_runtime_equals_one_batch(netlist, shards):
    meta, cd = netlist
    total, cycles = 1000, 24
    stim, rec = netlist_run_spec(meta, uniform=True)
    faults = job_faults(meta, total, seed=4)
    mode = sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT
    g = sim.GpuBatchSimulator(cd, lanes=total)
    g.set_faults(faults)
    want = g.run(cycles, seed=6, stim=stim, record=rec, mode=mode)
    rt = sim.Runtime(cd, total, shards)
    rt.set_faults(faults)
    got = rt.run(cycles, seed=6, stim=stim, record=rec, mode=mode)
    for k in ("trace", "hash", "detect"):
        assert np.array_equal(got[k], want[k]), k
    assert (got["detect"] != 0xFFFFFFFF).any()
    assert sum(rt.shard(k)[2] for k in range(shards)) == total
    rt.close()


def test_gate_runtime_cuts_input_traces_per_shard(netlist):
    meta, cd = netlist
    total, cycles = 700, 12
    words = (total + 31) // 32
    cols = [meta.rst] + meta.inputs
    trace = np.random.default_rng(3).integers(0, 2**32, size=(cycles, len(cols), words), dtype=np.uint64).astype(np.uint32)
    stim = [(meta.clk, sim.STIM_CONST, 1)] + [(n, sim.STIM_TRACE, k) for k, n in enumerate(cols)]
    rec = meta.outputs
    g = sim.GpuBatchSimulator(cd, lanes=total)
    want = g.run(cycles, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH, input_trace=trace)
    rt = sim.Runtime(cd, total, 4)
    got = rt.run(cycles, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH, input_trace=trace)
    assert np.array_equal(got["trace"], want["trace"])
    assert np.array_equal(got["hash"], want["hash"])


def test_word_runtime_equals_one_batch(engine):
    cd = sim.CompiledDesign(pipelined_cpu(), "Cpu8")
    total, cycles = 600, 150
    rom = cpu_rom_hashed(total, seed=8)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    rec = ["out_pc", "out_acc"]
    g = sim.GpuBatchSimulator(cd, lanes=total)
    g.set_memory_limbs("rom", rom)
    want = g.run(cycles, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    rt = sim.Runtime(cd, total, 3)
    for k in range(3):
        _, first, lanes = rt.shard(k)
        info = sim.ShardInfo()
        b = sim.c_void_p()
        sim.check(sim.lib().rrtl_runtime_shard(rt.h, k, sim.byref(info), sim.byref(b)))
        idx = cd.memory("rom")[0]
        part = np.ascontiguousarray(rom[:, :, first:first + lanes])
        sim.check(sim.lib().rrtl_batch_set_memory_limbs(b, idx, part.ctypes.data_as(sim.POINTER(sim.c_uint32)), part.size))
    got = rt.run(cycles, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    assert np.array_equal(got["trace"], want["trace"])
    assert np.array_equal(got["hash"], want["hash"])
    rt.close()
