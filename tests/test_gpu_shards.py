"""Lane shards on one GPU: batches at lane_base 0 and L run the two halves of
one 2L-lane run (the reference's shard plan, RuntimeShardInfo::start_lane,
crates/rrtl-runtime/src/lib.rs:168-175). Their per-cycle hashes add up to the
2L-lane batch's, their final states concatenate to its state, and each shard
equals the oracle run at the same lane_base. Lane-uniform stimulus (the
fault-simulation protocol) leaves fault-free lanes undetected on every path.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import gate_netlist, netlist_run_spec, pipelined_cpu, cpu_rom_hashed

from .helpers import oracle_bp_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def netlist(engine):
    d, meta = gate_netlist(n_gates=3000, n_ff=160, n_pi=16, n_po=24, depth=12, seed=19)
    js = d.to_json()
    return meta, sim.CompiledDesign(js, meta.top), ob.OracleDesign(js, meta.top)


@pytest.mark.parametrize("words", [0, 8, 4, -1])  # automatic (compiled or fused), fused widths, plain path
def test_gate_shards_compose(netlist, words):
    meta, cd, od = netlist
    half, cycles = 1024, 20
    stim, rec = netlist_run_spec(meta)

    def batch(lanes):
        g = sim.GpuBatchSimulator(cd, lanes=lanes)
        if words < 0:
            g.set_path(sim.PATH_PLAIN)
        else:
            g.set_tile_words(words)
        return g

    full = batch(2 * half)
    rf = full.run(cycles, seed=4, stim=stim, record=rec, mode=sim.REC_HASH)
    parts = []
    for base in (0, half):
        g = batch(half)
        r = g.run(cycles, seed=4, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=base)
        ref = oracle_bp_run(od, half, cycles, 4, [(od.signal(n), k, p) for n, k, p in stim],
                            [od.signal(x) for x in rec], 2, lane_base=base)
        assert np.array_equal(r["hash"], ref["hash"]), base
        parts.append((g, r))
    assert np.array_equal(parts[0][1]["hash"] + parts[1][1]["hash"], rf["hash"])
    for q in meta.regs[::9]:
        both = np.concatenate([parts[0][0].get_signal_bits(q), parts[1][0].get_signal_bits(q)])
        assert np.array_equal(both, full.get_signal_bits(q)), q


def test_word_shards_compose(engine):
    cd = sim.CompiledDesign(pipelined_cpu(), "Cpu8")
    half, cycles = 256, 300
    rom = cpu_rom_hashed(2 * half, seed=5)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    rec = ["out_pc", "out_acc"]
    full = sim.GpuBatchSimulator(cd, lanes=2 * half)
    full.set_memory_limbs("rom", rom)
    rf = full.run(cycles, stim=stim, record=rec, mode=sim.REC_HASH)
    hs = []
    for k, base in enumerate((0, half)):
        g = sim.GpuBatchSimulator(cd, lanes=half)
        g.set_memory_limbs("rom", rom[:, :, base:base + half])
        hs.append(g.run(cycles, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=base)["hash"])
        assert np.array_equal(g.get_signal_limbs("acc"), full.get_signal_limbs("acc")[:, base:base + half])
    assert np.array_equal(hs[0] + hs[1], rf["hash"])


def test_lane_base_must_be_word_aligned(netlist):
    meta, cd, od = netlist
    stim, rec = netlist_run_spec(meta)
    g = sim.GpuBatchSimulator(cd, lanes=64)
    with pytest.raises(sim.RrtlError, match="E_GPU_LANE_BASE"):
        g.run(2, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=16)


@pytest.mark.parametrize("path", ["fused", "plain", "compiled", "queue"])
def test_uniform_stimulus_fault_free_lanes_never_detect(netlist, path):
    meta, cd, od = netlist
    lanes, cycles = 700, 30
    stim, rec = netlist_run_spec(meta, uniform=True)
    g = sim.GpuBatchSimulator(cd, lanes=lanes)
    mode = sim.REC_DETECT | sim.REC_HASH
    if path == "plain":
        g.set_path(sim.PATH_PLAIN)
    elif path == "fused":
        g.set_tile_words(8)
    if path == "queue":
        ctx = sim.default_context()
        j = ctx.submit(g, cycles, seed=8, stim=stim, record=rec, mode=mode)
        ctx.launch()
        ctx.wait()
        res = j.outputs
    else:
        res = g.run(cycles, seed=8, stim=stim, record=rec, mode=mode)
    assert (res["detect"] == 0xFFFFFFFF).all()
    ref = oracle_bp_run(od, lanes, cycles, 8, [(od.signal(n), k, p) for n, k, p in stim],
                        [od.signal(x) for x in rec], 2)
    assert np.array_equal(res["hash"], ref["hash"])
