"""The per-design compiled gate kernel against the fused and plain gate
kernels and the bit-parallel oracle.

Netlists whose live nets fit in registers (crc32) run the compiled kernel
on the default path, so the crc32 oracle tests elsewhere already check it; these tests pin that it is the kernel that runs and that it equals the
other paths under every record mode and stimulus kind."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

from .helpers import crc32_netlist_json, oracle_bp_run

pytestmark = pytest.mark.gpu


def _paths(cd, lanes, cycles, stim, rec, mode, input_trace=None, seed=3):
    out = {}
    for key, path, words in (("compiled", sim.PATH_FUSED, 0), ("fused", sim.PATH_FUSED, 8), ("plain", sim.PATH_PLAIN, 0)):
        g = sim.GpuBatchSimulator(cd, lanes=lanes)
        g.set_path(path)
        if words:
            g.set_tile_words(words)
        res = g.run(cycles, seed=seed, stim=stim, record=rec, mode=mode, input_trace=input_trace)
        out[key] = (res, g)
    return out


@pytest.mark.parametrize("lanes", [1, 33, 2048, 262144])
def test_crc32_compiled_equals_fused_and_plain(engine, lanes):
    d = crc32_netlist_json()
    cd = sim.CompiledDesign(d, "crc32")
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)] + [(f"din_{i}", sim.STIM_RANDOM, 40 + i)
                                                                       for i in range(8)]
    rec = [f"crc_{i}" for i in range(32)]
    cycles = 50 if lanes > 10000 else 120
    out = _paths(cd, lanes, cycles, stim, rec, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT)
    assert out["compiled"][1].tile_words == 0 and out["fused"][1].tile_words == 8
    for key in ("fused", "plain"):
        for k in ("trace", "hash", "detect"):
            assert np.array_equal(out["compiled"][0][k], out[key][0][k]), (key, k)
        for name in rec[::5]:
            assert np.array_equal(out["compiled"][1].get_signal(name), out[key][1].get_signal(name)), (key, name)


@pytest.mark.parametrize("seed", range(4))
def test_small_netlists_compiled_match_oracle(engine, seed, monkeypatch):
    # these netlists have more live nets than the automatic choice puts in
    # registers: force the compiled kernel
    monkeypatch.setenv("RRTL_GATE_JIT", "2")
    d, meta = gate_netlist(n_gates=300 + 150 * seed, n_ff=24 + 8 * seed, n_pi=12, n_po=16, depth=6 + seed, seed=70 + seed)
    js = d.to_json()
    cd = sim.CompiledDesign(js, meta.top)
    od = ob.OracleDesign(js, meta.top)
    stim, rec = netlist_run_spec(meta)
    lanes, cycles = 333, 40
    # one input from a trace, to cover every stimulus kind
    tr_name = meta.inputs[0]
    stim = [s for s in stim if s[0] != tr_name] + [(tr_name, sim.STIM_TRACE, 0)]
    rng = np.random.default_rng(seed)
    trace = rng.integers(0, 2**32, size=(cycles, 1, (lanes + 31) // 32), dtype=np.uint64).astype(np.uint32)
    g = sim.GpuBatchSimulator(cd, lanes=lanes)
    res = g.run(cycles, seed=5, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH, input_trace=trace)
    assert g.tile_words == 0  # the compiled kernel ran
    ref = oracle_bp_run(od, lanes, cycles, 5, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec],
                        3, input_trace=trace)
    assert np.array_equal(res["trace"], ref["trace"])
    assert np.array_equal(res["hash"], ref["hash"])
    out = _paths(cd, lanes, cycles, stim, rec, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT, input_trace=trace, seed=5)
    for k in ("trace", "hash", "detect"):
        assert np.array_equal(out["compiled"][0][k], out["fused"][0][k]), k
    for name in meta.regs[::3] + meta.gate_names[::37]:
        assert np.array_equal(out["compiled"][1].get_signal_bits(name), out["plain"][1].get_signal_bits(name)), name


def test_faults_and_explicit_widths_use_the_fused_kernel(engine):
    d = crc32_netlist_json()
    cd = sim.CompiledDesign(d, "crc32")
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)] + [(f"din_{i}", sim.STIM_RANDOM, i) for i in range(8)]
    rec = [f"crc_{i}" for i in range(32)]
    g = sim.GpuBatchSimulator(cd, lanes=64)
    g.set_faults([(l, f"crc_{l % 32}", l // 32) for l in range(1, 64) if l % 32])
    g.run(10, stim=stim, record=rec, mode=sim.REC_DETECT)
    assert g.tile_words != 0
    g2 = sim.GpuBatchSimulator(cd, lanes=64)
    g2.set_tile_words(4)
    g2.run(10, stim=stim, record=rec, mode=sim.REC_HASH)
    assert g2.tile_words == 4
