"""Word values of 65 to 128 bits on the GPU word engine against the packed
oracle (the reference's limb semantics, crates/rrtl-sim-ir/src/lib.rs:13018-13196;
its GPU interpreter goes to four limbs, crates/rrtl-gpu-sim/src/interp.rs:1810-1814).

At widths 63, 64, 65, 96, 127 and 128: add, sub, mul, unsigned and signed
lt, eq, sext, zext, concat, slice, trunc, mux, a wide accumulator and a
memory written and read every cycle; per-lane random inputs; the full trace
of every register and the output, on the compiled kernel (fused path) and
the interpreted kernel, bit-exact per lane per cycle."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim

from .designs import wide_ops_design
from .helpers import oracle_packed_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_WORD_INTERP])
@pytest.mark.parametrize("w", [63, 64, 65, 96, 127, 128])
def test_wide_ops_match_packed_oracle(engine, w, path):
    d, meta = wide_ops_design(w)
    js = d.to_json()
    top = meta["top"]
    od = ob.OracleDesign(js, top)
    lanes, cycles = 96, 40
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)] + [
        (n, sim.STIM_RANDOM, 10 + i) for i, (n, _) in enumerate(meta["inputs"])]
    rec = [n for n, _ in meta["regs"]] + ["o"]
    g = sim.GpuBatchSimulator(js, top, lanes)
    g.set_path(path)
    if path == sim.PATH_FUSED:
        active, _, why = g.design.word_jit()
        assert active, why
    res = g.run(cycles, seed=w, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    ref = oracle_packed_run(od, lanes, cycles, w, [(od.signal(n), k, p) for n, k, p in stim],
                            [od.signal(r) for r in rec], 3)
    assert np.array_equal(res["trace"], ref["trace"])
    assert np.array_equal(res["hash"], ref["hash"])
    # the state after the run, memories included
    v_gpu, m_gpu = g.snapshot_storage()
    v_or, m_or = ref["sim"].snapshot()
    assert np.array_equal(v_gpu, v_or)
    assert np.array_equal(m_gpu, m_or)
    assert (res["trace"] != 0).sum() > res["trace"].size // 4
