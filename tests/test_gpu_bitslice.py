"""Bit-sliced multi-bit designs on the GPU gate engine against the packed
oracle of the original design, per lane and cycle."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, counter

from .designs import random_word_design

pytestmark = pytest.mark.gpu


def _limbs(vals, w):
    n = max(1, (w + 31) // 32)
    return np.array([[(v >> (32 * l)) & 0xFFFFFFFF for v in vals] for l in range(n)], dtype=np.uint32)


def _run_both(js, top, inputs, observe, lanes, cycles, seed):
    orig = ob.OracleDesign(js, top)
    po = ob.PackedSim(orig, lanes)
    bs = sim.BitSliceSimulator(js, top, lanes)
    assert bs.design.info.engine == sim.ENGINE_GATE
    rng = Rng(seed)
    for c in range(cycles):
        for name, w in inputs:
            vals = [rng.next() & ((1 << w) - 1) if w < 64 else rng.next() for _ in range(lanes)]
            if name == "rst":
                vals = [1 if c < 2 else 0] * lanes
            po.set_signal(orig.signal(name), _limbs(vals, w), settle=False)
            bs.set_signal(name, vals)
        po.tick()
        bs.tick()
        for name, w in observe:
            a = po.get_signal(orig.signal(name))
            ref = [sum(int(a[l, k]) << (32 * l) for l in range(a.shape[0])) for k in range(lanes)]
            assert bs.get_signal(name) == ref, (c, name)


@pytest.mark.parametrize("seed", range(6))
def test_random_designs_bitsliced_match_oracle(engine, seed):
    d, meta = random_word_design(300 + seed, n_wires=14, depth=3, n_mems=0, async_resets=False, no_mul=True)
    inputs = [("clk", 1), ("rst", 1)] + list(meta["inputs"])
    observe = list(meta["outputs"]) + list(meta["regs"])
    _run_both(d.to_json(), meta["top"], inputs, observe, lanes=100, cycles=12, seed=seed)


def test_counter_bitsliced_many_lanes(engine):
    _run_both(counter().to_json(), "Counter", [("clk", 1), ("rst", 1), ("en", 1)], [("count", 8)], lanes=2000,
              cycles=40, seed=7)
