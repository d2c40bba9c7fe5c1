"""The CPU oracle against the reference's own known answers (no GPU)."""
import numpy as np

from oracle import binding as ob
from rrtl_gb300.builder import Design, lit_u, mux, uint
from rrtl_gb300.workloads import Rng, smix64, stim_word

from .helpers import crc32_netlist_json, oracle_bp_run


def _counter():
    d = Design()
    m = d.module("Counter")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    en = m.input("en", uint(1))
    count = m.reg("count", uint(8))
    m.clock(count, clk)
    m.reset(count, rst, 0)
    m.next(count, mux(en, count + lit_u(1, 8), count))
    return d


def test_counter_known_answer_packed_and_scalar(oracle_lib):
    """crates/rrtl-gpu-sim/src/lib.rs:5763-5787 -> [1, 0, 2, 2]."""
    od = ob.OracleDesign(_counter().to_json(), "Counter")
    p = ob.PackedSim(od, 4)
    p.set_signal(od.signal("rst"), [1, 0, 0, 0])
    p.set_signal(od.signal("en"), [1, 0, 1, 1])
    p.tick()
    p.set_signal(od.signal("rst"), [0, 0, 0, 0])
    p.tick()
    assert list(p.get_signal(od.signal("count"))[0]) == [1, 0, 2, 2]
    got = []
    for lane in range(4):
        s = ob.ScalarSim(od)
        s.set("rst", [1, 0, 0, 0][lane])
        s.set("en", [1, 0, 1, 1][lane])
        s.tick()
        s.set("rst", 0)
        s.tick()
        got.append(s.get("count"))
    assert got == [1, 0, 2, 2]


def test_crc32_netlist_scalar_matches_crc_step(oracle_lib):
    """crates/rrtl-sim-ir/examples/netlist_crc32.rs:26-51: 64 cycles, rst on cycle 0."""
    d = crc32_netlist_json()
    od = ob.OracleDesign(d.to_json(), "crc32")
    s = ob.ScalarSim(od)
    s.set("clk", 1)
    ref = 0
    for cyc in range(64):
        rst = 1 if cyc < 1 else 0
        din = (cyc * 2654435761 >> 13) & 0xFF
        s.set("rst", rst)
        for i in range(8):
            s.set(f"din_{i}", (din >> i) & 1)
        s.tick()
        ref = 0xFFFFFFFF if rst else ob.crc_step(ref, din)
        assert sum(s.get(f"crc_{i}") << i for i in range(32)) == ref


def test_crc32_netlist_bitparallel_per_lane_matches_scalar(oracle_lib):
    """Per-lane stimulus din = ((cyc + l) * 2654435761 >> 13) & 0xff (netlist_crc32.rs:63-83)."""
    d = crc32_netlist_json()
    od = ob.OracleDesign(d.to_json(), "crc32")
    lanes = 40
    bp = ob.BitParallel(od, lanes)
    sc = [ob.ScalarSim(od) for _ in range(lanes)]
    for l in range(lanes):
        bp.set(od.signal("clk"), l, 1)
        sc[l].set("clk", 1)
    for cyc in range(24):
        for l in range(lanes):
            din = ((cyc + l) * 2654435761 >> 13) & 0xFF
            bp.set(od.signal("rst"), l, cyc < 1)
            sc[l].set("rst", int(cyc < 1))
            for i in range(8):
                bp.set(od.signal(f"din_{i}"), l, (din >> i) & 1)
                sc[l].set(f"din_{i}", (din >> i) & 1)
        bp.tick()
        for l in range(lanes):
            sc[l].tick()
            a = sum(bp.get(od.signal(f"crc_{i}"), l) << i for i in range(32))
            assert a == sum(sc[l].get(f"crc_{i}") << i for i in range(32))


def test_crc32_fault_sim_known_answer(oracle_lib):
    """Stuck-at-0/1 on all 32 flops, lane 0 golden, 96 cycles: 64/64 detected,
    latency min 1 / max 6 / mean 2.1 (crates/rrtl-sim-ir/examples/fault_sim.rs;
    docs/rrtl-optimizations.md:1411-1416)."""
    d = crc32_netlist_json()
    od = ob.OracleDesign(d.to_json(), "crc32")
    regs = [i for i in range(od.num_signals) if od.kind(i) == 3]
    faults = [(r, v) for r in regs for v in (0, 1)]
    bp = ob.BitParallel(od, len(faults) + 1)
    for f, (sig, v) in enumerate(faults):
        bp.set_force(sig, f + 1, v)
    bp.set_all(od.signal("clk"), 1)
    outs = [od.signal(f"crc_{i}") for i in range(32)]
    det = [None] * len(faults)
    for cyc in range(96):
        bp.set_all(od.signal("rst"), cyc < 1)
        din = (cyc * 2654435761 >> 13) & 0xFF
        for i in range(8):
            bp.set_all(od.signal(f"din_{i}"), (din >> i) & 1)
        bp.tick()
        words = np.stack([bp.get_bits(o) for o in outs])
        vals = [sum(((int(words[b][l // 32]) >> (l % 32)) & 1) << b for b in range(32)) for l in range(len(faults) + 1)]
        for f in range(len(faults)):
            if det[f] is None and vals[f + 1] != vals[0]:
                det[f] = cyc
    lat = [c + 1 for c in det if c is not None]
    assert len(lat) == 64
    assert (min(lat), max(lat)) == (1, 6)
    assert round(sum(lat) / len(lat), 1) == 2.1


def test_crc32_atpg_vector_confirmed_on_the_bit_parallel_engine(oracle_lib):
    """The reference's symbolic ATPG test for crc_5 stuck-at-0 (din = 0x01,
    initial state 0), confirmed concretely: lane 0 golden, lane 1 faulted,
    one tick gives golden 0x690ce0ee and faulty 0x690ce0ce
    (crates/rrtl-sim-ir/examples/symbolic_exec.rs:192-212;
    docs/rrtl-optimizations.md:1931-1934)."""
    d = crc32_netlist_json()
    od = ob.OracleDesign(d.to_json(), "crc32")
    bp = ob.BitParallel(od, 2)
    din, state = 0x01, 0
    for l in range(2):
        bp.set(od.signal("clk"), l, 1)
        bp.set(od.signal("rst"), l, 0)
        for i in range(8):
            bp.set(od.signal(f"din_{i}"), l, (din >> i) & 1)
        for k in range(32):
            bp.set(od.signal(f"crc_{k}"), l, (state >> k) & 1)
    bp.set_force(od.signal("crc_5"), 1, 0)
    bp.tick()
    golden, faulty = (sum(bp.get(od.signal(f"crc_{i}"), l) << i for i in range(32)) for l in range(2))
    assert (golden, faulty) == (0x690CE0EE, 0x690CE0CE)
    assert golden == ob.crc_step(state, din)
    # the same vector through the run protocol the GPU engines follow:
    # constant stimulus; a cycle records before its clock edge, so the second
    # cycle's row holds the state after one edge
    stim = [(od.signal("clk"), 3, 1), (od.signal("rst"), 3, 0)]
    stim += [(od.signal(f"din_{i}"), 3, (din >> i) & 1) for i in range(8)]
    tr = oracle_bp_run(od, 2, 2, 0, stim, [od.signal(f"crc_{i}") for i in range(32)], 1,
                       faults=[(1, od.signal("crc_5"), 0)])["trace"]
    row = [[sum(((int(tr[c, i, 0]) >> l) & 1) << i for i in range(32)) for l in range(2)] for c in range(2)]
    assert row == [[0, 0], [0x690CE0EE, 0x690CE0CE]]


def test_reconvergent_cone_fault_answers(oracle_lib):
    """The reference's ATPG answers on y = (a&b) | (a&~b), confirmed
    exhaustively on the concrete engine (comb-wire forces clamp on store):
    nb stuck-at-1 is untestable, nb stuck-at-0 is detected only by a=1,b=0,
    w stuck-at-0 only by a=1,b=1, v stuck-at-1 by a=0
    (crates/rrtl-sim-ir/examples/symbolic_exec.rs:76-135;
    docs/rrtl-optimizations.md:1926-1929). One 32-lane word per fault, lanes
    1-4 of it take the four input pairs, through the engines' run protocol."""
    d = Design()
    m = d.module("Redund")
    a, b = m.input("a", uint(1)), m.input("b", uint(1))
    nb, w, v = m.wire("nb", uint(1)), m.wire("w", uint(1)), m.wire("v", uint(1))
    y = m.output("y", uint(1))
    m.assign(nb, ~b)
    m.assign(w, a & b)
    m.assign(v, a & nb)
    m.assign(y, w | v)
    od = ob.OracleDesign(d.to_json(), "Redund")
    faults = [("nb", 1), ("nb", 0), ("w", 0), ("v", 1)]
    pairs = [(0, 0), (0, 1), (1, 0), (1, 1)]
    trace = np.zeros((1, 2, len(faults)), np.uint32)
    for f in range(len(faults)):
        for k, (av, bv) in enumerate(pairs):
            trace[0, 0, f] |= av << (k + 1)
            trace[0, 1, f] |= bv << (k + 1)
    stim = [(od.signal("a"), 4, 0), (od.signal("b"), 4, 1)]
    placed = [(32 * f + k + 1, od.signal(n), val) for f, (n, val) in enumerate(faults) for k in range(4)]
    tr = oracle_bp_run(od, 32 * len(faults), 1, 0, stim, [od.signal("y")], 1, faults=placed,
                       input_trace=trace)["trace"]
    detected = {}
    for f, fault in enumerate(faults):
        ys = [(int(tr[0, 0, f]) >> (k + 1)) & 1 for k in range(4)]
        detected[fault] = [pairs[k] for k in range(4) if ys[k] != pairs[k][0]]  # golden y = a
    assert detected == {("nb", 1): [], ("nb", 0): [(1, 0)], ("w", 0): [(1, 1)], ("v", 1): [(0, 0), (0, 1)]}


def test_stuck_at_force_clamps_and_isolates_lanes(oracle_lib):
    """crates/rrtl-sim-ir/src/bitparallel.rs:582-628."""
    d = Design()
    m = d.module("Chain")
    clk = m.input("clk", uint(1))
    a = m.input("a", uint(1))
    b = m.input("b", uint(1))
    q = m.reg("q", uint(1))
    w1 = m.wire("w1", uint(1))
    w2 = m.wire("w2", uint(1))
    m.clock(q, clk)
    m.assign(w1, a & b)
    m.assign(w2, w1 ^ q)
    m.next(q, w2)
    o = m.output("o", uint(1))
    m.assign(o, q)
    od = ob.OracleDesign(d.to_json(), "Chain")
    bp, ctl = ob.BitParallel(od, 3), ob.BitParallel(od, 3)
    bp.set_force(od.signal("q"), 1, 1)
    bp.set_force(od.signal("q"), 2, 0)
    for sim in (bp, ctl):
        for l in range(3):
            for n in ("clk", "a", "b"):
                sim.set(od.signal(n), l, 1)
    for _ in range(12):
        bp.tick()
        ctl.tick()
        assert bp.get(od.signal("o"), 1) == 1
        assert bp.get(od.signal("o"), 2) == 0
        assert bp.get(od.signal("o"), 0) == ctl.get(od.signal("o"), 0)
    assert bp.get(od.signal("o"), 1) != bp.get(od.signal("o"), 0)


def test_stimulus_hash_copies_agree(oracle_lib):
    """The stimulus/hash convention exists in C++ (engines), C (oracle) and
    Python (workloads); pin all three to the same known answers."""
    L = ob.lib()
    assert smix64(0) == 0xE220A8397B1DCDAF  # SplitMix64 first output for state 0
    rng = Rng(7)
    for _ in range(200):
        s, st, c, i = rng.next(), rng.below(1 << 20), rng.below(1 << 32), rng.below(1 << 30)
        assert L.orc_stim_word(s, st, c, i) == stim_word(s, st, c, i)
    assert stim_word(1, 0, 0, 0) == L.orc_stim_word(1, 0, 0, 0)
    assert L.orc_hash_term(3, 1, 5, 0xDEADBEEF) == L.orc_hash_term(3, 1, 5, 0xDEADBEEF)
    assert L.orc_hash_term(3, 1, 5, 0xDEADBEEF) != L.orc_hash_term(4, 1, 5, 0xDEADBEEF)


def test_comb_fused_tick_many_matches_tick_loop(oracle_lib):
    """tick_many(n) == n x tick() for n in {0,1,2,3,17,64,257}
    (crates/rrtl-sim-ir/src/lib.rs:14634; docs/rrtl-optimizations.md:846-848)."""
    from .designs import random_word_design

    d, meta = random_word_design(5, async_resets=False)
    od = ob.OracleDesign(d.to_json(), meta["top"])
    for n in (0, 1, 2, 3, 17, 64, 257):
        a, b = ob.PackedSim(od, 5), ob.PackedSim(od, 5)
        for name, w in meta["inputs"]:
            v = np.full((max(1, (w + 31) // 32), 5), 0x9E37 & ((1 << min(w, 32)) - 1), dtype=np.uint32)
            a.set_signal(od.signal(name), v)
            b.set_signal(od.signal(name), v)
        a.tick_many(n)
        for _ in range(n):
            b.tick()
        va, ma = a.snapshot()
        vb, mb = b.snapshot()
        assert np.array_equal(va, vb) and np.array_equal(ma, mb)
