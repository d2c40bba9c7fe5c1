"""The compiled word kernel's emitter and its NVRTC compile, on the CPU (no
device needed): sources compile for sm_103a and hold one statement per word
instruction of each stream."""
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import counter, pipelined_cpu

from .designs import random_word_design


def _compile(d, top):
    try:
        return sim.word_jit_emit(d, top, "sm_103a")
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise


def test_counter_source_shape():
    src, cub, _ = sim.word_jit_emit(counter(), "Counter")
    assert cub == 0
    assert 'extern "C" __global__' in src and "rrtl_word_jit" in src
    assert "JitLane::settle()" in src and "JitLane::edge()" in src
    # count' = rst ? 0 : (en ? count + 1 : count): one capture, committed after the captures
    assert src.count("c0 = (uint32_t)t;") == 1
    assert src.rstrip().endswith("}")


@pytest.mark.parametrize("which", ["counter", "cpu", "rand0", "rand1", "rand_mems"])
def test_sources_compile_for_sm103a(which):
    if which == "counter":
        d, top = counter(), "Counter"
    elif which == "cpu":
        d, top = pipelined_cpu(), "Cpu8"
    elif which == "rand_mems":
        d, meta = random_word_design(501, n_wires=18, n_mems=10)
        top = meta["top"]
    else:
        d, meta = random_word_design(int(which[-1]) + 40)
        top = meta["top"]
    src, cub, log = _compile(d, top)
    assert cub > 0, log
    assert "error" not in log.lower()


@pytest.mark.parametrize("w", [65, 96, 128])
def test_wide_value_sources_compile_for_sm103a(w):
    """Values of 65 to 128 bits run on 128-bit integers in slot pairs."""
    from .designs import wide_ops_design

    d, meta = wide_ops_design(w)
    src, cub, log = _compile(d, meta["top"])
    assert cub > 0, log
    assert "u128" in src


def test_values_past_128_bits_are_outside_the_word_engine():
    from rrtl_gb300.builder import Design, uint

    d = Design()
    m = d.module("Wide")
    clk = m.input("clk", uint(1))
    a = m.input("a", uint(130))
    r = m.reg("r", uint(130))
    m.clock(r, clk)
    m.next(r, a)
    o = m.output("o", uint(130))
    m.assign(o, r)
    with pytest.raises(sim.RrtlError) as e:
        sim.word_jit_emit(d, "Wide")
    assert e.value.code == "E_WORD_SCOPE" and e.value.status == 7  # RRTL_E_UNSUPPORTED


def _run_for(design, top, stim, record, mode):
    """A Run naming packed signal indices (looked up through the oracle's lowering)."""
    import ctypes

    from oracle import binding as ob

    od = ob.OracleDesign(design.to_json(), top)
    st = (sim.Stim * max(1, len(stim)))(*[sim.Stim(od.signal(n), k, p) for n, k, p in stim])
    rec = (ctypes.c_uint32 * max(1, len(record)))(*[od.signal(n) for n in record])
    r = sim.Run()
    r.n_stim, r.stim = len(stim), st
    r.n_record, r.record = len(record), rec
    r.record_mode = mode
    r._keep = (st, rec)
    return r


@pytest.mark.parametrize("which", ["counter", "cpu"])
def test_run_specialised_sources_compile(which):
    """The kernel compiled for one run's tables holds them as constants."""
    if which == "counter":
        d, top = counter(), "Counter"
        stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 0)]
        rec = ["out"]
    else:
        d, top = pipelined_cpu(), "Cpu8"
        stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
        rec = ["out_pc", "out_acc"]
    run = _run_for(d, top, stim, rec, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT)
    src, cub, log = sim.word_jit_emit(d, top, None, run)
    assert "struct RunSpec" in src and f"n_stim() {{ return {len(stim)}u; }}" in src
    assert "JitDynamicRun" not in src
    src, cub, log = _compile_run(d, top, run)
    assert cub > 0, log


def _compile_run(d, top, run):
    try:
        return sim.word_jit_emit(d, top, "sm_103a", run)
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise


@pytest.mark.parametrize("which", ["crc32", "netlist"])
def test_compiled_gate_kernel_sources_compile(which):
    """The compiled gate kernel (one thread per 32-lane word, one LOP3 per
    cell) for the reference's crc32 netlist and a generated netlist."""
    from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

    from .helpers import crc32_netlist_json

    if which == "crc32":
        d, top = crc32_netlist_json(), "crc32"
        stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)] + [(f"din_{i}", sim.STIM_RANDOM, i)
                                                                           for i in range(8)]
        rec = [f"crc_{i}" for i in range(32)]
    else:
        d, meta = gate_netlist(n_gates=900, n_ff=40, n_pi=8, n_po=8, depth=8, seed=3)
        top = meta.top
        stim, rec = netlist_run_spec(meta)
    run = _run_for(d, top, stim, rec, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT)
    src, _, _ = sim.gate_jit_emit(d, top, run)
    assert src.count("lop3<") >= 2 * 100  # the cells, in the cycle body and the closing settle
    try:
        src, cub, log = sim.gate_jit_emit(d, top, run, "sm_103a")
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log


@pytest.mark.parametrize("n_ff,mode", [(0, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT), (40, 0)])
def test_compiled_gate_kernel_edge_shapes_compile(n_ff, mode):
    """A netlist without registers, and a run that records nothing."""
    from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

    d, meta = gate_netlist(n_gates=200, n_ff=n_ff, n_pi=4, n_po=4, depth=5, seed=11)
    stim, rec = netlist_run_spec(meta)
    run = _run_for(d, meta.top, stim, rec if mode else [], mode)
    try:
        src, cub, log = sim.gate_jit_emit(d, meta.top, run, "sm_103a")
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log


def test_two_warp_split_source_compiles():
    """The two-warp form of the pipelined CPU's run kernel: both halves, the
    register exchange and the split run protocol compile for sm_103a; a design
    with an asynchronous reset does not split."""
    d, top = pipelined_cpu(), "Cpu8"
    run = _run_for(d, top, [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)], ["out_pc", "out_acc"],
                   sim.REC_HASH)
    src, _, _ = sim.word_jit_emit(d, top, None, run, split=True)
    assert "word_jit_run_split" in src and "settle_part" in src and "xin_all" in src
    try:
        src, cub, log = sim.word_jit_emit(d, top, "sm_103a", run, split=True)
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log
    from rrtl_gb300.builder import Design, lit_u, uint

    a = Design()
    m = a.module("A")
    clk, rst = m.input("clk", uint(1)), m.input("rst", uint(1))
    r = m.reg("r", uint(8))
    m.clock(r, clk)
    m.async_reset(r, rst, 3)
    m.next(r, r + lit_u(1, 8))
    o = m.output("o", uint(8))
    m.assign(o, r)
    run = _run_for(a, "A", [("clk", sim.STIM_CONST, 1)], ["o"], sim.REC_HASH)
    with pytest.raises(sim.RrtlError) as e:
        sim.word_jit_emit(a, "A", None, run, split=True)
    assert e.value.code == "E_WORD_JIT_SPLIT"


@pytest.mark.parametrize("seed", range(8))
def test_run_kernels_of_random_designs_compile(seed):
    """Every instruction form the emitter has (64- and 32-bit arithmetic,
    compares at every width, slices past 32 bits, sign extension, concat,
    memories in and beyond the placement table, resets of every kind) in
    kernels compiled for a run: random designs with all record modes."""
    d, meta = random_word_design(1200 + seed, n_wires=24, depth=4, n_mems=3 if seed % 2 else 9)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim += [(n, sim.STIM_RANDOM, i + 7) for i, (n, w) in enumerate(meta["inputs"])]
    rec = [n for n, w in meta["outputs"]]
    run = _run_for(d, meta["top"], stim, rec, sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT)
    try:
        src, cub, log = sim.word_jit_emit(d, meta["top"], "sm_103a", run)
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log
    assert "struct RunSpec" in src


def test_compiled_gate_kernel_of_a_plane_design_compiles():
    """A bit-sliced design's plane netlist (deep, narrow levels: the compiled
    gate kernel's case) compiles; its cells are one LOP3 each."""
    from rrtl_gb300.workloads import narrow_alu

    planes = sim.bitslice_json(narrow_alu(16), "Alu")
    stim = [("__bitslice_clk", sim.STIM_CONST, 1), ("rst[0]", sim.STIM_PULSE, 1)]
    stim += [(f"din[{p}]", sim.STIM_RANDOM, p) for p in range(16)]
    rec = [f"out[{p}]" for p in range(16)] + ["flag[0]"]
    from oracle import binding as ob

    od = ob.OracleDesign(planes, "Alu")
    import ctypes

    st = (sim.Stim * len(stim))(*[sim.Stim(od.signal(n), k, p) for n, k, p in stim])
    rc = (ctypes.c_uint32 * len(rec))(*[od.signal(n) for n in rec])
    run = sim.Run()
    run.n_stim, run.stim = len(stim), st
    run.n_record, run.record = len(rec), rc
    run.record_mode = sim.REC_HASH | sim.REC_TRACE
    try:
        src, cub, log = sim.gate_jit_emit(planes, "Alu", run, "sm_103a")
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log
    assert src.count("lop3<") >= 2 * 500


@pytest.mark.parametrize("which,w", [("netlist", 8), ("netlist", 4), ("crc32", 2), ("plane", 1)])
def test_fused_kernel_compiled_for_a_design(which, w):
    """The fused gate kernel compiled for a design's truth-table classes: its
    dispatch lists exactly those classes (and 0, an empty run), and it
    compiles for sm_103a at every tile width."""
    from rrtl_gb300.workloads import gate_netlist, narrow_alu

    from .helpers import crc32_netlist_json

    if which == "netlist":
        d, meta = gate_netlist(n_gates=3000, n_ff=64, n_pi=16, n_po=16, depth=12, seed=5)
        js, top = d.to_json(), meta.top
    elif which == "crc32":
        js, top = crc32_netlist_json(), "crc32"
    else:
        js, top = sim.bitslice_json(narrow_alu(16), "Alu"), "Alu"
    src, _, _ = sim.gate_fused_jit_emit(js, top, w)
    line = next(l for l in src.splitlines() if l.startswith("#define RRTL_LUT_CLASSES(X)"))
    listed = [int(t[2:-1]) for t in line.split()[2:]]
    assert listed[0] == 0 and listed == sorted(set(listed)) and len(listed) < 80
    assert f"fused_kernel_body<{w}, true>" in src and "#define RRTL_FUSED_WARPS 16" in src
    try:
        src, cub, log = sim.gate_fused_jit_emit(js, top, w, "sm_103a")
    except sim.RrtlError as e:
        if "NVRTC not found" in str(e):
            pytest.skip("NVRTC is not installed")
        raise
    assert cub > 0, log
