"""GPU parity of the device job queue and the graph-captured plain path.

A queued job must give exactly what the same run gives alone on a fresh
batch (which the other GPU tests pin to the oracle): per-cycle traces and
hashes, first-detection cycles and the final net state.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, counter, gate_netlist, netlist_run_spec

from .helpers import oracle_bp_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def designs(engine):
    out = []
    for ng, nff, depth, seed in [(2000, 96, 8, 11), (6000, 300, 14, 12), (24000, 900, 24, 13)]:
        d, meta = gate_netlist(n_gates=ng, n_ff=nff, n_pi=16, n_po=24, depth=depth, seed=seed)
        js = d.to_json()
        out.append((meta, sim.CompiledDesign(js, meta.top), js))
    return out


def _job_specs():
    rng = Rng(2024)
    specs = []
    lanes_opts = [1, 33, 300, 1000, 2048, 5000]
    for i in range(14):
        specs.append(dict(design=i % 3, lanes=lanes_opts[rng.below(len(lanes_opts))], cycles=[1, 7, 25, 60][rng.below(4)],
                          seed=1000 + i, words=[0, 0, 8, 4, 2, 1][rng.below(6)], faults=(i % 4 == 3)))
    return specs


def _make_batch(designs, spec):
    meta, cd, _ = designs[spec["design"]]
    g = sim.GpuBatchSimulator(cd, lanes=spec["lanes"])
    if spec["words"]:
        g.set_tile_words(spec["words"])
    if spec["faults"]:
        rng = Rng(spec["seed"])
        sites = meta.gate_names + meta.regs + meta.outputs
        g.set_faults([(l, sites[rng.below(len(sites))], rng.below(2)) for l in range(spec["lanes"]) if l % 32])
    return g


def _mode(spec):
    return sim.REC_HASH | sim.REC_TRACE | (sim.REC_DETECT if spec["faults"] else 0)


def test_queue_jobs_match_runs_alone(designs):
    ctx = sim.default_context()
    specs = _job_specs()
    queued = []
    for spec in specs:
        meta = designs[spec["design"]][0]
        stim, rec = netlist_run_spec(meta, uniform=spec["faults"])
        g = _make_batch(designs, spec)
        job = ctx.submit(g, spec["cycles"], seed=spec["seed"], stim=stim, record=rec, mode=_mode(spec))
        assert job.status == sim.JOB_QUEUED
        queued.append((spec, g, job))
    ctx.launch()
    ctx.wait()
    assert ctx.queue_ms > 0
    for spec, g, job in queued:
        assert job.status == sim.JOB_DONE
        meta = designs[spec["design"]][0]
        stim, rec = netlist_run_spec(meta, uniform=spec["faults"])
        alone = _make_batch(designs, spec)
        ref = alone.run(spec["cycles"], seed=spec["seed"], stim=stim, record=rec, mode=_mode(spec))
        for k in ("trace", "hash", "detect"):
            if ref[k] is not None:
                assert np.array_equal(job.outputs[k], ref[k]), (spec, k)
        for name in meta.regs[::11] + meta.outputs[::3]:
            assert np.array_equal(g.get_signal_bits(name), alone.get_signal_bits(name)), (spec, name)


def test_queue_job_matches_oracle(designs):
    meta, cd, js = designs[1]
    od = ob.OracleDesign(js, meta.top)
    stim, rec = netlist_run_spec(meta)
    ctx = sim.default_context()
    jobs = []
    for lanes, cycles, seed in [(77, 19, 5), (640, 9, 6)]:
        g = sim.GpuBatchSimulator(cd, lanes=lanes)
        jobs.append((lanes, cycles, seed, ctx.submit(g, cycles, seed=seed, stim=stim, record=rec,
                                                     mode=sim.REC_TRACE | sim.REC_HASH)))
    ctx.launch()
    ctx.wait()
    for lanes, cycles, seed, job in jobs:
        ref = oracle_bp_run(od, lanes, cycles, seed, [(od.signal(n), k, p) for n, k, p in stim],
                            [od.signal(r) for r in rec], 3)
        assert np.array_equal(job.outputs["trace"], ref["trace"])
        assert np.array_equal(job.outputs["hash"], ref["hash"])


def test_queue_fault_job_detection_matches_oracle(designs):
    """A fault-simulation job (one stuck-at fault per lane, lane-uniform
    stimulus, lane 0 of each word fault-free) on the persistent queue: its
    detection vector equals the bit-parallel oracle's with the same forces."""
    from rrtl_gb300.workloads import job_faults

    meta, cd, js = designs[1]
    od = ob.OracleDesign(js, meta.top)
    stim, rec = netlist_run_spec(meta, uniform=True)
    lanes, cycles, seed = 600, 40, 12
    faults = job_faults(meta, lanes, seed)
    ctx = sim.default_context()
    g = sim.GpuBatchSimulator(cd, lanes=lanes)
    g.set_faults(faults)
    job = ctx.submit(g, cycles, seed=seed, stim=stim, record=rec, mode=sim.REC_HASH | sim.REC_DETECT)
    ctx.launch()
    ctx.wait()
    ref = oracle_bp_run(od, lanes, cycles, seed, [(od.signal(n), k, p) for n, k, p in stim],
                        [od.signal(r) for r in rec], 6, faults=[(l, od.signal(s), v) for l, s, v in faults])
    assert np.array_equal(job.outputs["detect"], ref["detect"])
    assert np.array_equal(job.outputs["hash"], ref["hash"])
    n_det = int((ref["detect"] != 0xFFFFFFFF).sum())
    assert 0 < n_det < len(faults)


def test_queue_status_and_errors(designs):
    meta, cd, _ = designs[0]
    stim, rec = netlist_run_spec(meta)
    ctx = sim.default_context()
    g = sim.GpuBatchSimulator(cd, lanes=64)
    job = ctx.submit(g, 3, seed=1, stim=stim, record=rec, mode=sim.REC_HASH)
    with pytest.raises(sim.RrtlError) as e:
        ctx.submit(g, 3, seed=1, stim=stim, record=rec, mode=sim.REC_HASH)
    assert e.value.code == "E_QUEUE"
    assert ctx.poll(job.id) == sim.JOB_QUEUED
    ctx.launch()
    while ctx.poll(job.id) == sim.JOB_RUNNING:
        pass
    assert ctx.poll(job.id) == sim.JOB_DONE
    with pytest.raises(sim.RrtlError):
        ctx.poll(987654321)
    w = sim.GpuBatchSimulator(counter(), "Counter", lanes=8)
    with pytest.raises(sim.RrtlError) as e:
        ctx.submit(w, 2)
    assert e.value.code == "E_QUEUE"
    # the batch takes a new job once the last one finished
    job2 = ctx.submit(g, 2, seed=2, stim=stim, record=rec, mode=sim.REC_HASH)
    ctx.launch()
    ctx.wait()
    assert job2.status == sim.JOB_DONE


def test_plain_graph_path_matches_fused(designs):
    meta, cd, _ = designs[2]
    stim, rec = netlist_run_spec(meta)
    out = {}
    for path in (sim.PATH_FUSED, sim.PATH_PLAIN, sim.PATH_PLAIN_GRAPH):
        g = sim.GpuBatchSimulator(cd, lanes=3000)
        g.set_path(path)
        out[path] = g.run(31, seed=9, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    for path in (sim.PATH_PLAIN, sim.PATH_PLAIN_GRAPH):
        assert np.array_equal(out[path]["trace"], out[sim.PATH_FUSED]["trace"])
        assert np.array_equal(out[path]["hash"], out[sim.PATH_FUSED]["hash"])


def test_word_engine_graph_path_matches(engine):
    cd = sim.CompiledDesign(counter(), "Counter")
    res = {}
    for path in (sim.PATH_FUSED, sim.PATH_PLAIN_GRAPH):
        g = sim.GpuBatchSimulator(cd, lanes=1024)
        g.set_path(path)
        res[path] = g.run(300, seed=3, stim=[("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1),
                                             ("en", sim.STIM_RANDOM, 7)], record=["count"],
                          mode=sim.REC_TRACE | sim.REC_HASH)
    assert np.array_equal(res[sim.PATH_FUSED]["trace"], res[sim.PATH_PLAIN_GRAPH]["trace"])
    assert np.array_equal(res[sim.PATH_FUSED]["hash"], res[sim.PATH_PLAIN_GRAPH]["hash"])
