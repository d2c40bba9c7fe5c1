"""GPU tests of the serving loop (rrtl_server_*): each request's results are
bit-exact with the same run alone on a fresh batch, whether it ran alone or
in a mix of requests that overlapped on the device."""
import threading
import time

import numpy as np
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, counter, cpu_rom, gate_netlist, netlist_run_spec, pipelined_cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served_designs(engine):
    out = {}
    for key, (ng, nff, depth, seed) in {"n2k": (2000, 96, 8, 21), "n7k": (7000, 320, 16, 22)}.items():
        d, meta = gate_netlist(n_gates=ng, n_ff=nff, n_pi=16, n_po=24, depth=depth, seed=seed)
        stim, rec = netlist_run_spec(meta)
        out[key] = dict(cd=sim.CompiledDesign(d.to_json(), meta.top), meta=meta, stim=stim, rec=rec)
    out["counter"] = dict(cd=sim.CompiledDesign(counter(), "Counter"), meta=None,
                          stim=[("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 5)],
                          rec=["count"])
    out["cpu"] = dict(cd=sim.CompiledDesign(pipelined_cpu(), "Cpu8"), meta=None,
                      stim=[("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)], rec=["out_pc", "out_acc"])
    return out


def _requests(n=16, seed=77):
    rng = Rng(seed)
    keys = ["n2k", "n7k", "counter", "cpu"]
    reqs = []
    for i in range(n):
        k = keys[i % 4]
        lanes = [1, 40, 333, 1500, 3000][rng.below(5)]
        if k == "cpu":
            lanes = min(lanes, 300)
        reqs.append(dict(key=k, lanes=lanes, cycles=[0, 1, 17, 90, 250][rng.below(5)], seed=500 + i,
                         fault=(k.startswith("n") and rng.below(3) == 0)))
    return reqs


def _extras(req, d):
    faults, mems = (), None
    if req["fault"]:
        rng = Rng(req["seed"])
        meta = d["meta"]
        sites = meta.gate_names + meta.regs + meta.outputs
        faults = [(l, sites[rng.below(len(sites))], rng.below(2)) for l in range(req["lanes"]) if l % 32]
    if req["key"] == "cpu":
        mems = {"rom": cpu_rom(req["lanes"], seed=req["seed"])}
    mode = sim.REC_TRACE | sim.REC_HASH | (sim.REC_DETECT if req["fault"] else 0)
    return faults, mems, mode


def _offline(served_designs, req):
    d = served_designs[req["key"]]
    faults, mems, mode = _extras(req, d)
    g = sim.GpuBatchSimulator(d["cd"], lanes=req["lanes"])
    if faults:
        g.set_faults(faults)
    for name, arr in (mems or {}).items():
        g.set_memory_limbs(name, arr)
    return g.run(req["cycles"], seed=req["seed"], stim=d["stim"], record=d["rec"], mode=mode)


def _submit(server, served_designs, req):
    d = served_designs[req["key"]]
    faults, mems, mode = _extras(req, d)
    return server.submit(d["cd"], req["lanes"], req["cycles"], seed=req["seed"], stim=d["stim"], record=d["rec"],
                         mode=mode, faults=faults, memories=mems)


def _check(served, ref):
    for k in ("trace", "hash", "detect"):
        if ref[k] is not None:
            assert np.array_equal(served[k], ref[k]), k


def test_mixed_requests_match_offline_and_overlap(served_designs):
    reqs = _requests()
    refs = [_offline(served_designs, r) for r in reqs]
    server = sim.Server(chunk_cycles=16)
    handles = [None] * len(reqs)

    def producer():
        rng = Rng(3)
        for i, r in enumerate(reqs):
            handles[i] = _submit(server, served_designs, r)
            time.sleep(rng.below(3) * 0.002)

    t = threading.Thread(target=producer)
    t.start()
    t.join()
    server.drain()
    infos = []
    for h, ref in zip(handles, refs):
        info = h.info()
        assert info["status"] == sim.JOB_DONE
        _check(h.outputs, ref)
        infos.append(info)
    # some requests were on the device at the same time
    overlap = any(a["admit_ns"] < b["done_ns"] and b["admit_ns"] < a["done_ns"]
                  for i, a in enumerate(infos) for b in infos[i + 1:])
    assert overlap
    st = server.stats
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rounds"] >= 2
    server.close()


def test_one_at_a_time_budget_gives_same_results(served_designs):
    reqs = _requests(n=8, seed=78)
    refs = [_offline(served_designs, r) for r in reqs]
    server = sim.Server(hbm_budget=1, chunk_cycles=40)  # admits a request only when nothing else is active
    hs = [_submit(server, served_designs, r) for r in reqs]
    server.drain()
    infos = [h.info() for h in hs]
    for h, ref in zip(hs, refs):
        _check(h.outputs, ref)
    for i, a in enumerate(infos):
        for b in infos[i + 1:]:
            assert not (a["admit_ns"] < b["done_ns"] and b["admit_ns"] < a["done_ns"])
    server.close()


def test_server_errors(served_designs):
    server = sim.Server()
    d = served_designs["n2k"]
    with pytest.raises(sim.RrtlError) as e:
        server.submit(d["cd"], 0, 5, stim=d["stim"], record=d["rec"], mode=sim.REC_HASH)
    assert e.value.code == "E_GPU_LANES"
    h = server.submit(d["cd"], 64, 5, seed=1, stim=d["stim"], record=d["rec"], mode=sim.REC_HASH)
    h.wait(timeout_ms=60000)
    server.release(h.id)
    with pytest.raises(sim.RrtlError):
        server.info(h.id)
    # a request the engine rejects fails without stopping the server
    bad = server.submit(served_designs["counter"]["cd"], 8, 3, record=["count"], mode=sim.REC_DETECT | sim.REC_HASH,
                        faults=[(1, "count", 1)])
    with pytest.raises(sim.RrtlError):
        bad.wait(timeout_ms=60000)
    ok = server.submit(d["cd"], 32, 2, seed=2, stim=d["stim"], record=d["rec"], mode=sim.REC_HASH)
    ok.wait(timeout_ms=60000)
    server.close()


def test_shortest_first_policy_gives_same_results(served_designs):
    """Under shortest-remaining-first rounds every request still ends with
    the results of its run alone, and a short request submitted beside long
    ones finishes first."""
    reqs = _requests(n=10, seed=91)
    refs = [_offline(served_designs, r) for r in reqs]
    server = sim.Server(chunk_cycles=64, round_us=2000, policy=sim.SERVE_SHORTEST_FIRST)
    hs = [_submit(server, served_designs, r) for r in reqs]
    server.drain()
    for h, ref in zip(hs, refs):
        assert h.info()["status"] == sim.JOB_DONE
        _check(h.outputs, ref)
    server.close()
    with pytest.raises(sim.RrtlError):
        sim.Server(policy=7)
