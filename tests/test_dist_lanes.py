"""Multi-GPU path of the benchmark on CPU: world_size-2 gloo ranks each own a
lane shard (no data-path collective); the step time is the max over ranks and
the throughput counts every rank's lanes (bench.py --gpus N semantics)."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        lanes_per_rank, cycles, steps = 4096, 100, 5
        my_ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        ms = bench.reduce_max(dist, my_ms)
        value = bench.throughput(ws, lanes_per_rank, cycles, steps, ms)
        first, last = bench.lane_shard(ws * lanes_per_rank, rank, ws)
        gathered = [None] * ws
        dist.all_gather_object(gathered, (first, last, ms, value))
        if rank == 0:
            out.put(gathered)
    finally:
        dist.destroy_process_group()


def test_two_rank_lane_shards_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 2000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (f0, l0, ms0, v0), (f1, l1, ms1, v1) = got
    assert (f0, l0, f1, l1) == (0, 4096, 4096, 8192)  # disjoint, covering, contiguous
    assert ms0 == ms1 == 15.0  # max over ranks
    assert v0 == v1 == pytest.approx(2 * 4096 * 100 * 5 / 0.015)


def _failing_rank(rank, ws, port, out):
    """Rank 1 fails between steps (raises, then its process exits); rank 0
    learns of it at its next collective, which errors instead of hanging."""
    import time

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank), RRTL_DIST_TIMEOUT_S="20")
    _, _, _, d = bench.dist_setup()
    bench.reduce_max(d, 1.0)  # one step that both ranks finish
    if rank == 1:
        raise SystemExit(3)  # a failure on the host between steps
    t0 = time.time()
    try:
        bench.reduce_max(d, 2.0)
        out.put(("no error", time.time() - t0))
    except Exception as e:  # the collective reports the missing peer
        out.put((type(e).__name__, time.time() - t0))


def test_a_failed_rank_is_detected_at_the_next_collective():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 31500 + os.getpid() % 2000
    procs = [ctx.Process(target=_failing_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    kind, secs = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert procs[1].exitcode == 3
    assert kind != "no error" and secs < 60


def _shard_rank(rank, ws, port, out):
    """Rank r simulates global lanes lane_shard(total, r, ws) of one run on the
    oracle (lane_base = its first lane); rank 0 sums the ranks' per-cycle
    hashes, the host-side gather the multi-GPU bench does."""
    import numpy as np

    from oracle import binding as ob
    from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        d, meta = gate_netlist(n_gates=800, n_ff=40, n_pi=10, n_po=10, depth=8, seed=71)
        od = ob.OracleDesign(d.to_json(), meta.top)
        stim, rec = netlist_run_spec(meta)
        si = [(od.signal(n), k, p) for n, k, p in stim]
        ri = [od.signal(r) for r in rec]
        total, cycles = 384, 12
        first, last = bench.lane_shard(total, rank, ws, align=32)
        h = np.zeros(cycles, dtype=np.uint64)
        ob.BitParallel(od, last - first).run(ob.make_run(cycles, 3, si, ri, 2, out_hash=h, lane_base=first))
        got = bench.sum_hashes(dist, h)
        if rank == 0:
            full = np.zeros(cycles, dtype=np.uint64)
            ob.BitParallel(od, total).run(ob.make_run(cycles, 3, si, ri, 2, out_hash=full))
            out.put((first, last, bool(np.array_equal(got, full)), bool(full.any())))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_compose_into_one_run(oracle_lib):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 33500 + os.getpid() % 2000
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    first, last, equal, nonzero = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert (first, last) == (0, 192)
    assert equal and nonzero
