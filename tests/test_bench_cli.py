"""The benchmark entry point parses its arguments and its CPU-only pieces
run without a GPU (the timed legs need one)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_help_lists_every_leg_switch():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       cwd=ROOT, timeout=300)
    assert p.returncode == 0, p.stderr
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--word-only", "--crc32-only", "--fold-only", "--jobs",
                 "--serve-rates", "--serve-round-us", "--no-cpu-baseline"):
        assert flag in p.stdout, flag


def test_net_streaming_byte_model_of_the_headline_netlist():
    """The roofline's algorithmic bytes per lane-cycle: 4 B per 32 lanes for
    every gate's fanin reads and output write, each flop's D read and Q write,
    and the inputs and outputs (about 19.3 KB per lane-cycle at 50k gates)."""
    sys.path.insert(0, ROOT)
    import bench

    d, meta, js, stim, rec = bench.build_workload()
    bpl = bench.net_stream_bytes_per_lane_cycle(bench.gate_fanins(js), bench.FFS, bench.PIS, bench.POS)
    assert 19_000 < bpl < 19_600
    json.dumps({"bytes_per_lane_cycle": bpl})


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` times the CPU restatement of the path on
    the host (no GPU) and prints one JSON line with the arm's keys."""
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference" and r["unit"] == "lane-cycles/s" and r["higher_is_better"] is True
    assert r["steps"] == 1 and r["warmup"] == 3 and r["n_gpus"] == 1
    assert r["value"] > 0 and r["cpu_baseline"]["value"] == r["value"]
    assert r["cpu_baseline"]["kind"] in ("port", "reference") and r["cpu_baseline"]["cores"] >= 1
    assert r["e2e"] == {"value": r["value"], "unit": r["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in r["config"]


def test_reference_arm_under_two_ranks_prints_from_rank_zero_only():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    p = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference" and r["n_gpus"] == 2 and r["value"] > 0
