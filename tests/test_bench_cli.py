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
