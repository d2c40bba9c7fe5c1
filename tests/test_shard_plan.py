"""The lane-shard plan (RuntimeShardInfo, crates/rrtl-runtime/src/lib.rs:168-175)
on the CPU: contiguous, covering, each shard starting on a 32-lane word."""
import pytest

from rrtl_gb300 import build, sim


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


@pytest.mark.parametrize("total,n", [(1, 1), (1000, 3), (65536, 8), (33, 2), (4097, 5)])
def test_plan_is_contiguous_covering_and_word_aligned(total, n):
    plan = sim.shard_plan(total, n)
    assert [w for w, _, _ in plan] == list(range(n))
    start = 0
    for _, first, lanes in plan:
        assert first == start and first % 32 == 0
        start += lanes
    assert start == total
    assert all(lanes > 0 for _, _, lanes in plan)


def test_plan_rejects_impossible_splits():
    with pytest.raises(sim.RrtlError):
        sim.shard_plan(0, 1)
    with pytest.raises(sim.RrtlError):
        sim.shard_plan(64, 3)  # three shards need three 32-lane words
