"""Failure detection on the device without a fault: the bounded mbarrier wait
that the fused and queue kernels put around their copies gives up on a
barrier that nothing arrives on, reports RRTL_E_TIMEOUT through device
memory, and the context stays usable (a run afterwards is still exact).
Collected last so a failure here comes after every other test."""
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import counter

pytestmark = pytest.mark.gpu

RRTL_E_TIMEOUT = 6


@pytest.mark.parametrize("polls", [1, 16, 256])
def test_wait_on_a_barrier_nothing_arrives_on_times_out(engine, ctx, polls):
    status, completed = ctx.check_wait_timeout(polls)
    assert status == RRTL_E_TIMEOUT
    assert completed


def test_context_is_usable_after_a_timed_out_wait(engine, ctx):
    ctx.check_wait_timeout(256)
    c = sim.GpuBatchSimulator(counter(), "Counter", 4, ctx)
    c.set_input("rst", [1, 0, 0, 0])
    c.set_input("en", [1, 0, 1, 1])
    c.tick()
    c.set_input("rst", [0, 0, 0, 0])
    c.tick()
    assert list(c.get_signal("count")) == [1, 0, 2, 2]


def test_poll_count_is_checked_on_the_host(engine, ctx):
    for bad in (0, (1 << 22) + 1):
        with pytest.raises(sim.RrtlError):
            ctx.check_wait_timeout(bad)
