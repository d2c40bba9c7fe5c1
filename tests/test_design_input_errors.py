"""Malformed design JSON is rejected through the C ABI with an error code and
message (RrtlError in Python), never a crash: truncations, byte edits,
spliced text and out-of-range numbers in otherwise well-formed designs, fed
to the host-only entry points (bit-slice lowering, instance-fold analysis,
compiled word kernel emission)."""
import json
import random

import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import counter, narrow_alu, replicated_datapath


def _mutants(seed, n):
    rng = random.Random(seed)
    designs = [(counter().to_json(), "Counter"), (narrow_alu(8).to_json(), "Alu"),
               (replicated_datapath(2).to_json(), "Top")]
    for _ in range(n):
        js, top = rng.choice(designs)
        k = rng.randrange(4)
        if k == 0:
            m = js[: rng.randrange(len(js))]
        elif k == 1:
            i = rng.randrange(len(js))
            m = js[:i] + rng.choice('{}[],:"0x-1e9 tnf') + js[i + 1:]
        elif k == 2:
            i, j = rng.randrange(len(js)), rng.randrange(len(js))
            m = js[:i] + js[j:]
        else:
            obj = json.loads(js)

            def walk(o):
                items = o.items() if isinstance(o, dict) else enumerate(o) if isinstance(o, list) else ()
                for key, v in list(items):
                    if isinstance(v, int) and not isinstance(v, bool) and rng.random() < 0.05:
                        o[key] = rng.choice([0, -1, 2**40, 65, 1 << 20, 3])
                    else:
                        walk(v)

            walk(obj)
            m = json.dumps(obj)
        yield m, top


ENTRY_POINTS = {
    "bitslice_json": lambda j, t: sim.bitslice_json(j, t),
    "instance_fold_plan": lambda j, t: sim.instance_fold_plan(j, t),
    "word_jit_emit": lambda j, t: sim.word_jit_emit(j, t),
}


@pytest.mark.parametrize("entry", sorted(ENTRY_POINTS))
def test_mutated_designs_fail_with_an_error_code(entry):
    f = ENTRY_POINTS[entry]
    rejected = 0
    for m, top in _mutants(sorted(ENTRY_POINTS).index(entry) + 7, 150):
        try:
            f(m, top)
        except sim.RrtlError as e:
            assert str(e), "an error without a message"
            rejected += 1
    assert rejected > 100


@pytest.mark.parametrize("entry", sorted(ENTRY_POINTS))
def test_unknown_top_and_empty_input(entry):
    f = ENTRY_POINTS[entry]
    for js, top in (("", "Counter"), ("{}", "Counter"), ('{"modules": []}', "Counter"),
                    (counter().to_json(), "NoSuchModule")):
        with pytest.raises(sim.RrtlError):
            f(js, top)
