"""Autotune recommendation table lookup (rrtl_autotune_find, no device): the
reference's exact and nearest rules (crates/rrtl-gpu-sim/src/lib.rs:123-189)
and its error codes."""
import json

import pytest

from rrtl_gb300 import sim

TABLE = [
    {"case": "c2", "lanes": 65536, "steps": 1000, "tile_words": 8, "autotune_metric": "kernel_ms",
     "autotune_metric_ns": 78500000},
    {"case": "c2", "lanes": 16384, "steps": 400, "tile_words": 4, "autotune_metric": "kernel_ms",
     "autotune_metric_ns": 12000000},
    {"case": "c2", "lanes": 16384, "steps": 1000, "tile_words": 4, "autotune_metric": "kernel_ms",
     "autotune_metric_ns": None},
    {"case": "crc32", "lanes": 262144, "steps": 2000, "tile_words": 0, "autotune_metric": "kernel_ms",
     "autotune_metric_ns": 670000},
    {"case": "c2", "lanes": 16384, "steps": 1000, "tile_words": 2, "autotune_metric": "kernel_ms",
     "autotune_metric_ns": 5000000},
]


def test_exact_match_takes_the_first_equal_record():
    assert sim.autotune_find(TABLE, "c2", 65536, 1000) == 0
    assert sim.autotune_find(TABLE, "crc32", 262144, 2000) == 3
    # two records with the same key: the first one, as the reference's iter().find
    assert sim.autotune_find(json.dumps(TABLE), "c2", 16384, 1000) == 2


def test_nearest_orders_by_lanes_then_steps_then_metric():
    # lanes 20,000: 16,384 is nearer than 65,536; among those, steps 1,000 (|0|)
    # before 400; between the two 1,000-step records the measured metric wins
    # over an absent one
    assert sim.autotune_find(TABLE, "c2", 20000, 1000, nearest=True) == 4
    assert sim.autotune_find(TABLE, "c2", 20000, 300, nearest=True) == 1
    assert sim.autotune_find(TABLE, "c2", 60000, 10, nearest=True) == 0
    # nearest never crosses cases
    assert sim.autotune_find(TABLE, "crc32", 1, 1, nearest=True) == 3


def test_missing_and_malformed_tables_have_the_reference_codes():
    with pytest.raises(sim.RrtlError) as e:
        sim.autotune_find(TABLE, "c2", 65536, 999)
    assert e.value.code == "E_GPU_AUTOTUNE_RECOMMENDATION" and e.value.status == 1
    with pytest.raises(sim.RrtlError) as e:
        sim.autotune_find(TABLE, "c3", 1, 1, nearest=True)
    assert e.value.code == "E_GPU_AUTOTUNE_RECOMMENDATION"
    for bad in ("{", "{}", json.dumps([{"case": "c2", "lanes": 1}]),
                json.dumps([{"case": "c2", "lanes": 1, "steps": 1, "tile_words": 3}])):
        with pytest.raises(sim.RrtlError) as e:
            sim.autotune_find(bad, "c2", 1, 1)
        assert e.value.code == "E_GPU_AUTOTUNE_JSON" and e.value.status == 1
