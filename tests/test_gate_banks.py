"""Shared-memory layout of the gate lowering (CPU, no device): the slot bank
residues and the commit order keep the fused kernel's operand reads and
register commit near one wavefront per access."""
import pytest

from rrtl_gb300 import sim
from rrtl_gb300.workloads import gate_netlist

from .helpers import crc32_netlist_json


@pytest.fixture(scope="module")
def netlist():
    d, meta = gate_netlist(n_gates=12000, n_ff=512, n_pi=32, n_po=32, depth=16, seed=21)
    return d.to_json(), meta


def test_operand_and_commit_wavefronts_near_the_floor_at_8_words(netlist):
    js, meta = netlist
    info = sim.gate_program_info(js, meta.top, 8)
    assert info["tile_words"] == 8 and info["group"] == 4
    assert info["cells"] >= 12000 and info["levels"] >= 16
    assert info["groups"] * 4 == info["cells"] + info["pad_cells"]
    # balanced residues: within 10% of one wavefront per group and position
    assert info["operand_wavefronts"] <= 1.10 * info["operand_rows"], info
    # commit order: within 10% of one wavefront per group of 4 registers
    assert info["commit_groups"] == (512 + 3) // 4
    assert info["commit_wavefronts"] <= 1.10 * info["commit_groups"], info
    # the generated gate mix canonicalises to a handful of truth-table classes
    assert info["classes"] <= 12


@pytest.mark.parametrize("w,g", [(4, 8), (2, 16), (1, 32)])
def test_narrower_tiles_report_their_groups(netlist, w, g):
    js, meta = netlist
    info = sim.gate_program_info(js, meta.top, w)
    assert info["group"] == g and info["groups"] * g == info["cells"] + info["pad_cells"]
    # never more wavefronts than rows a group reads, never fewer than its floor
    assert info["operand_rows"] <= info["operand_wavefronts"] <= g * info["operand_rows"]


def test_crc32_fixture_layout():
    """A 195-cell netlist leaves the grouping little choice: its operand reads
    still stay within 15% of the floor, its 32-register commit within 2x."""
    info = sim.gate_program_info(crc32_netlist_json().to_json(), "crc32", 8)
    assert info["cells"] == 195 and info["commit_groups"] == 8  # 32 flip-flops
    assert info["operand_wavefronts"] <= 1.15 * info["operand_rows"], info
    assert info["commit_wavefronts"] <= 2 * info["commit_groups"], info


def test_bad_width_and_word_design_are_rejected():
    from rrtl_gb300.workloads import counter

    with pytest.raises(sim.RrtlError) as e:
        sim.gate_program_info(counter(), "Counter", 3)
    assert e.value.status == 1  # RRTL_E_ARG
    with pytest.raises(sim.RrtlError) as e:
        sim.gate_program_info(counter(), "Counter", 8)  # multi-bit signals: the word engine's design
    assert e.value.status == 7  # RRTL_E_UNSUPPORTED
