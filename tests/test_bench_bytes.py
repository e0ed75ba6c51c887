"""The byte counts behind bench.py's roofline figures (no GPU needed).

* grid_sizes follows the icosahedral grid of RES_ID r: 10 * 4^r + 2 cells,
  30 * 4^r edges, 20 * 4^r triangles (Euler: cells - edges + triangles = 2);
* b_step, the compulsory bytes of one step (every state, tendency and grid
  array once per substage), is 1 452 322 240 bytes for the moist RES_ID=6,
  26-layer mixed step (FP64 state and tendencies, FP32 grid);
* kernel_bytes has an entry for every kernel of the committed ncu summary of
  that step, under bench.py's mapping of profiled names to scope names, so
  the roofline lookup finds the numerator of each kernel it is asked about;
* each kernel's bytes per launch lie between the smallest array it must
  touch and the whole step's algorithmic traffic.
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("res, cells, edges, triangles", [(5, 10242, 30720, 20480), (6, 40962, 122880, 81920),
                                                         (7, 163842, 491520, 327680)])
def test_grid_sizes(res, cells, edges, triangles):
    g = bench.grid_sizes(res, 26)
    assert (g["nc"], g["ne"], g["nt"]) == (cells, edges, triangles)
    assert g["nc"] - g["ne"] + g["nt"] == 2
    assert g["s"] == 26 * cells
    assert g["vt"] == 26 * edges + 27 * cells          # horizontal + vertical wind points
    assert g["dv"] == 27 * edges + 26 * triangles      # dual vectors


def test_step_bytes_of_the_moist_res6_mixed_step():
    assert bench.b_step(6, 6, 8, 8, 4) == 1452322240
    # FP64 grid tables instead of FP32 only add bytes
    assert bench.b_step(6, 6, 8, 8, 8) > bench.b_step(6, 6, 8, 8, 4)


def _scope_name(profiled):
    for scope, names in bench.NCU_NAMES.items():
        if profiled in names:
            return scope
    return profiled


def test_every_profiled_kernel_has_algorithmic_bytes():
    with open(bench.PROFILE_JSON) as f:
        profiled = json.load(f)["kernels"]
    kb = bench.kernel_bytes(6, 6, 4)
    missing = [k for k in profiled if _scope_name(k) not in kb]
    assert not missing, missing
    # and the lookup by scope name finds each profiled kernel's DRAM bytes
    for k in profiled:
        v, src = bench.read_profile(_scope_name(k), "dram_bytes_per_launch")
        assert v == profiled[k]["dram_bytes_per_launch"] and src["commit"], k


def test_kernel_bytes_are_bounded_by_the_step():
    g = bench.grid_sizes(6, 26)
    kb = bench.kernel_bytes(6, 6, 4)
    step = bench.b_step(6, 6, 8, 8, 4)
    for name, (per_step, launches) in kb.items():
        assert launches in (1, 2), name
        per_launch = per_step / launches
        # at least one FP32 layer field of cells (k_theta reads two, writes one)
        assert per_launch >= g["s"] * 4, name
        assert per_launch < step, name
