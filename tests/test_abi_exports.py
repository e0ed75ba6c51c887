"""The C-ABI library loads and exports every function include/game_gb300.h
declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "game_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|long long|const char \*)\s+\**(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for n in ("manage_rkhevi", "grad", "divv_h", "divv_h_tracer", "calc_pot_vort", "vorticity_flux", "inner_product",
              "scalar_times_vector", "linear_combine_two_states", "game_gpu_init", "interpolate_to_ll",
              "epv_diagnostics", "edges_to_cells_lowest_layer", "calc_uv_at_edge", "curl_field_to_cells",
              "edges_to_cells", "game_gpu_write_out_fields"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from game_archived_gb300 import build
    if not os.path.exists(build.GPU_LIB):
        pytest.skip("libgame_gb300.so not built")
    lib = ctypes.CDLL(build.GPU_LIB)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_the_header():
    from game_archived_gb300 import abi
    missing = [n for n in declared_functions() if n not in abi.SIGNATURES]
    assert not missing, missing
