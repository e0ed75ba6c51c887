"""Lat-lon interpolation tables of the grid-table builder against the
reference's own generator.

The reference computes, for every point of its regular lat-lon output grid,
the five nearest cells and inverse-distance weights by scanning every cell
(grid_generator/src/interpolate_ll.c:16-85, selection by
index_helpers.c:find_min_index_exclude).  The table builder reaches the same
five cells through a bucketed search; here both run on the same cell
coordinates and must give identical indices and bit-identical weights.
"""
import ctypes

import numpy as np
import pytest

import refbind
from game_archived_gb300 import tables
from helpers import grid_tables

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference sources not present")


@pytest.mark.parametrize("res,mountain", [(3, False), (4, True), (5, False)])
def test_latlon_tables_equal_reference(res, mountain):
    from oracle import build_ref
    tab = grid_tables(res, mountain, 200, 26)
    lib = ctypes.CDLL(build_ref.build(res, 0))
    n_ll = (4 << res) * (2 << res)
    idx = np.zeros(5 * n_ll, dtype=np.int32)
    w = np.zeros(5 * n_ll)
    lat = np.ascontiguousarray(tab["latitude_scalar"])
    lon = np.ascontiguousarray(tab["longitude_scalar"])
    dp = ctypes.POINTER(ctypes.c_double)
    lib.interpolate_ll(lat.ctypes.data_as(dp), lon.ctypes.data_as(dp),
                       idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), w.ctypes.data_as(dp))
    assert np.array_equal(tab["latlon_interpol_indices"], idx)
    assert np.array_equal(tab["latlon_interpol_weights"], w)


def test_latlon_tables_shape_and_normalisation():
    tab = tables.GridTables(3, n_lloyd=50)
    n_ll = (4 << 3) * (2 << 3)
    idx = tab["latlon_interpol_indices"].reshape(n_ll, 5)
    w = tab["latlon_interpol_weights"].reshape(n_ll, 5)
    assert idx.min() >= 0 and idx.max() < tab.nc
    assert np.allclose(w.sum(axis=1), 1.0, rtol=0, atol=1e-14)
    assert np.all(w > 0)
