"""Test helpers: the library's netCDF writers of write_out's files
(csrc/common/ncwrite.c, built into libgame_tables.so as well), called from
host arrays, and a reader of the resulting files' structure and data."""
import ctypes

import numpy as np

from game_archived_gb300 import native

DP = ctypes.POINTER(ctypes.c_double)
PRESSURE_LEVELS = np.array([20000.0, 30000.0, 50000.0, 70000.0, 85000.0, 92500.0])
POINTERS = ("mslp", "surface_p", "t2", "tcdc", "rprate", "sprate", "cape", "sfc_sw_down", "u10", "v10", "gusts",
            "pressure_levels", "geopotential_height", "t_pl", "rh_pl", "epv_pl", "u_pl", "v_pl", "rel_vort_pl",
            "densities", "temperature", "wind", "rh", "rel_vort", "divv_h", "tke", "t_soil")


class NcwOutput(ctypes.Structure):
    _fields_ = [(n, ctypes.c_longlong) for n in ("n_cells", "n_scalars", "n_vectors", "n_densities", "n_h_vectors",
                                                 "n_v_vectors", "n_curl", "n_soil")] + [(n, DP) for n in POINTERS]


def write_files(lay, fields, directory, stem):
    """writes <stem>_surface.nc, <stem>_pressure_levels.nc, <stem>.nc from a
    dict of reference-order arrays named as POINTERS; returns the paths"""
    lib = native.tables()
    keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in fields.items()}
    keep["pressure_levels"] = PRESSURE_LEVELS
    o = NcwOutput(lay.nc, lay.n_scalars, lay.n_vectors, lay.n_const * lay.n_scalars, lay.nl * lay.ne,
                  (lay.nl + 1) * lay.nc, lay.n_curl, len(fields["t_soil"]),
                  *[keep[k].ctypes.data_as(DP) for k in POINTERS])
    paths = {}
    for kind, fn, suffix in (("surface", lib.ncw_write_surface, "_surface.nc"),
                             ("pressure_levels", lib.ncw_write_pressure_levels, "_pressure_levels.nc"),
                             ("model_levels", lib.ncw_write_model_levels, ".nc")):
        path = f"{directory}/{stem}{suffix}"
        fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(NcwOutput)]
        assert fn(path.encode(), ctypes.byref(o)) == 0, path
        paths[kind] = path
    return paths


def read_file(path):
    """(definitions as the stand-in records them, {variable: values})"""
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        defs = [("D", n, "", "", f.dimensions[n]) for n in f._dims]
        data = {}
        for n, v in f.variables.items():
            units = v._attributes.get("units", b"")
            units = units.decode() if isinstance(units, bytes) else str(units)
            defs.append(("V", n, ",".join(v.dimensions), units, int(np.prod(v.shape)) if v.shape else 1))
            data[n] = np.array(v.data, dtype=np.float64).reshape(-1)
    return defs, data
