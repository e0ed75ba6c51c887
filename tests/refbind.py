"""Binding of the reference's own C build in oracle/_ref (this container only)."""
import ctypes
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402


def available():
    return build_ref.available()


class Reference:
    """The reference library for one (RES_ID, MOISTURE_ON), driven on a Model."""

    def __init__(self, model):
        lay = model.layout
        self.lib = ctypes.CDLL(build_ref.build(lay.res_id, lay.moisture_on, lay.n_layers))
        vp, dbl = ctypes.c_void_p, ctypes.c_double
        self.lib.manage_rkhevi.argtypes = [vp] * 9 + [dbl, dbl]
        self.lib.linear_combine_two_states.argtypes = [vp, vp, vp, dbl, dbl, vp]
        self.lib.ref_offsetof.restype = ctypes.c_long
        self.lib.ref_offsetof.argtypes = [ctypes.c_int, ctypes.c_char_p]
        self.lib.ref_sizeof.restype = ctypes.c_long
        self.lib.global_scalar_integrator = None
        self.m = model

    def manage_rkhevi(self, dt, t=0.0):
        m = self.m
        rc = self.lib.manage_rkhevi(m.state_old.ptr, m.state_new.ptr, m.grid.ptr, m.dualgrid.ptr,
                                    m.state_tendency.ptr, m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr,
                                    m.config.ptr, dt, t)
        assert rc == 0

    def linear_combine_two_states(self, s0, s1, out, c0, c1):
        self.lib.linear_combine_two_states(s0.ptr, s1.ptr, out.ptr, c0, c1, self.m.grid.ptr)


from game_archived_gb300.structs import ConfigIo  # noqa: E402


def write_out(ref, state, wind_lowest, n_wind_steps, workdir, t_init=0.0, t_write=3600.0):
    """Runs the reference's write_out (src/io/write_output.c:51) with every
    output switch on, in workdir (it opens its GRIB template at
    ../../src/io/grib_template.grb2 relative to the working directory), and
    returns what it handed to the netCDF and GRIB writers, recorded by the
    harness's stand-ins: {"surface": {var: array}, "pressure_levels": {...},
    "model_levels": {...}, "grib_surface": [arrays in message order],
    "grib_pressure_levels": [...], "grib_model_levels": [...]}."""
    lib = ref.lib
    m = ref.m
    cio = ConfigIo(1, 1, 1, 1, 1, 3600, 0, 2000, 1, 1, 0, b"ref", b"01", b"01", b"00", 0)
    tmpl = os.path.join(workdir, "src", "io")
    os.makedirs(tmpl, exist_ok=True)
    open(os.path.join(tmpl, "grib_template.grb2"), "wb").close()
    run_dir = os.path.join(workdir, "a", "b")
    os.makedirs(run_dir, exist_ok=True)
    vp, dbl = ctypes.c_void_p, ctypes.c_double
    lib.write_out.argtypes = [vp, vp, ctypes.c_int, dbl, dbl, vp, vp, vp, vp, vp, vp, vp]
    lib.ref_io_record.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_char_p),
                                  ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long),
                                  ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    import numpy as np
    wl = np.ascontiguousarray(wind_lowest, dtype=np.float64)
    lib.ref_io_reset()
    lib.ref_nc_def_reset()
    cwd = os.getcwd()
    os.chdir(run_dir)
    # one thread: the reference's gust loop shares a work array between
    # threads (write_output.c:298, vector_to_minimize is not private)
    n_threads = lib.ref_get_max_threads()
    lib.ref_set_num_threads(1)
    try:
        rc = lib.write_out(state.ptr, wl.ctypes.data, n_wind_steps, t_init, t_write, m.diagnostics.ptr,
                           m.forcings.ptr, m.grid.ptr, m.dualgrid.ptr, ctypes.byref(cio), m.config.ptr, m.irrev.ptr)
    finally:
        os.chdir(cwd)
        lib.ref_set_num_threads(n_threads)
    assert rc == 0
    out = {"surface": {}, "pressure_levels": {}, "model_levels": {}, "grib_surface": [], "grib_pressure_levels": [],
           "grib_model_levels": []}
    f, nm = ctypes.c_char_p(), ctypes.c_char_p()
    meta = (ctypes.c_long * 4)()
    n = ctypes.c_long()
    data = ctypes.POINTER(ctypes.c_double)()
    for k in range(lib.ref_io_count()):
        lib.ref_io_record(k, ctypes.byref(f), ctypes.byref(nm), meta, ctypes.byref(n), ctypes.byref(data))
        arr = np.ctypeslib.as_array(data, shape=(n.value,)).copy()
        fname, vname = f.value.decode(), nm.value.decode()
        if fname.endswith("_surface.nc"):
            out["surface"][vname] = arr
        elif fname.endswith("_pressure_levels.nc"):
            out["pressure_levels"][vname] = arr
        elif fname.endswith(".nc"):
            out["model_levels"][vname] = arr
        elif fname.endswith("_surface.grb2"):
            out["grib_surface"].append(arr)
        elif fname.endswith("_pressure_levels.grb2"):
            out["grib_pressure_levels"].append(arr)
        else:
            out["grib_model_levels"].append(arr)
    lib.ref_io_reset()
    # the netCDF file structure: (file kind, 'D' or 'V', name, dimension
    # names, units, length) in definition order
    lib.ref_nc_def_get.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_char),
                                   ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_char_p),
                                   ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong)]
    kind, dims, units, ln = ctypes.c_char(), ctypes.c_char_p(), ctypes.c_char_p(), ctypes.c_longlong()
    out["defs"] = []
    for k in range(lib.ref_nc_def_count()):
        lib.ref_nc_def_get(k, ctypes.byref(f), ctypes.byref(kind), ctypes.byref(nm), ctypes.byref(dims),
                           ctypes.byref(units), ctypes.byref(ln))
        fname = f.value.decode()
        fk = "surface" if fname.endswith("_surface.nc") else \
            "pressure_levels" if fname.endswith("_pressure_levels.nc") else "model_levels"
        out["defs"].append((fk, kind.value.decode(), nm.value.decode(), dims.value.decode(), units.value.decode(),
                            ln.value))
    lib.ref_nc_def_reset()
    return out


def run_gridgen(res_id, n_iterations, workdir, n_layers=26, stretching=1.3, n_oro_layers=23, toa=41152.0,
                radius_rescale=1.0):
    """Runs the reference's grid generator program (grid_generator/src/
    coordinator.c main, flat orography) in-process in workdir and returns the
    tables it writes to its grid file, recorded by the netCDF stand-in:
    {variable name: array} (integer tables as float arrays)."""
    import numpy as np
    lib = ctypes.CDLL(build_ref.build_gridgen(res_id, n_layers))
    os.makedirs(os.path.join(workdir, "statistics"), exist_ok=True)
    os.makedirs(os.path.join(workdir, "grids"), exist_ok=True)
    args = [b"grid_generator", b"0", str(n_iterations).encode(), b"0", b"none", repr(stretching).encode(),
            str(n_oro_layers).encode(), repr(toa).encode(), repr(radius_rescale).encode(), b"7"]
    argv = (ctypes.c_char_p * len(args))(*args)
    lib.ref_run_gridgen.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
    lib.ref_io_record.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_char_p),
                                  ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long),
                                  ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    lib.ref_io_reset()
    cwd = os.getcwd()
    try:
        rc = lib.ref_run_gridgen(workdir.encode(), len(args), argv)
    finally:
        os.chdir(cwd)
    assert rc == 0
    out = {}
    f, nm = ctypes.c_char_p(), ctypes.c_char_p()
    meta = (ctypes.c_long * 4)()
    n = ctypes.c_long()
    data = ctypes.POINTER(ctypes.c_double)()
    for k in range(lib.ref_io_count()):
        lib.ref_io_record(k, ctypes.byref(f), ctypes.byref(nm), meta, ctypes.byref(n), ctypes.byref(data))
        out[nm.value.decode()] = np.ctypeslib.as_array(data, shape=(n.value,)).copy()
    lib.ref_io_reset()
    return out
