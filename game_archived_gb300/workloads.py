"""The five benchmark configurations of the RKHEVI step, and their inputs on
disk.

Each configuration names a grid (RES_ID, 26 layers, flat or with the 2 km
Gaussian mountain), a build (dry or moist), an initial state recipe of
cases.py, a time step and a step count.  ``prepare`` writes what a
configuration's processes read: the grid tables (tables.py file format,
2000 Lloyd iterations up to RES_ID 6 and 500 at RES_ID 7, the reference
generator's defaults) and the struct layout of the build (JSON), into
``input_dir()``.  ``load`` rebuilds the host structs from those files with
numpy alone -- no native library -- and fills the initial state with the
operators it is given, so a process that must not load this package's
libraries (the CPU reference timing) reads the same grid as the GPU run.
"""
import json
import os

from . import cases, structs, tables

HERE = os.path.dirname(os.path.abspath(__file__))
MOUNTAIN = (2000.0, 1.5e6, 30.0, 90.0)   # 2 km Gaussian mountain, 1500 km half-width, 30N 90E

# name -> (res_id, moist, case, mountain, dt, steps)
CONFIGS = {
    "config1": (4, 0, "std_wind", False, 400.0, 10),
    "config2": (5, 0, "std_wind_tpert", True, 200.0, 72),
    "config3": (6, 1, "baroclinic_moist", False, 100.0, 864),
    "config4": (5, 0, "std_wind_tpert", True, 200.0, 12),
    "config5": (7, 1, "tracers", True, 50.0, 1728),
}
N_LAYERS = 26


def input_dir():
    return os.environ.get("GAME_INPUT_DIR", os.path.join(HERE, "_inputs"))


def n_lloyd_default(res_id):
    return 2000 if res_id <= 6 else 500


def _table_kw(res_id, mountain, n_lloyd):
    return dict(n_layers=N_LAYERS, n_lloyd=n_lloyd if n_lloyd is not None else n_lloyd_default(res_id),
                mountain=MOUNTAIN if mountain else None)


def _layout_path(res_id, moist):
    return os.path.join(input_dir(), f"layout_R{res_id}_L{N_LAYERS}_M{moist}.json")


def prepare(name, n_lloyd=None):
    """builds (or finds) the tables and the layout of a configuration; uses
    the native table library"""
    res, moist, _, mountain, _, _ = CONFIGS[name]
    tab = tables.cached(input_dir(), res, **_table_kw(res, mountain, n_lloyd))
    path = _layout_path(res, moist)
    if not os.path.exists(path):
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(structs.Layout(res, N_LAYERS, moist).to_dict(), f)
        os.replace(tmp, path)
    return tab


def available(name, n_lloyd=None):
    res, moist, _, mountain, _, _ = CONFIGS[name]
    kw = _table_kw(res, mountain, n_lloyd)
    return (os.path.exists(os.path.join(input_dir(), tables.table_file_name(res, **kw)))
            and os.path.exists(_layout_path(res, moist)))


def load(name, n_lloyd=None, buffers=None):
    """(tables, model) of a prepared configuration, read with numpy only; the
    model's grid and config are filled, its state is not (see initial_state)"""
    res, moist, _, mountain, _, _ = CONFIGS[name]
    kw = _table_kw(res, mountain, n_lloyd)
    tab = tables.GridTables.load(os.path.join(input_dir(), tables.table_file_name(res, **kw)))
    with open(_layout_path(res, moist)) as f:
        lay = structs.Layout.from_dict(json.load(f))
    m = structs.Model(lay, buffers)
    tables.fill_grid(tab, m.grid, m.dualgrid)
    cases.default_config(m)
    return tab, m


def initial_state(name, tab, model, ops):
    """fills the configuration's initial state with the operators of ops"""
    case = CONFIGS[name][2]
    cases.build_initial_state(model, tab, case, ops)
    return model
