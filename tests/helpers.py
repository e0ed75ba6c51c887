"""Shared test set-up: grids, initial states and comparisons.

Initial states are built with the oracle's operators (tests may use the
oracle); the GPU library is then compared with the oracle on identical inputs.
"""
import functools

import numpy as np

from game_archived_gb300 import cases, structs, tables
from oracle.bind import Oracle

MOUNTAIN = (2000.0, 1.5e6, 30.0, 90.0)   # 2 km Gaussian mountain, 1500 km half-width, 30N 90E
FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


@functools.lru_cache(maxsize=8)
def grid_tables(res, mountain=False, n_lloyd=200, n_layers=26):
    return tables.GridTables(res, n_layers=n_layers, n_lloyd=n_lloyd, mountain=MOUNTAIN if mountain else None)


def make_model(res, moist, case, mountain=False, n_lloyd=200, n_layers=26):
    tab = grid_tables(res, mountain, n_lloyd, n_layers)
    lay = structs.Layout(res, n_layers, moist)
    m = structs.Model(lay)
    tables.fill_grid(tab, m.grid, m.dualgrid)
    cases.default_config(m)
    cases.build_initial_state(m, tab, case, Oracle(m))
    return tab, m


def clone(model, buffers=None):
    m2 = structs.Model(model.layout, buffers)
    for k in structs.Model.KINDS:
        getattr(m2, k).copy_from(getattr(model, k))
    return m2


def rel_err(a, b):
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / scale)


def state_errors(s_a, s_b, lay):
    """norm-relative error max|a-b| / max|b| per prognostic field; the wind's
    vertical and horizontal parts and each constituent separately"""
    out = {}
    ns = lay.n_scalars
    for k in range(lay.n_const):
        out[f"rho[{k}]"] = rel_err(s_a["rho"][k * ns:(k + 1) * ns], s_b["rho"][k * ns:(k + 1) * ns])
    for f in ("rhotheta_v", "theta_v_pert", "exner_pert"):
        out[f] = rel_err(s_a[f], s_b[f])
    w_a, w_b = wind_parts(s_a["wind"], lay), wind_parts(s_b["wind"], lay)
    out["wind_h"] = rel_err(w_a[1], w_b[1])
    out["wind_v"] = rel_err(w_a[0], w_b[0])
    return out


def rel_err_pointwise(a, b, floor=1e-6):
    """max |a - b| / |b| over the entries with |b| >= floor * max |b|"""
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a - b)))
    mask = np.abs(b) >= floor * scale
    return float(np.max(np.abs(a[mask] - b[mask]) / np.abs(b[mask])))


def state_errors_pointwise(s_a, s_b, lay, floor=1e-6):
    """rel_err_pointwise per prognostic field, split as state_errors"""
    out = {}
    ns = lay.n_scalars
    for k in range(lay.n_const):
        out[f"rho[{k}]"] = rel_err_pointwise(s_a["rho"][k * ns:(k + 1) * ns], s_b["rho"][k * ns:(k + 1) * ns], floor)
    for f in ("rhotheta_v", "theta_v_pert", "exner_pert"):
        out[f] = rel_err_pointwise(s_a[f], s_b[f], floor)
    w_a, w_b = wind_parts(s_a["wind"], lay), wind_parts(s_b["wind"], lay)
    out["wind_h"] = rel_err_pointwise(w_a[1], w_b[1], floor)
    out["wind_v"] = rel_err_pointwise(w_a[0], w_b[0], floor)
    return out


def wind_parts(wind, lay):
    nc, ne, vpl = lay.nc, lay.ne, lay.vpl
    w = np.stack([wind[k * vpl:k * vpl + nc] for k in range(lay.nl + 1)])
    u = np.stack([wind[k * vpl + nc:(k + 1) * vpl] for k in range(lay.nl)])
    return w, u


def output_scenario(res, moist, case, mountain=False, steps=2, dt=300.0, gust_scheme=False, seed=11):
    """A model after a few oracle steps, prepared for the output diagnostics:
    seeded cloud condensates and rain/snow (so that cloud cover and
    precipitation rates take values on both sides of their thresholds), a
    seeded short-wave flux, and the lowest-layer winds of the last n output
    steps as the reference's driver collects them (src/coordinator.c:350-358).
    gust_scheme: the boundary-layer switch on and Monin-Obukhov lengths,
    roughness velocities and v_squared set, so that the gust diagnostics take
    their turbulence branch.  Returns (model, wind_lowest, n_wind_steps)."""
    from game_archived_gb300 import driver
    _, m = make_model(res, moist, case, mountain)
    orc = Oracle(m)
    driver.run(m, steps, dt, orc.linear_combine_two_states, orc.manage_rkhevi)
    lay = m.layout
    rng = np.random.default_rng(seed)
    ns, nc, ne = lay.n_scalars, lay.nc, lay.ne
    s = m.state_new
    if lay.n_cond == 4:
        s["rho"][0:ns] = 2e-6 * rng.random(ns) ** 2
        s["rho"][ns:2 * ns] = 2e-6 * rng.random(ns) ** 2
        cloudy = np.tile(rng.random(nc) < 0.6, lay.nl)
        s["rho"][2 * ns:3 * ns] = 1e-5 * rng.random(ns) ** 3 * cloudy
        s["rho"][3 * ns:4 * ns] = 1e-5 * rng.random(ns) ** 3 * cloudy
    m.forcings["sfc_sw_in"][:] = 400.0 * rng.random(nc)
    n_wind = 3
    lo = lay.n_vectors - lay.vpl  # the lowest layer's horizontal wind (coordinator.c:356)
    wind_lowest = np.concatenate([s["wind"][lo:lo + ne] * (1.0 + 0.1 * rng.standard_normal(ne))
                                  for _ in range(n_wind)])
    if gust_scheme:
        m.config["pbl_scheme"][0] = 1
        m.diagnostics["monin_obukhov_length"][:] = rng.choice([-1.0, 1.0], nc) * (10.0 + 500.0 * rng.random(nc))
        m.diagnostics["monin_obukhov_length"][:5] = 0.0
        m.diagnostics["roughness_velocity"][:] = 0.5 * rng.random(nc)
        m.diagnostics["v_squared"][:] = 400.0 * rng.random(ns)
    return m, wind_lowest, n_wind
