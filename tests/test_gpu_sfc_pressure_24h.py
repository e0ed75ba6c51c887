"""The mixed-precision step over 24 hours against the FP64 step and against
the oracle's own FP64 run.

RES_ID=6 (40962 cells), 26 layers, moist build, the baroclinic jet of
Jablonowski and Williamson (2006) with its thermal-wind-balanced temperature
(cases.baroclinic_moist), relative humidity 0.7 below 8 km, N(0, 0.5 m/s)
wind noise, dt = 100 s, 864 steps.  All three runs start from the same state;
the GPU runs stay on the device (resident mode, CUDA graphs), the oracle runs
on the host cores (about 6 minutes on 16 cores).

* At the end the surface pressure of every column (write_output.c:105-121)
  of the mixed run must be within 0.1 Pa of the FP64 GPU run and of the
  oracle; the FP64 GPU run must be within 0.1 Pa of the oracle as well.
  The per-field errors after 1, 72 and 864 steps are printed, both
  norm-relative (max |diff| / max |ref|) and pointwise.
* The dry-air mass (compensated global integral) of the mixed run must stay
  within 1e-12 of the FP64 run: the mixed path keeps the mass-flux
  divergence in double-word accumulation and the density update in flux
  form, so it conserves mass like the FP64 path.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, cases, driver, structs, tables
from game_archived_gb300.ops import CAbiOps
from helpers import state_errors, state_errors_pointwise
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

RES, DT, STEPS = 6, 100.0, 864
CASE = "baroclinic_moist"
SFC_TOL_PA = 0.1
SNAPSHOTS = (1, 72, STEPS)


def _initial_model():
    tab = tables.GridTables(RES, n_lloyd=200)
    m = structs.Model(structs.Layout(RES, 26, 1))
    tables.fill_grid(tab, m.grid, m.dualgrid)
    cases.default_config(m)
    g = abi.GpuModel(m, abi.FP64)
    try:
        cases.build_initial_state(m, tab, CASE, CAbiOps(g.lib, m))
    finally:
        g.close()
    return m


def _copy(m0):
    m = structs.Model(m0.layout)
    for k in structs.Model.KINDS:
        getattr(m, k).copy_from(getattr(m0, k))
    return m


def _run_gpu(m0, precision):
    m = _copy(m0)
    g = abi.GpuModel(m, precision, resident=True, graphs=True)
    snaps = {}

    def snapshot(i, model):
        if i + 1 in SNAPSHOTS:
            g.sync_to_host(model.state_new)
            snaps[i + 1] = model.state_new.clone()

    try:
        for s in (m.state_old, m.state_new, m.state_tendency):
            g.sync_to_device(s)
        mass0 = g.write_out_integral(m.state_old, 0)
        driver.run(m, STEPS, DT, g.linear_combine_two_states, g.manage_rkhevi, callback=snapshot)
        g.synchronize()
        ps = g.surface_pressure(m.state_new)
        mass = g.write_out_integral(m.state_new, 0)
        g.sync_to_host(m.state_new)
        finite = bool(np.isfinite(m.state_new["rho"]).all() and np.isfinite(m.state_new["wind"]).all())
    finally:
        g.close()
    return {"ps": ps, "mass0": mass0, "mass": mass, "finite": finite, "snaps": snaps}


def _run_oracle(m0):
    m = _copy(m0)
    orc = Oracle(m)
    snaps = {}

    def snapshot(i, model):
        if i + 1 in SNAPSHOTS:
            snaps[i + 1] = model.state_new.clone()

    driver.run(m, STEPS, DT, orc.linear_combine_two_states, orc.manage_rkhevi, callback=snapshot)
    ps = orc.surface_pressure(m.state_new, orc.temperature(m.state_new))
    return {"ps": ps, "snaps": snaps}


@pytest.fixture(scope="module")
def runs():
    m0 = _initial_model()
    return m0, _run_gpu(m0, abi.FP64), _run_gpu(m0, abi.MIXED), _run_oracle(m0)


def _report(label, a, b, lay):
    for n in SNAPSHOTS:
        e = state_errors(a["snaps"][n], b["snaps"][n], lay)
        pw = state_errors_pointwise(a["snaps"][n], b["snaps"][n], lay)
        print(f"{label} after {n} steps: norm " + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
        print(f"{label} after {n} steps: pointwise " + ", ".join(f"{k} {v:.2e}" for k, v in pw.items()))
    err = np.abs(a["ps"] - b["ps"])
    print(f"{label}: 24 h surface pressure max |diff| = {err.max():.4g} Pa, rms {np.sqrt(np.mean(err ** 2)):.4g} Pa, "
          f"p_sfc range {b['ps'].min():.1f}..{b['ps'].max():.1f} Pa")
    return err


def test_mixed_surface_pressure_within_0p1_pa_of_fp64_after_24h(runs):
    m0, r64, r32, _ = runs
    assert r64["finite"] and r32["finite"]
    for n in SNAPSHOTS:
        e = state_errors(r32["snaps"][n], r64["snaps"][n], m0.layout)
        assert max(e.values()) < 1e-2, (n, e)
    err = _report("mixed vs FP64 GPU", r32, r64, m0.layout)
    # gas phase = rho[n_cond], water vapour = rho[n_cond + 1]: dry air is their difference
    cond = m0.layout.n_cond
    dry64, dry32, dry0 = (x[cond] - x[cond + 1] for x in (r64["mass"], r32["mass"], r64["mass0"]))
    print(f"dry-air mass drift over 24 h: fp64 {dry64 / dry0 - 1:.3g}, mixed {dry32 / dry0 - 1:.3g}")
    assert err.max() < SFC_TOL_PA
    assert abs(dry32 / dry64 - 1) < 1e-12


def test_surface_pressure_within_0p1_pa_of_the_oracle_after_24h(runs):
    """the target as stated: the mixed run against the FP64 oracle (the
    reference's algorithm on the host) after 24 h; the FP64 GPU run too"""
    m0, r64, r32, ro = runs
    err32 = _report("mixed vs oracle", r32, ro, m0.layout)
    err64 = _report("FP64 GPU vs oracle", r64, ro, m0.layout)
    assert err32.max() < SFC_TOL_PA, err32.max()
    assert err64.max() < SFC_TOL_PA, err64.max()
