"""Mixed-precision step against the FP64 step over 24 hours.

RES_ID=6 (40962 cells), 26 layers, moist barotropic jet with relative
humidity 0.7 below 8 km, dt = 100 s, 864 steps.  Both runs start from the
same state and stay on the device (resident mode, CUDA graphs); at the end
the surface pressure of every column (write_output.c:105-121) must agree to
within 0.1 Pa, and the dry-air mass (compensated global integral) to within
1e-12 relative: the mixed path keeps the mass-flux divergence and the
vertical solves in FP64, so it conserves mass like the FP64 path.  The FP64
path itself follows the oracle to 1e-12 per step (test_gpu_step.py).
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, cases, driver, structs, tables
from game_archived_gb300.ops import CAbiOps
from helpers import state_errors

pytestmark = pytest.mark.gpu

RES, DT, STEPS = 6, 100.0, 864
SFC_TOL_PA = 0.1


def _initial_model():
    tab = tables.GridTables(RES, n_lloyd=200)
    m = structs.Model(structs.Layout(RES, 26, 1))
    tables.fill_grid(tab, m.grid, m.dualgrid)
    cases.default_config(m)
    g = abi.GpuModel(m, abi.FP64)
    try:
        cases.build_initial_state(m, tab, "jet_moist", CAbiOps(g.lib, m))
    finally:
        g.close()
    return m


SNAPSHOTS = (1, 72, STEPS)


def _run(m0, precision):
    m = structs.Model(m0.layout)
    for k in structs.Model.KINDS:
        getattr(m, k).copy_from(getattr(m0, k))
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
    return ps, mass0, mass, finite, snaps


def test_mixed_surface_pressure_within_0p1_pa_after_24h():
    m0 = _initial_model()
    ps64, mass0_64, mass64, ok64, sn64 = _run(m0, abi.FP64)
    ps32, mass0_32, mass32, ok32, sn32 = _run(m0, abi.MIXED)
    assert ok64 and ok32
    # per-field error of the mixed path against the FP64 path (max |diff| / max |fp64|)
    for n in SNAPSHOTS:
        e = state_errors(sn32[n], sn64[n], m0.layout)
        print(f"mixed vs FP64 after {n} steps: " + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
        assert max(e.values()) < 1e-2, (n, e)
    err = np.abs(ps32 - ps64)
    print(f"24 h surface pressure: max |mixed - fp64| = {err.max():.4g} Pa, rms {np.sqrt(np.mean(err ** 2)):.4g} Pa, "
          f"p_sfc range {ps64.min():.1f}..{ps64.max():.1f} Pa")
    # gas phase = rho[n_cond], water vapour = rho[n_cond + 1]: dry air is their difference
    cond = m0.layout.n_cond
    dry64, dry32, dry0 = (x[cond] - x[cond + 1] for x in (mass64, mass32, mass0_64))
    print(f"dry-air mass drift over 24 h: fp64 {dry64 / dry0 - 1:.3g}, mixed {dry32 / dry0 - 1:.3g}")
    assert err.max() < SFC_TOL_PA
    assert abs(dry32 / dry64 - 1) < 1e-12
