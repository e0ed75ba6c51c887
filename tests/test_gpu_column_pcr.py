"""Column solvers for any layer count (C ABI) against the oracle.

* FP64 with the default solver (per-thread Thomas sweeps, the reference's
  elimination order; registers at 26 layers, local memory at 40, 80 and 256):
  every prognostic field within 1e-12 relative of the oracle after every
  step, dry over a mountain and moist with falling condensates;
* FP64 with the warp-cooperative parallel cyclic reduction forced
  (game_gpu_set_column_solver(2)) at 26 and 80 layers: within 1e-12 as well.
  At 256 layers the reduction's different elimination order leaves rho*theta_v
  about 1e-14 relative from the oracle, and Pi', a perturbation about 3e-3
  the size of the full Exner pressure it is derived from, carries that
  difference at its own scale (2.3e-12 measured): Pi' is held to 1e-11 there,
  every other field to 1e-12;
* the mixed path with cyclic reduction (its default for batches of fewer
  than 6144 columns at layer counts other than 26) stays as close to FP64 as
  the mixed path with Thomas sweeps does, and the two mixed-path solvers
  agree to rounding;
* the solver switch rejects unknown modes and a 257-layer context is refused.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver
from helpers import clone, make_model, state_errors
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12

CASES = [
    # (res, moist, case, mountain, n_layers, column_solver, dt, steps, tolerance of Pi')
    (3, 0, "std_wind_tpert", True, 26, 2, 300.0, 4, TOL),
    (3, 1, "tracers", True, 26, 2, 300.0, 4, TOL),
    (3, 0, "std_wind_tpert", True, 80, 2, 200.0, 4, TOL),
    (3, 1, "tracers", True, 80, 2, 200.0, 4, TOL),
    (3, 0, "std_wind_tpert", True, 80, 0, 200.0, 4, TOL),
    (3, 1, "tracers", True, 80, 0, 200.0, 4, TOL),
    (3, 1, "jet_moist", False, 40, 0, 300.0, 3, TOL),
    # the library's layer limit, dt shortened for the thin layers; flat,
    # because 17 terrain-following layers of a 256-layer column are too thin
    # to hold the 2 km mountain
    (3, 1, "tracers", False, 256, 0, 60.0, 3, TOL),
    (3, 1, "tracers", False, 256, 2, 60.0, 3, 1e-11),
]


def _ids(c):
    solver = {0: "auto", 1: "sweep", 2: "pcr"}[c[5]]
    return f"R{c[0]}M{c[1]}-{c[2]}{'-oro' if c[3] else ''}-L{c[4]}-{solver}"


def _step_pairs(res, moist, case, mountain, n_layers, solver, dt, steps):
    _, m_orc = make_model(res, moist, case, mountain, n_layers=n_layers)
    m_gpu = clone(m_orc)
    orc = Oracle(m_orc)
    gpu = abi.GpuModel(m_gpu, abi.FP64, column_solver=solver)
    errs = []
    try:
        driver.start(m_orc, orc.linear_combine_two_states)
        driver.start(m_gpu, gpu.linear_combine_two_states)
        for n in range(steps):
            driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
            driver.step(m_gpu, gpu.linear_combine_two_states, gpu.manage_rkhevi, dt, n * dt)
            errs.append(state_errors(m_gpu.state_new, m_orc.state_new, m_gpu.layout))
            m_gpu.state_new.copy_from(m_orc.state_new)
    finally:
        gpu.close()
    return errs


@pytest.mark.parametrize("cfg", CASES, ids=_ids)
def test_column_solver_matches_oracle(cfg):
    *run, tol_exner = cfg
    errs = _step_pairs(*run)
    worst = {f: max(e[f] for e in errs) for f in errs[0]}
    print(f"{_ids(cfg)}: worst per-step relative error {max(worst.values()):.3g} "
          f"(Pi' {worst['exner_pert']:.3g}, rho*theta_v {worst['rhotheta_v']:.3g})")
    for n, e in enumerate(errs):
        assert e["exner_pert"] <= tol_exner, f"step {n}: {e}"
        assert max(v for f, v in e.items() if f != "exner_pert") <= TOL, f"step {n}: {e}"


def _run(m, precision, solver, steps, dt, double_float=1):
    g = abi.GpuModel(m, precision, column_solver=solver, double_float=double_float)
    try:
        driver.run(m, steps, dt, g.linear_combine_two_states, g.manage_rkhevi)
    finally:
        g.close()


@pytest.mark.parametrize("n_layers,solver", [(26, 2), (80, 2), (80, 0)])
def test_mixed_pcr_close_to_fp64(n_layers, solver):
    """solver 0 at 80 layers: the default, cyclic reduction for both batches
    of this 642-column grid"""
    res, moist, case, dt, steps = 3, 1, "jet_moist", 300.0, 4
    _, m64 = make_model(res, moist, case, n_layers=n_layers)
    m32 = clone(m64)
    _run(m64, abi.FP64, 0, steps, dt)
    _run(m32, abi.MIXED, solver, steps, dt)
    e = state_errors(m32.state_new, m64.state_new, m64.layout)
    print(f"mixed (cyclic reduction, solver {solver}) vs FP64, {n_layers} layers, {steps} steps: {e}")
    assert e["rho[4]"] < 1e-5 and e["rhotheta_v"] < 1e-5 and e["exner_pert"] < 1e-3, e
    assert e["wind_h"] < 1e-3, e


@pytest.mark.parametrize("n_layers", [26, 80])
def test_mixed_pcr_equals_thomas_to_rounding(n_layers):
    """mixed path with FP64 eliminations: the cyclic reduction and the Thomas
    sweeps solve the same systems, so two steps agree far below the mixed
    path's own error"""
    _, m_a = make_model(3, 1, "jet_moist", False, n_layers=n_layers)
    m_b = clone(m_a)
    _run(m_a, abi.MIXED, 1, 2, 300.0, double_float=0)
    _run(m_b, abi.MIXED, 2, 2, 300.0, double_float=0)
    e = state_errors(m_b.state_new, m_a.state_new, m_a.layout)
    print(f"mixed, {n_layers} layers, cyclic reduction vs FP64 Thomas sweeps after 2 steps: {e}")
    assert max(e.values()) < 1e-9, e


def test_mixed_pcr_close_to_double_float_thomas():
    """the default mixed path at 26 layers sweeps in double-float (48
    significand bits): its inputs' rounding, 2^-48, is amplified by the
    acoustic system's condition number (of order (c dt / dz)^2, about 1e4 at
    dt = 300 s on this grid), so two steps agree with the FP64 cyclic
    reduction to about 1e-10 in the state and 1e-7 in the (small) vertical
    wind -- still far below the mixed path's own error against FP64 (1e-6
    in w after one step)"""
    _, m_a = make_model(3, 1, "jet_moist", False, n_layers=26)
    m_b = clone(m_a)
    _run(m_a, abi.MIXED, 1, 2, 300.0, double_float=1)
    _run(m_b, abi.MIXED, 2, 2, 300.0)
    e = state_errors(m_b.state_new, m_a.state_new, m_a.layout)
    print(f"mixed, 26 layers, cyclic reduction vs double-float Thomas sweeps after 2 steps: {e}")
    w = e.pop("wind_v")
    assert w < 1e-6, w
    assert max(e.values()) < 1e-8, e


def test_solver_switch_and_layer_limit():
    _, m = make_model(3, 0, "std_wind", n_layers=80)
    with pytest.raises(abi.GpuError, match="column solver mode"):
        abi.GpuModel(m, abi.FP64, column_solver=3)
    for solver in (0, 1, 2):
        abi.GpuModel(m, abi.FP64, column_solver=solver).close()
    assert np.isfinite(m.state_old["rho"]).all()
    _, m = make_model(3, 0, "std_wind", n_layers=257)
    with pytest.raises(abi.GpuError, match="256 layers"):
        abi.GpuModel(m, abi.FP64)
