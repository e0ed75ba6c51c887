"""Adjoint and tangent-linear models of the dry RKHEVI step (C ABI, FP64).

* the window forward of the differentiable kernels equals the fused FP64 step
  (the time loop through manage_rkhevi) to 1e-13 relative per field;
* dot-product test: <TL dx, ybar> = <dx, AD ybar> to 1e-10 relative, for
  random perturbations of every control field and random bars of every
  output field, over windows that start with the model's first step and
  over a window that starts in the middle of a run (lagged fields fixed);
* central finite differences of the objective J = sum over a 20-degree cap
  at 45N/0E of area_sfc * p_sfc^2 after a 12-step window at dt = 200 s
  (RES_ID=5, 2 km mountain): 64 seeded directions at h = 1e-6, each within
  1e-6 relative of <grad J, d>.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model, state_errors
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


def _dot(a, b):
    return sum(float(np.dot(a[f], b[f])) for f in FIELDS)


def _state_like(lay):
    return structs.HostStruct(lay, "state")


def _random_dx(m, rng):
    """perturbation of the control fields, scaled to each field's spread;
    theta_v' is not a control (rediagnosed), so it stays 0"""
    s = _state_like(m.layout)
    so = m.state_old
    for f, scale in (("rho", np.std(so["rho"])), ("rhotheta_v", np.std(so["rhotheta_v"])),
                     ("exner_pert", np.std(so["exner_pert"])), ("wind", 1.0)):
        s[f][:] = 1e-3 * scale * rng.standard_normal(s[f].size)
    return s


def _random_bar(m, rng):
    s = _state_like(m.layout)
    so = m.state_old
    for f in FIELDS:
        scale = np.std(so[f]) if f != "wind" else 1.0
        s[f][:] = rng.standard_normal(s[f].size) / max(scale, 1e-30)
    return s


@pytest.fixture(scope="module")
def dry4():
    return make_model(4, 0, "std_wind_tpert", mountain=True)


def test_window_forward_equals_the_fused_step(dry4):
    _, m = dry4
    n, dt = 4, 200.0
    m_a, m_b = clone(m), clone(m)
    g = abi.GpuModel(m_a, abi.FP64)
    try:
        driver.run(m_a, n, dt, g.linear_combine_two_states, g.manage_rkhevi)
    finally:
        g.close()
    g = abi.GpuModel(m_b, abi.FP64)
    try:
        m_b.config["totally_first_step_bool"][0] = 1
        g.window_forward(m_b.state_old, m_b.state_new, dt, n)
    finally:
        g.close()
    e = state_errors(m_b.state_new, m_a.state_new, m.layout)
    assert max(e.values()) <= 1e-13, e


@pytest.mark.parametrize("n_steps", [1, 3])
def test_dot_product_first_step_window(dry4, n_steps):
    _, m0 = dry4
    m = clone(m0)
    rng = np.random.default_rng(100 + n_steps)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, 200.0, n_steps)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"dot product, {n_steps}-step window from the first step: <TL dx, ybar> = {lhs:.17g}, "
          f"<dx, AD ybar> = {rhs:.17g}, relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert np.all(xb["theta_v_pert"] == 0.0)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_dot_product_mid_run_window(dry4):
    """a window that starts after two steps: the lagged fields of forcings are
    fixed inputs, and the lagged dependence between the window's steps is
    differentiated"""
    _, m0 = dry4
    m = clone(m0)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, 200.0, n * 200.0)
    orc.linear_combine_two_states(m.state_new, m.state_old, m.state_old, 1.0, 0.0)
    rng = np.random.default_rng(7)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 0
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, 200.0, 3)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"dot product, 3-step window from step 3: <TL dx, ybar> = {lhs:.17g}, <dx, AD ybar> = {rhs:.17g}, "
          f"relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_dot_product_config4_window():
    """the dot-product test on the adjoint configuration's own window: RES_ID=5
    with the 2 km mountain and the 1 K temperature noise, 12 steps at
    dt = 200 s from the first step"""
    _, m0 = make_model(5, 0, "std_wind_tpert", mountain=True)
    m = clone(m0)
    rng = np.random.default_rng(412)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, 200.0, 12)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"dot product, RES_ID=5 12-step window at dt = 200 s: <TL dx, ybar> = {lhs:.17g}, "
          f"<dx, AD ybar> = {rhs:.17g}, relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def cap_weights(m, lat0=45.0, lon0=0.0, radius_deg=20.0):
    """area_sfc of the columns within radius_deg of (lat0, lon0), else 0"""
    lay = m.layout
    lat, lon = m.grid["latitude_scalar"][:lay.nc], m.grid["longitude_scalar"][:lay.nc]
    p0, l0 = np.radians(lat0), np.radians(lon0)
    cosd = np.sin(lat) * np.sin(p0) + np.cos(lat) * np.cos(p0) * np.cos(lon - l0)
    inside = cosd >= np.cos(np.radians(radius_deg))
    area_sfc = m.grid["area"][lay.n_vectors - lay.nc:lay.n_vectors]
    return np.where(inside, area_sfc, 0.0)


def test_finite_differences_of_the_surface_pressure_objective():
    _, m = make_model(5, 0, "std_wind_tpert", mountain=True)
    n_steps, dt, h, n_dir = 12, 200.0, 1e-6, 64
    w = cap_weights(m)
    assert np.count_nonzero(w) > 100
    x0 = clone(m).state_old
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(x0, out, dt, n_steps)
        jb = _state_like(m.layout)
        J0 = g.sfc_pressure_objective(out, w, jb)
        grad = _state_like(m.layout)
        g.window_backward(jb, grad)
        rng = np.random.default_rng(4)
        xp, xm = _state_like(m.layout), _state_like(m.layout)
        worst = 0.0
        for k in range(n_dir):
            d = _state_like(m.layout)
            d["rho"][:] = x0["rho"] * rng.standard_normal(x0["rho"].size)
            d["rhotheta_v"][:] = x0["rhotheta_v"] * rng.standard_normal(x0["rhotheta_v"].size)
            d["exner_pert"][:] = np.std(x0["exner_pert"]) * rng.standard_normal(x0["exner_pert"].size)
            d["wind"][:] = rng.standard_normal(x0["wind"].size)
            for f in FIELDS:
                xp[f][:] = x0[f] + h * d[f]
                xm[f][:] = x0[f] - h * d[f]
            g.window_forward(xp, out, dt, n_steps)
            Jp = g.sfc_pressure_objective(out, w)
            g.window_forward(xm, out, dt, n_steps)
            Jm = g.sfc_pressure_objective(out, w)
            fd = (Jp - Jm) / (2 * h)
            ad = _dot(grad, d)
            rel = abs(fd - ad) / max(abs(ad), 1e-300)
            worst = max(worst, rel)
            assert rel <= 1e-6, (k, fd, ad, J0)
    finally:
        g.close()
    print(f"FD vs adjoint over {n_dir} directions: worst relative difference {worst:.3g}, J = {J0:.6g}")


def test_adjoint_matches_the_torch_cpu_adjoint():
    """the gradient of the surface-pressure objective after a 3-step window
    (RES_ID=3, mountain): hand-written GPU adjoint vs reverse-mode automatic
    differentiation of the FP64 PyTorch restatement on the CPU (itself pinned
    to the oracle in test_torch_adjoint.py); every control field within 1e-9
    relative"""
    torch = pytest.importorskip("torch")
    import torch_dry_step as tds
    from helpers import rel_err
    _, m = make_model(3, 0, "std_wind_tpert", mountain=True)
    n, dt = 3, 300.0
    w = cap_weights(m)
    m_g = clone(m)
    g = abi.GpuModel(m_g, abi.FP64)
    try:
        m_g.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m_g.state_old, out, dt, n)
        jb = _state_like(m.layout)
        J_gpu = g.sfc_pressure_objective(out, w, jb)
        grad = _state_like(m.layout)
        g.window_backward(jb, grad)
    finally:
        g.close()
    step = tds.make_step(m, dt)
    x = tds.state_tensors(m, m.state_old)
    for k in ("rho", "rt", "ep", "w", "u"):
        x[k].requires_grad_(True)
    s = step.window(x, n)
    ps = step.sfc_pressure(s)
    J = (torch.tensor(w) * ps * ps).sum()
    J.backward()
    ref = _state_like(m.layout)
    tds.tensors_to_state(m, {"rho": x["rho"].grad, "rt": x["rt"].grad, "tp": None, "ep": x["ep"].grad,
                             "w": x["w"].grad, "u": x["u"].grad}, ref)
    assert abs(J_gpu - float(J)) <= 1e-12 * abs(float(J))
    errs = {f: rel_err(grad[f], ref[f]) for f in ("rho", "rhotheta_v", "exner_pert", "wind")}
    print(f"GPU adjoint vs CPU (torch) adjoint, max |diff| / max |ref| per field: {errs}")
    assert max(errs.values()) <= 1e-9, errs


def test_manage_rkhevi_adj_is_the_one_step_window(dry4):
    """the single-step adjoint equals a one-step window (to 1e-12 of each
    field's largest bar: the adjoint scatters with atomic additions, whose
    order varies from run to run) and passes the dot-product test against
    the one-step tangent-linear model; mid-run, so the lagged fields of
    forcings are constants of the call"""
    _, m0 = dry4
    m = clone(m0)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, 200.0, n * 200.0)
    orc.linear_combine_two_states(m.state_new, m.state_old, m.state_old, 1.0, 0.0)
    orc.linear_combine_two_states(m.state_old, m.state_old, m.state_new, 1.0, 0.0)
    rng = np.random.default_rng(11)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 0
        yb = _random_bar(m, rng)
        xb_step = _state_like(m.layout)
        g.manage_rkhevi_adj(200.0, 400.0, yb, xb_step)
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, 200.0, 1)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        xb_win = _state_like(m.layout)
        g.window_backward(yb, xb_win)
    finally:
        g.close()
    for f in FIELDS:
        assert np.max(np.abs(xb_step[f] - xb_win[f])) <= 1e-12 * max(np.max(np.abs(xb_win[f])), 1e-300), f
    lhs, rhs = _dot(dy, yb), _dot(dx, xb_step)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)
