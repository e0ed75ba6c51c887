"""Windows whose forward of record is the mixed-precision step (C ABI).

With the library's precision set to the mixed one, rkhevi_window_forward
runs the fused mixed step (FP32 horizontal operators, double-float vertical
eliminations, FP64 state) and checkpoints its trajectory; the tangent-linear
and adjoint models are the FP64 ones, linearised about that trajectory (the
backward sweep recomputes every step in FP64 from its mixed checkpoint).

* the window's end state equals the mixed time loop through manage_rkhevi
  (the reference's loop, src/coordinator.c:302-324), bit for bit;
* dot-product test <TL dx, ybar> = <dx, AD ybar> to 1e-10 relative, dry and
  moist builds, windows from the first step;
* the gradient of the surface-pressure objective from the mixed window is
  within 1e-4 (norm-relative per field) of the FP64 window's: the two
  trajectories differ by the mixed path's rounding (about 1e-7 relative);
* a device-resident mixed run interrupted by a mixed window continues bit
  for bit as if it had not been: the window saves and restores the lagged
  step fields the run carries between calls.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model, state_errors

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


def _dot(a, b):
    return sum(float(np.dot(a[f], b[f])) for f in FIELDS)


def _state_like(lay):
    return structs.HostStruct(lay, "state")


def _random_dx(m, rng):
    s = _state_like(m.layout)
    so = m.state_old
    s["rho"][:] = 1e-3 * so["rho"] * rng.standard_normal(so["rho"].size)
    for f, scale in (("rhotheta_v", np.std(so["rhotheta_v"])), ("exner_pert", np.std(so["exner_pert"])),
                     ("wind", 1.0)):
        s[f][:] = 1e-3 * scale * rng.standard_normal(s[f].size)
    return s


def _random_bar(m, rng):
    s = _state_like(m.layout)
    so = m.state_old
    lay = m.layout
    ns = lay.n_scalars
    for k in range(lay.n_const):
        sl = slice(k * ns, (k + 1) * ns)
        s["rho"][sl] = rng.standard_normal(ns) / max(np.std(so["rho"][sl]), 1e-30)
    for f in ("rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        scale = np.std(so[f]) if f != "wind" else 1.0
        s[f][:] = rng.standard_normal(s[f].size) / max(scale, 1e-30)
    return s


CASES = {"dry": (3, 0, "std_wind_tpert", 200.0), "moist": (3, 1, "tracers", 300.0)}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    res, moist, name, dt = CASES[request.param]
    _, m = make_model(res, moist, name, mountain=True)
    return request.param, m, dt


@pytest.mark.parametrize("double_float", [1, 0])
def test_mixed_window_forward_is_the_mixed_time_loop(case, double_float):
    """with the vertical eliminations in double-float (default) and in FP64"""
    label, m, dt = case
    n = 3
    m_a, m_b = clone(m), clone(m)
    g = abi.GpuModel(m_a, abi.MIXED, double_float=double_float)
    try:
        driver.run(m_a, n, dt, g.linear_combine_two_states, g.manage_rkhevi)
    finally:
        g.close()
    g = abi.GpuModel(m_b, abi.MIXED, double_float=double_float)
    try:
        m_b.config["totally_first_step_bool"][0] = 1
        g.window_forward(m_b.state_old, m_b.state_new, dt, n)
    finally:
        g.close()
    e = state_errors(m_b.state_new, m_a.state_new, m.layout)
    print(f"\n{label}: mixed window forward (double-float {double_float}) vs the mixed time loop after {n} steps: "
          f"max {max(e.values()):.3g}")
    assert max(e.values()) == 0.0, e


@pytest.mark.parametrize("n_steps", [1, 3])
def test_mixed_window_dot_product(case, n_steps):
    label, m0, dt = case
    m = clone(m0)
    rng = np.random.default_rng(300 + n_steps)
    g = abi.GpuModel(m, abi.MIXED)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, dt, n_steps)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"\n{label}: mixed-window dot product, {n_steps} steps: <TL dx, ybar> = {lhs:.17g}, "
          f"<dx, AD ybar> = {rhs:.17g}, relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def _cap_weights(m, lat0=45.0, lon0=0.0, radius_deg=20.0):
    lay = m.layout
    lat, lon = m.grid["latitude_scalar"][:lay.nc], m.grid["longitude_scalar"][:lay.nc]
    p0, l0 = np.radians(lat0), np.radians(lon0)
    cosd = np.sin(lat) * np.sin(p0) + np.cos(lat) * np.cos(p0) * np.cos(lon - l0)
    area_sfc = m.grid["area"][lay.n_vectors - lay.nc:lay.n_vectors]
    return np.where(cosd >= np.cos(np.radians(radius_deg)), area_sfc, 0.0)


def _gradient(m, precision, dt, n_steps):
    g = abi.GpuModel(m, precision)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, dt, n_steps)
        jb = _state_like(m.layout)
        J = g.sfc_pressure_objective(out, _cap_weights(m), jb)
        grad = _state_like(m.layout)
        g.window_backward(jb, grad)
    finally:
        g.close()
    return J, grad


def test_mixed_window_gradient_close_to_the_fp64_window(case):
    label, m0, dt = case
    J64, g64 = _gradient(clone(m0), abi.FP64, dt, 3)
    J32, g32 = _gradient(clone(m0), abi.MIXED, dt, 3)
    e = state_errors(g32, g64, m0.layout)
    e = {k: v for k, v in e.items() if np.isfinite(v)}
    print(f"\n{label}: objective mixed {J32:.17g} vs FP64 {J64:.17g}; gradient mixed vs FP64 window: "
          + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
    assert abs(J32 / J64 - 1) < 1e-6
    assert max(e.values()) < 1e-4, e


def test_resident_run_unaffected_by_a_mixed_window(case):
    label, m0, dt = case
    n1, n2 = 2, 2

    def run(with_window):
        m = clone(m0)
        g = abi.GpuModel(m, abi.MIXED, resident=True, graphs=True)
        try:
            for s in (m.state_old, m.state_new, m.state_tendency):
                g.sync_to_device(s)
            driver.start(m, g.linear_combine_two_states)
            t = 0.0
            for _ in range(n1):
                driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
                t += dt
            if with_window:
                g.sync_to_host(m.state_new)
                init = m.state_new.clone()
                out = _state_like(m.layout)
                first = int(m.config["totally_first_step_bool"][0])
                m.config["totally_first_step_bool"][0] = 1
                g.window_forward(init, out, dt, 2)
                m.config["totally_first_step_bool"][0] = first
            for _ in range(n2):
                driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
                t += dt
            g.sync_to_host(m.state_new)
        finally:
            g.close()
        return m.state_new

    a, b = run(False), run(True)
    e = state_errors(b, a, m0.layout)
    print(f"\n{label}: resident mixed run with a window in between vs without: max {max(e.values()):.3g}")
    assert max(e.values()) == 0.0, e
