"""Adjoint and tangent-linear models of the moist RKHEVI step (C ABI, FP64).

The moist build adds to the dry step the temperature and phase transitions
of every step (src/constituents/phase_trans.c:16-311), the moist scalar
tendencies (src/time_stepping/scalar_tendencies_expl.c:90-178), the tracer
column solve with the sedimentation heat (column_solvers.c:385-639) and the
condensate terms of the pressure gradient and of the vertical momentum
(manage_pressure_gradient.c:63-87).  The main case has every constituent
seeded (snow, rain, cloud ice and water, vapour: cases.py "tracers") and the
2 km mountain, so phase transitions, sedimentation and the terrain terms all
act.

* the window forward of the differentiable kernels equals the fused FP64
  step (the time loop through manage_rkhevi) to 1e-13 relative per field;
* dot-product test <TL dx, ybar> = <dx, AD ybar> to 1e-10 relative, for
  random perturbations of every control field (all six densities, rho
  theta_v, Pi', w, u) and random bars of every output field, over windows
  from the model's first step and from the middle of a run;
* central finite differences of the moist surface-pressure objective
  (write_output.c:105-121 with the vapour's gas constant) on 64 seeded
  directions (every density in proportion to itself, rho theta_v, Pi' and
  the wind), h = 1e-6, within 1e-6 relative of <grad J, d>, on the moist
  baroclinic state (relative humidity 0.7, no condensate; with the 2 km
  mountain) spun up by the oracle for 6 steps, then a 3-step window.  The
  spin-up matters: the vertical tracer transport takes its upstream density
  by the sign of w (column_solvers.c:453-463, 478-542), and an initial state has
  w = 0 exactly, so at the model's first step every interface sits on that
  switch and a central difference averages two one-sided slopes (the
  vapour's derivative by the wind then differs from FD by up to 100 %); once
  |w| > 0 almost everywhere the switch is crossed by a vanishing share of
  the interfaces.  With every condensate seeded (the "tracers" case) the
  step is not differentiable everywhere even then -- all snow turns into
  rain within one step where T >= T_0 (src/constituents/phase_trans.c:
  236-262), and evaporation is capped by the available cloud water (fmin)
  -- so there the median agreement is bounded (1e-4) and the worst reported.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model, state_errors
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")
DT = 300.0


def _dot(a, b):
    return sum(float(np.dot(a[f], b[f])) for f in FIELDS)


def _state_like(lay):
    return structs.HostStruct(lay, "state")


def _random_dx(m, rng):
    """perturbation of the control fields (theta_v' is rediagnosed, so it
    stays 0): each density in proportion to itself, the rest scaled to the
    field's spread"""
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
        scale = max(np.std(so["rho"][sl]), 1e-30)
        s["rho"][sl] = rng.standard_normal(ns) / scale
    for f in ("rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        scale = np.std(so[f]) if f != "wind" else 1.0
        s[f][:] = rng.standard_normal(s[f].size) / max(scale, 1e-30)
    return s


@pytest.fixture(scope="module")
def moist3():
    return make_model(3, 1, "tracers", mountain=True)


def test_moist_window_forward_equals_the_fused_step(moist3):
    _, m = moist3
    n = 3
    m_a, m_b = clone(m), clone(m)
    g = abi.GpuModel(m_a, abi.FP64)
    try:
        driver.run(m_a, n, DT, g.linear_combine_two_states, g.manage_rkhevi)
    finally:
        g.close()
    g = abi.GpuModel(m_b, abi.FP64)
    try:
        m_b.config["totally_first_step_bool"][0] = 1
        g.window_forward(m_b.state_old, m_b.state_new, DT, n)
    finally:
        g.close()
    e = state_errors(m_b.state_new, m_a.state_new, m.layout)
    print(f"\nmoist window forward vs fused FP64 step after {n} steps: {e}")
    assert max(e.values()) <= 1e-13, e


@pytest.mark.parametrize("n_steps", [1, 3])
def test_moist_dot_product_first_step_window(moist3, n_steps):
    _, m0 = moist3
    m = clone(m0)
    rng = np.random.default_rng(200 + n_steps)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, DT, n_steps)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"\nmoist dot product, {n_steps}-step window from the first step: <TL dx, ybar> = {lhs:.17g}, "
          f"<dx, AD ybar> = {rhs:.17g}, relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert np.all(xb["theta_v_pert"] == 0.0)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_moist_dot_product_mid_run_window(moist3):
    """a window that starts after two steps: the lagged fields (pressure
    gradient, vorticity flux, kinetic-energy gradient, sedimentation heat)
    are fixed inputs"""
    _, m0 = moist3
    m = clone(m0)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, DT, n * DT)
    orc.linear_combine_two_states(m.state_new, m.state_old, m.state_old, 1.0, 0.0)
    rng = np.random.default_rng(17)
    g = abi.GpuModel(m, abi.FP64)
    try:
        m.config["totally_first_step_bool"][0] = 0
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, DT, 2)
        dx = _random_dx(m, rng)
        dy = _state_like(m.layout)
        g.window_tl(dx, dy)
        yb = _random_bar(m, rng)
        xb = _state_like(m.layout)
        g.window_backward(yb, xb)
    finally:
        g.close()
    lhs, rhs = _dot(dy, yb), _dot(dx, xb)
    print(f"\nmoist dot product, 2-step window from step 3: <TL dx, ybar> = {lhs:.17g}, <dx, AD ybar> = {rhs:.17g}, "
          f"relative difference {abs(lhs - rhs) / abs(lhs):.3g}")
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def cap_weights(m, lat0=45.0, lon0=0.0, radius_deg=20.0):
    lay = m.layout
    lat, lon = m.grid["latitude_scalar"][:lay.nc], m.grid["longitude_scalar"][:lay.nc]
    p0, l0 = np.radians(lat0), np.radians(lon0)
    cosd = np.sin(lat) * np.sin(p0) + np.cos(lat) * np.cos(p0) * np.cos(lon - l0)
    area_sfc = m.grid["area"][lay.n_vectors - lay.nc:lay.n_vectors]
    return np.where(cosd >= np.cos(np.radians(radius_deg)), area_sfc, 0.0)


def _spun_up(case, n_spin):
    """the case after n_spin oracle steps, as the state_old of a window that
    does not start with the model's first step (lagged fields in forcings)"""
    _, m = make_model(3, 1, case, mountain=True)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(n_spin):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, DT, n * DT)
    orc.linear_combine_two_states(m.state_new, m.state_old, m.state_old, 1.0, 0.0)
    m.config["totally_first_step_bool"][0] = 0
    return m


def _fd_run(m, n_steps, h, n_dir, seed):
    """(worst, median, all, J) of the relative differences between central
    finite differences of the objective and <grad J, d> over n_dir
    directions; the window starts from m.state_old with m's first-step flag"""
    w = cap_weights(m)
    x0 = clone(m).state_old
    g = abi.GpuModel(m, abi.FP64)
    try:
        out = _state_like(m.layout)
        g.window_forward(x0, out, DT, n_steps)
        jb = _state_like(m.layout)
        J0 = g.sfc_pressure_objective(out, w, jb)
        grad = _state_like(m.layout)
        g.window_backward(jb, grad)
        rng = np.random.default_rng(seed)
        xp, xm = _state_like(m.layout), _state_like(m.layout)
        rels = []
        for _ in range(n_dir):
            d = _state_like(m.layout)
            d["rho"][:] = x0["rho"] * rng.standard_normal(x0["rho"].size)
            d["rhotheta_v"][:] = x0["rhotheta_v"] * rng.standard_normal(x0["rhotheta_v"].size)
            d["exner_pert"][:] = np.std(x0["exner_pert"]) * rng.standard_normal(x0["exner_pert"].size)
            d["wind"][:] = rng.standard_normal(x0["wind"].size)
            for f in FIELDS:
                xp[f][:] = x0[f] + h * d[f]
                xm[f][:] = x0[f] - h * d[f]
            g.window_forward(xp, out, DT, n_steps)
            Jp = g.sfc_pressure_objective(out, w)
            g.window_forward(xm, out, DT, n_steps)
            Jm = g.sfc_pressure_objective(out, w)
            fd = (Jp - Jm) / (2 * h)
            ad = _dot(grad, d)
            rels.append(abs(fd - ad) / max(abs(ad), 1e-300))
    finally:
        g.close()
    return max(rels), float(np.median(rels)), rels, J0


def test_moist_finite_differences_of_the_surface_pressure_objective():
    m = _spun_up("baroclinic_moist", 6)
    worst, med, rels, J0 = _fd_run(m, 3, 1e-6, 64, 9)
    print(f"\nmoist (baroclinic, after 6 steps) FD vs adjoint over 64 directions: worst relative difference "
          f"{worst:.3g}, median {med:.3g}, J = {J0:.6g}")
    assert worst <= 1e-6, sorted(rels)[-5:]


def test_moist_finite_differences_across_microphysics_switches():
    m = _spun_up("tracers", 6)
    worst, med, rels, _ = _fd_run(m, 3, 1e-6, 16, 19)
    print(f"\nmoist (all condensates seeded, after 6 steps) FD vs adjoint over 16 directions: worst relative "
          f"difference {worst:.3g}, median {med:.3g}")
    assert med <= 1e-4, sorted(rels)
