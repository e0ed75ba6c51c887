"""Operator adjoints through the C ABI against their forward drop-ins.

For every forward/backward pair, <J dx, ybar> (tangent of the forward along
dx) must equal <dx, J^T ybar> (the adjoint's bars):
* linear operators (grad, divv_h): the forward itself is the tangent,
  tolerance 1e-12;
* bilinear or quadratic operators (scalar_times_vector, inner_product,
  vorticity_flux): the central difference of the forward is exact up to
  rounding, tolerance 1e-10;
* calc_pot_vort (rational in the density) and the sound-wave column solver:
  central differences at h = 1e-5 / 1e-6, tolerance 1e-7 / 1e-6.
RES_ID=3, dry, 2 km mountain (the terrain-following terms are active).
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


@pytest.fixture(scope="module")
def model():
    _, m = make_model(3, 0, "std_wind_tpert", mountain=True)
    return m


@pytest.fixture()
def gpu(model):
    g = abi.GpuModel(clone(model), abi.FP64)
    yield g
    g.close()


def _close(lhs, rhs, tol):
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs, abs(lhs - rhs) / abs(lhs))


def test_grad_adj(model, gpu):
    lay = model.layout
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(lay.n_scalars), rng.standard_normal(lay.n_vectors)
    out = np.zeros(lay.n_vectors)
    gpu.grad(x, out)
    xb = np.zeros(lay.n_scalars)
    gpu.grad_adj(y, xb)
    _close(out @ y, x @ xb, 1e-12)


def test_divv_h_adj(model, gpu):
    lay = model.layout
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(lay.n_vectors), rng.standard_normal(lay.n_scalars)
    out = np.zeros(lay.n_scalars)
    gpu.divv_h(x, out)
    xb = np.zeros(lay.n_vectors)
    gpu.divv_h_adj(y, xb)
    _close(out @ y, x @ xb, 1e-12)


def test_scalar_times_vector_adj(model, gpu):
    lay = model.layout
    rng = np.random.default_rng(3)
    s, v = model.state_old["rho"].copy(), model.state_old["wind"].copy()
    ds, dv = 1e-3 * rng.standard_normal(s.size), rng.standard_normal(v.size)
    h = 1e-3
    op, om = np.zeros(lay.n_vectors), np.zeros(lay.n_vectors)
    gpu.scalar_times_vector(s + h * ds, v + h * dv, op)
    gpu.scalar_times_vector(s - h * ds, v - h * dv, om)
    tl = (op - om) / (2 * h)
    yb = rng.standard_normal(lay.n_vectors)
    sb, vb = np.zeros(s.size), np.zeros(v.size)
    gpu.scalar_times_vector_adj(s, v, yb, sb, vb)
    _close(tl @ yb, ds @ sb + dv @ vb, 1e-10)


def test_inner_product_adj(model, gpu):
    lay = model.layout
    rng = np.random.default_rng(4)
    a = model.state_old["wind"].copy()
    b = a + rng.standard_normal(a.size)
    da, db = rng.standard_normal(a.size), rng.standard_normal(a.size)
    h = 1e-3
    op, om = np.zeros(lay.n_scalars), np.zeros(lay.n_scalars)
    gpu.inner_product(a + h * da, b + h * db, op)
    gpu.inner_product(a - h * da, b - h * db, om)
    tl = (op - om) / (2 * h)
    yb = rng.standard_normal(lay.n_scalars)
    ab, bb = np.zeros(a.size), np.zeros(a.size)
    gpu.inner_product_adj(a, b, yb, ab, bb)
    _close(tl @ yb, da @ ab + db @ bb, 1e-10)


def test_vorticity_flux_adj(model, gpu):
    lay = model.layout
    m = gpu.m
    rng = np.random.default_rng(5)
    flux = np.zeros(lay.n_vectors)
    gpu.scalar_times_vector(m.state_old["rho"], m.state_old["wind"], flux)
    gpu.calc_pot_vort(m.state_old["wind"], m.state_old["rho"])
    pv = m.diagnostics["pot_vort"].copy()
    dflux, dpv = rng.standard_normal(flux.size), 1e-8 * rng.standard_normal(pv.size)
    h = 1e-3
    op, om = np.zeros(lay.n_vectors), np.zeros(lay.n_vectors)
    gpu.vorticity_flux(flux + h * dflux, pv + h * dpv, op)
    gpu.vorticity_flux(flux - h * dflux, pv - h * dpv, om)
    tl = (op - om) / (2 * h)
    yb = rng.standard_normal(lay.n_vectors)
    fb, pb = np.zeros(flux.size), np.zeros(pv.size)
    gpu.vorticity_flux_adj(flux, pv, yb, fb, pb)
    _close(tl @ yb, dflux @ fb + dpv @ pb, 1e-10)


def test_calc_pot_vort_adj(model, gpu):
    m = gpu.m
    rng = np.random.default_rng(6)
    wind, rho = m.state_old["wind"].copy(), m.state_old["rho"].copy()
    dw, dr = rng.standard_normal(wind.size), rho * rng.standard_normal(rho.size)
    h = 1e-5
    gpu.calc_pot_vort(wind + h * dw, rho + h * dr)
    pp = m.diagnostics["pot_vort"].copy()
    gpu.calc_pot_vort(wind - h * dw, rho - h * dr)
    pm = m.diagnostics["pot_vort"].copy()
    tl = (pp - pm) / (2 * h)
    yb = rng.standard_normal(pp.size) / np.std(pp)
    wb, rb = np.zeros(wind.size), np.zeros(rho.size)
    gpu.calc_pot_vort_adj(wind, rho, yb, wb, rb)
    _close(tl @ yb, dw @ wb + dr @ rb, 1e-7)


@pytest.mark.parametrize("rk", [0, 1])
def test_three_band_solver_ver_waves_adj(model, rk):
    m = clone(model)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, 300.0, n * 300.0)
    lay = m.layout
    rng = np.random.default_rng(10 + rk)
    dt, h = 300.0, 1e-6

    def rand_state(scale_from, fields):
        s = structs.HostStruct(lay, "state")
        for f in fields:
            scale = np.abs(scale_from[f]) + np.std(scale_from[f]) if f != "wind" else 1.0
            s[f][:] = scale * rng.standard_normal(s[f].size)
        return s

    dso = rand_state(m.state_old, FIELDS)
    dsn = rand_state(m.state_new, FIELDS)
    dst = rand_state(m.state_tendency, ("rho", "rhotheta_v", "wind"))
    g = abi.GpuModel(clone(m), abi.FP64)
    try:
        outs = []
        for sgn in (1.0, -1.0):
            mm = clone(m)
            for s, d in ((mm.state_old, dso), (mm.state_new, dsn), (mm.state_tendency, dst)):
                for f in FIELDS:
                    s[f][:] = s[f] + sgn * h * d[f]
            g.three_band_solver_ver_waves(mm.state_old, mm.state_new, mm.state_tendency, dt, rk)
            outs.append(mm.state_new)
        yb = structs.HostStruct(lay, "state")
        for f in FIELDS:
            yb[f][:] = rng.standard_normal(yb[f].size) / (np.std(m.state_new[f]) + 1e-30)
        lhs = sum(float((outs[0][f] - outs[1][f]) @ yb[f]) / (2 * h) for f in FIELDS)
        sob, stb = structs.HostStruct(lay, "state"), structs.HostStruct(lay, "state")
        snb = structs.HostStruct(lay, "state")
        snb.copy_from(yb)
        g.three_band_solver_ver_waves_adj(m.state_old, m.state_new, m.state_tendency, dt, rk, sob, snb, stb)
    finally:
        g.close()
    rhs = sum(float(dso[f] @ sob[f] + dsn[f] @ snb[f] + dst[f] @ stb[f]) for f in FIELDS)
    print(f"column solver adjoint, rk {rk}: FD tangent {lhs:.15g}, adjoint {rhs:.15g}")
    _close(lhs, rhs, 1e-6)


def test_divv_h_tracer_adj(model, gpu):
    """bilinear in (density, wind) with the upstream pick held: central
    differences at a small step are exact up to rounding"""
    lay = model.layout
    rng = np.random.default_rng(7)
    v = rng.standard_normal(lay.n_vectors)
    dens, wind = model.state_old["rho"][:lay.n_scalars].copy(), model.state_old["wind"].copy()
    dv, dd, dw = rng.standard_normal(v.size), dens * rng.standard_normal(dens.size), rng.standard_normal(wind.size)
    h = 1e-6
    op, om = np.zeros(lay.n_scalars), np.zeros(lay.n_scalars)
    gpu.divv_h_tracer(v + h * dv, dens + h * dd, wind + h * dw, op)
    gpu.divv_h_tracer(v - h * dv, dens - h * dd, wind - h * dw, om)
    tl = (op - om) / (2 * h)
    yb = rng.standard_normal(lay.n_scalars)
    vb, db, wb = np.zeros(v.size), np.zeros(dens.size), np.zeros(wind.size)
    gpu.divv_h_tracer_adj(v, dens, wind, yb, vb, db, wb)
    _close(tl @ yb, dv @ vb + dd @ db + dw @ wb, 1e-8)
    # the terrain term alone (flux field unperturbed) is exercised too
    assert np.abs(db).max() > 0 and np.abs(wb).max() > 0


@pytest.fixture(scope="module")
def moist_model():
    """RES_ID=3, moist build, seeded tracers, 2 km mountain, after two oracle
    steps (tendencies, temperature and vertical wind of a running model)"""
    _, m = make_model(3, 1, "tracers", mountain=True)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, 300.0, n * 300.0)
    return m


@pytest.mark.parametrize("rk", [0, 1])
def test_three_band_solver_gen_densities_adj(moist_model, rk):
    """central differences of the tracer column solver (densities and, at rk
    0, sedimentation heat) along random directions in the old and new
    vertical wind, the old densities, the tendencies and the temperature"""
    m = moist_model
    lay = m.layout
    ns, n_const, cond = lay.n_scalars, lay.n_const, lay.n_cond
    tracer = np.ones(n_const * ns, dtype=bool)
    tracer[cond * ns:(cond + 1) * ns] = False
    rng = np.random.default_rng(20 + rk)
    dt, h = 300.0, 1e-6
    dso, dsn, dst = (structs.HostStruct(lay, "state") for _ in range(3))
    dso["rho"][:] = np.where(tracer, m.state_old["rho"] * rng.standard_normal(n_const * ns), 0.0)
    # scaled by the local density so that no perturbed solution crosses the clip at zero
    dst["rho"][:] = np.where(tracer, m.state_old["rho"] / dt * rng.standard_normal(n_const * ns), 0.0)
    for d in (dso, dsn):
        d["wind"][:(lay.nl + 1) * lay.nc] = 0.1 * rng.standard_normal((lay.nl + 1) * lay.nc)
    t0 = m.diagnostics["temperature"].copy()
    dT = rng.standard_normal(t0.size)
    g = abi.GpuModel(clone(m), abi.FP64)
    mm = g.m
    try:
        outs = []
        for sgn in (1.0, -1.0):
            so, sn, st = (structs.HostStruct(lay, "state") for _ in range(3))
            for s, base, d in ((so, m.state_old, dso), (sn, m.state_new, dsn), (st, m.state_tendency, dst)):
                for f in FIELDS:
                    s[f][:] = base[f] + sgn * h * d[f]
            mm.diagnostics["temperature"][:] = t0 + sgn * h * dT
            mm.irrev["condensates_sediment_heat"][:] = 0.0
            g.three_band_solver_gen_densities(so, sn, st, dt, rk)
            outs.append((sn["rho"].copy(), mm.irrev["condensates_sediment_heat"].copy()))
        yb = np.where(tracer, rng.standard_normal(n_const * ns) / np.std(m.state_new["rho"][tracer]), 0.0)
        hb = rng.standard_normal(ns) / (np.std(outs[0][1]) + 1e-30) if rk == 0 else np.zeros(ns)
        lhs = float((outs[0][0] - outs[1][0]) @ yb) / (2 * h)
        if rk == 0:
            lhs += float((outs[0][1] - outs[1][1]) @ hb) / (2 * h)
        mm.diagnostics["temperature"][:] = t0
        sob, snb, stb = (structs.HostStruct(lay, "state") for _ in range(3))
        snb["rho"][:] = yb
        db, ib = structs.HostStruct(lay, "diagnostics"), structs.HostStruct(lay, "irrev")
        ib["condensates_sediment_heat"][:] = hb
        g.three_band_solver_gen_densities_adj(m.state_old, m.state_new, m.state_tendency, dt, rk, sob, snb, stb, db,
                                              ib)
    finally:
        g.close()
    assert np.all(snb["rho"][tracer] == 0.0)
    if rk == 0:
        assert np.all(ib["condensates_sediment_heat"] == 0.0)
    rhs = sum(float(dso[f] @ sob[f] + dsn[f] @ snb[f] + dst[f] @ stb[f]) for f in FIELDS)
    rhs += float(dT @ db["temperature"])
    print(f"tracer solver adjoint, rk {rk}: FD tangent {lhs:.15g}, adjoint {rhs:.15g}")
    _close(lhs, rhs, 1e-6)
