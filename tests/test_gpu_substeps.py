"""The sub-steps of manage_rkhevi as separate C-ABI calls (FP64) against the
oracle's sub-steps, on identical inputs taken from the middle of a run.

Each case clones a model after two oracle steps (so the lagged forcings and
the sedimentation heat hold step values), evaluates the step's prelude
(temperature, phase-transition rates) on its state_old, and then runs one
sub-step on the GPU and in the oracle.  Every output member the reference
writes must agree to 1e-12 relative (max |gpu - oracle| / max |oracle|),
the tolerance of the whole step.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver
from helpers import clone, make_model, rel_err, state_errors
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
DT = 300.0


@pytest.fixture(scope="module", params=[(3, 1, "jet_moist", False), (3, 0, "std_wind_tpert", True)],
                ids=["R3-moist", "R3-dry-oro"])
def mid_run(request):
    res, moist, case, mountain = request.param
    _, m = make_model(res, moist, case, mountain)
    orc = Oracle(m)
    driver.start(m, orc.linear_combine_two_states)
    for n in range(2):
        driver.step(m, orc.linear_combine_two_states, orc.manage_rkhevi, DT, n * DT)
    # the next step's start: state_old = state_new, prelude evaluated
    orc.linear_combine_two_states(m.state_new, m.state_old, m.state_old, 1.0, 0.0)
    orc.step_prelude(m.state_old, DT)
    m.config["totally_first_step_bool"][0] = 0
    return m


def _pair(m):
    m_o, m_g = clone(m), clone(m)
    return m_o, Oracle(m_o), m_g, abi.GpuModel(m_g, abi.FP64)


def _close(a, b, what):
    e = rel_err(a, b)
    assert e <= TOL, f"{what}: {e:.3g}"


@pytest.mark.parametrize("first", [0, 1])
def test_manage_pressure_gradient(mid_run, first):
    m_o, orc, m_g, gpu = _pair(mid_run)
    try:
        for mm in (m_o, m_g):
            mm.config["totally_first_step_bool"][0] = first
        orc.manage_pressure_gradient(m_o.state_new)
        gpu.manage_pressure_gradient(m_g.state_new)
    finally:
        gpu.close()
    for f in ("pgrad_acc_old", "pressure_gradient_acc_neg_nl", "pressure_gradient_acc_neg_l"):
        _close(m_g.forcings[f], m_o.forcings[f], f)
    _close(m_g.irrev["pressure_gradient_decel_factor"], m_o.irrev["pressure_gradient_decel_factor"], "decel")


def test_calc_pressure_grad_condensates_v(mid_run):
    m_o, orc, m_g, gpu = _pair(mid_run)
    try:
        orc.calc_pressure_grad_condensates_v(m_o.state_new)
        gpu.calc_pressure_grad_condensates_v(m_g.state_new)
    finally:
        gpu.close()
    a, b = m_g.forcings["pressure_grad_condensates_v"], m_o.forcings["pressure_grad_condensates_v"]
    if np.max(np.abs(b)) == 0:  # dry: rho_gas / rho_total - 1 = 0 exactly
        assert np.max(np.abs(a)) == 0
    else:
        _close(a, b, "pressure_grad_condensates_v")
    _close(m_g.irrev["pressure_gradient_decel_factor"], m_o.irrev["pressure_gradient_decel_factor"], "decel - 1")


@pytest.mark.parametrize("rk", [0, 1])
def test_vector_tendencies_expl(mid_run, rk):
    m_o, orc, m_g, gpu = _pair(mid_run)
    try:
        orc.vector_tendencies_expl(m_o.state_new, m_o.state_tendency, rk, DT)
        gpu.vector_tendencies_expl(m_g.state_new, m_g.state_tendency, rk, DT)
    finally:
        gpu.close()
    _close(m_g.state_tendency["wind"], m_o.state_tendency["wind"], "tendency wind")
    if rk == 1:
        for f in ("pot_vort_tend", "v_squared_grad"):
            _close(m_g.forcings[f], m_o.forcings[f], f)
        for f in ("flux_density", "pot_vort", "rel_vort", "rel_vort_on_triangles", "v_squared"):
            _close(m_g.diagnostics[f], m_o.diagnostics[f], f)


@pytest.mark.parametrize("rk", [0, 1])
def test_scalar_tendencies_expl(mid_run, rk):
    m_o, orc, m_g, gpu = _pair(mid_run)
    try:
        orc.scalar_tendencies_expl(m_o.state_old, m_o.state_new, m_o.state_tendency, DT, rk)
        gpu.scalar_tendencies_expl(m_g.state_old, m_g.state_new, m_g.state_tendency, DT, rk)
    finally:
        gpu.close()
    lay = m_o.layout
    ns = lay.n_scalars
    for k in range(lay.n_const):
        _close(m_g.state_tendency["rho"][k * ns:(k + 1) * ns], m_o.state_tendency["rho"][k * ns:(k + 1) * ns],
               f"tendency rho[{k}]")
    _close(m_g.state_tendency["rhotheta_v"], m_o.state_tendency["rhotheta_v"], "tendency rhotheta_v")


@pytest.mark.parametrize("rk", [0, 1])
def test_three_band_solvers(mid_run, rk):
    m_o, orc, m_g, gpu = _pair(mid_run)
    try:
        orc.three_band_solver_ver_waves(m_o.state_old, m_o.state_new, m_o.state_tendency, DT, rk)
        gpu.three_band_solver_ver_waves(m_g.state_old, m_g.state_new, m_g.state_tendency, DT, rk)
        e = state_errors(m_g.state_new, m_o.state_new, m_o.layout)
        assert max(e.values()) <= TOL, e
        if m_o.layout.n_const > 1:
            orc.three_band_solver_gen_densities(m_o.state_old, m_o.state_new, m_o.state_tendency, DT, rk)
            gpu.three_band_solver_gen_densities(m_g.state_old, m_g.state_new, m_g.state_tendency, DT, rk)
            e = state_errors(m_g.state_new, m_o.state_new, m_o.layout)
            assert max(e.values()) <= TOL, e
            _close(m_g.irrev["condensates_sediment_heat"], m_o.irrev["condensates_sediment_heat"], "sediment heat")
    finally:
        gpu.close()


def test_substeps_compose_to_the_step(mid_run):
    """manage_rkhevi.c:48-97 driven through the sub-step entry points equals
    manage_rkhevi through the fused path (both on the GPU)"""
    m_a, m_b = clone(mid_run), clone(mid_run)
    g = abi.GpuModel(m_a, abi.FP64)
    try:
        g.manage_rkhevi(DT)
    finally:
        g.close()
    g = abi.GpuModel(m_b, abi.FP64)
    orc = Oracle(m_b)
    try:
        orc.step_prelude(m_b.state_old, DT)
        lay = m_b.layout
        for rk in range(2):
            if rk == 0:
                g.manage_pressure_gradient(m_b.state_new)
            g.calc_pressure_grad_condensates_v(m_b.state_new)
            g.vector_tendencies_expl(m_b.state_new, m_b.state_tendency, rk, DT)
            w_new, w_old, w_t = m_b.state_new["wind"], m_b.state_old["wind"], m_b.state_tendency["wind"]
            for l in range(lay.nl):
                a = lay.nc + l * lay.vpl
                w_new[a:a + lay.ne] = w_old[a:a + lay.ne] + DT * w_t[a:a + lay.ne]
            g.scalar_tendencies_expl(m_b.state_old, m_b.state_new, m_b.state_tendency, DT, rk)
            g.three_band_solver_ver_waves(m_b.state_old, m_b.state_new, m_b.state_tendency, DT, rk)
            g.three_band_solver_gen_densities(m_b.state_old, m_b.state_new, m_b.state_tendency, DT, rk)
    finally:
        g.close()
    e = state_errors(m_b.state_new, m_a.state_new, m_a.layout)
    assert max(e.values()) <= TOL, e
