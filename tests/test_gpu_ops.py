"""Single operators through the C ABI (FP64) against the oracle on identical
host arrays.  Tolerance 1e-12 relative; outputs the reference leaves
untouched (e.g. TOA/surface w of a gradient) must come back unchanged."""
import numpy as np
import pytest

from game_archived_gb300 import abi
from helpers import make_model, rel_err
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", params=[(4, 1, True), (3, 0, False)], ids=["R4-moist-oro", "R3-dry-flat"])
def setup(request):
    res, moist, mountain = request.param
    _, m = make_model(res, moist, "tracers" if moist else "std_wind", mountain)
    g = abi.GpuModel(m, abi.FP64)
    yield m, g, Oracle(m)
    g.close()


def _fields(m):
    lay = m.layout
    rng = np.random.default_rng(7)
    s = m.state_old
    rho = s["rho"][lay.n_cond * lay.n_scalars:(lay.n_cond + 1) * lay.n_scalars].copy()
    wind = s["wind"].copy()
    scal = s["exner_pert"].copy() + 1e-3 * rng.standard_normal(lay.n_scalars)
    return rho, wind, scal


def test_grad(setup):
    m, g, o = setup
    _, _, f = _fields(m)
    a = np.full(m.layout.n_vectors, 7.0)
    b = a.copy()
    g.grad(f, a)
    o.grad(f, b)
    assert rel_err(a, b) <= TOL
    nc = m.layout.nc
    assert np.all(a[:nc] == 7.0) and np.all(a[-nc:] == 7.0)  # TOA / surface w untouched


def test_divv_h(setup):
    m, g, o = setup
    rho, wind, _ = _fields(m)
    flux = np.zeros(m.layout.n_vectors)
    o.scalar_times_vector(rho, wind, flux)
    a, b = np.zeros(m.layout.n_scalars), np.zeros(m.layout.n_scalars)
    g.divv_h(flux, a)
    o.divv_h(flux, b)
    assert rel_err(a, b) <= TOL


def test_scalar_times_vector(setup):
    m, g, o = setup
    rho, wind, _ = _fields(m)
    a = np.full(m.layout.n_vectors, -3.0)
    b = a.copy()
    g.scalar_times_vector(rho, wind, a)
    o.scalar_times_vector(rho, wind, b)
    assert rel_err(a, b) <= TOL


def test_inner_product(setup):
    m, g, o = setup
    _, wind, _ = _fields(m)
    a, b = np.zeros(m.layout.n_scalars), np.zeros(m.layout.n_scalars)
    g.inner_product(wind, wind, a)
    o.inner_product(wind, wind, b)
    assert rel_err(a, b) <= TOL


def test_calc_pot_vort_and_vorticity_flux(setup):
    m, g, o = setup
    rho, wind, _ = _fields(m)
    d = m.diagnostics
    g.calc_pot_vort(wind, rho)
    pv_gpu, rel_gpu, tri_gpu = d["pot_vort"].copy(), d["rel_vort"].copy(), d["rel_vort_on_triangles"].copy()
    o.calc_pot_vort(wind, rho)
    assert rel_err(tri_gpu, d["rel_vort_on_triangles"]) <= TOL
    assert rel_err(rel_gpu, d["rel_vort"]) <= TOL
    assert rel_err(pv_gpu, d["pot_vort"]) <= TOL
    flux = np.zeros(m.layout.n_vectors)
    o.scalar_times_vector(rho, wind, flux)
    a, b = np.zeros(m.layout.n_vectors), np.zeros(m.layout.n_vectors)
    g.vorticity_flux(flux, d["pot_vort"], a)
    o.vorticity_flux(flux, d["pot_vort"], b)
    assert rel_err(a, b) <= TOL


def test_linear_combine(setup):
    m, g, o = setup
    from helpers import clone
    m2 = clone(m)
    rng = np.random.default_rng(3)
    m.state_new["wind"] += rng.standard_normal(m.layout.n_vectors)
    m2.state_new.copy_from(m.state_new)
    g.linear_combine_two_states(m.state_old, m.state_new, m.state_tendency, 0.3, 0.7)
    Oracle(m2).linear_combine_two_states(m2.state_old, m2.state_new, m2.state_tendency, 0.3, 0.7)
    for f in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        assert rel_err(m.state_tendency[f], m2.state_tendency[f]) <= TOL, f


def test_pointwise_products_and_vertical_divergence(setup):
    """scalar_times_scalar and vector_times_vector give numpy's products bit
    for bit; add_vertical_divv adds to its output as the oracle does"""
    import ctypes
    m, g, o = setup
    rho, wind, scal = _fields(m)
    out = np.zeros(m.layout.n_scalars)
    assert g.lib.scalar_times_scalar(abi._p(rho), abi._p(scal), abi._p(out)) == 0
    assert np.array_equal(out, rho * scal)
    outv = np.zeros(m.layout.n_vectors)
    assert g.lib.vector_times_vector(abi._p(wind), abi._p(wind), abi._p(outv)) == 0
    assert np.array_equal(outv, wind * wind)
    a, b = scal.copy(), scal.copy()
    assert g.lib.add_vertical_divv(abi._p(wind), abi._p(a), m.grid.ptr) == 0
    o.lib.orc_add_vertical_divv(ctypes.byref(o.g), wind.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rel_err(a, b) <= TOL
