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


# ---------------------------------------------------------------------------
# The exported operator variants the step does not call itself but the
# reference's initialisation, output and subgrid code call on host arrays
# (src/io/set_grid_properties.c:217-221, src/subgrid_scale/*.c): each through
# the C ABI against the oracle's restatement, on host arrays in the
# reference's layout.  Outputs start from a sentinel so that the entries the
# reference leaves untouched are compared too (they must come back as the
# sentinel on both sides).

def _orc(o, name, *arrays):
    import ctypes
    fn = getattr(o.lib, "orc_" + name)
    args = [ctypes.byref(o.g)] + [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrays]
    assert fn(*args) == 0, name


def _pointwise(a, b, floor=1e-300):
    """max |a - b| / |b| over the entries where b is not (near) zero"""
    scale = np.max(np.abs(b))
    mask = np.abs(b) > max(floor, 1e-9 * scale)
    if not np.any(mask):
        return 0.0
    return float(np.max(np.abs(a[mask] - b[mask]) / np.abs(b[mask])))


@pytest.mark.parametrize("name", ["grad_hor_cov", "grad_vert_cov", "grad_cov", "grad_hor"])
def test_gradient_variants(setup, name):
    """gradient_operators.c:14-91: covariant horizontal and vertical parts,
    their sum, and the horizontal part made contravariant"""
    m, g, o = setup
    _, _, f = _fields(m)
    a = np.full(m.layout.n_vectors, 7.0)
    b = a.copy()
    assert getattr(g.lib, name)(abi._p(f), abi._p(a), m.grid.ptr) == 0, g.lib.game_gpu_last_error()
    _orc(o, name, f, b)
    assert rel_err(a, b) <= TOL, name
    assert _pointwise(a, b) <= 1e-10, name
    assert np.array_equal(a == 7.0, b == 7.0), name  # the same entries untouched


def test_vector_field_hor_cov_to_con(setup):
    """averaging.c:113-133: in place, the terrain correction of the
    horizontal components in the orography layers"""
    m, g, o = setup
    rng = np.random.default_rng(17)
    v = m.state_old["wind"] + rng.standard_normal(m.layout.n_vectors)
    a, b = v.copy(), v.copy()
    assert g.lib.vector_field_hor_cov_to_con(abi._p(a), m.grid.ptr) == 0, g.lib.game_gpu_last_error()
    _orc(o, "vector_field_hor_cov_to_con", b)
    assert rel_err(a, b) <= TOL
    assert _pointwise(a, b) <= 1e-10


@pytest.mark.parametrize("name", ["scalar_times_vector_h", "scalar_times_vector_h_upstream",
                                  "scalar_times_vector_v"])
def test_scalar_times_vector_variants(setup, name):
    """multiplications.c:45-117: edge average (or the upstream cell's value)
    times the horizontal components, interface average times the vertical
    ones; the other components are left as they were"""
    m, g, o = setup
    rho, wind, _ = _fields(m)
    a = np.full(m.layout.n_vectors, -3.0)
    b = a.copy()
    assert getattr(g.lib, name)(abi._p(rho), abi._p(wind), abi._p(a), m.grid.ptr) == 0, g.lib.game_gpu_last_error()
    _orc(o, name, rho, wind, b)
    assert rel_err(a, b) <= TOL, name
    assert _pointwise(a, b) <= 1e-12, name
    assert np.array_equal(a == -3.0, b == -3.0), name


def test_divv_h_tracer(setup):
    """divergences.c:66-148: the flux divergence of a tracer, with the
    upstream densities in the terrain vertical term"""
    m, g, o = setup
    lay = m.layout
    rho, wind, _ = _fields(m)
    rng = np.random.default_rng(19)
    dens = rho * (1.0 + 0.1 * rng.standard_normal(lay.n_scalars))
    flux = np.zeros(lay.n_vectors)
    _orc(o, "scalar_times_vector", dens, wind, flux)
    a, b = np.zeros(lay.n_scalars), np.zeros(lay.n_scalars)
    assert g.lib.divv_h_tracer(abi._p(flux), abi._p(dens), abi._p(wind), abi._p(a), m.grid.ptr) == 0, \
        g.lib.game_gpu_last_error()
    _orc(o, "divv_h_tracer", flux, dens, wind, b)
    assert rel_err(a, b) <= TOL


def test_calc_rel_vort_and_add_f_to_rel_vort(setup):
    """vorticities.c:87-165: relative vorticity (rhombi and the tangential
    components) and the Coriolis parameter added to a curl field"""
    import ctypes
    m, g, o = setup
    lay = m.layout
    _, wind, _ = _fields(m)
    d = m.diagnostics
    assert g.lib.calc_rel_vort(abi._p(wind), d.ptr, m.grid.ptr, m.dualgrid.ptr) == 0, g.lib.game_gpu_last_error()
    rel_gpu, tri_gpu = d["rel_vort"].copy(), d["rel_vort_on_triangles"].copy()
    od = o.diag()
    assert o.lib.orc_calc_rel_vort(ctypes.byref(o.g), wind.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.byref(od)) == 0
    assert rel_err(rel_gpu, d["rel_vort"]) <= TOL
    assert rel_err(tri_gpu, d["rel_vort_on_triangles"]) <= TOL
    rel = d["rel_vort"].copy()
    a = np.full(rel.size, 5.0)
    b = a.copy()
    assert g.lib.add_f_to_rel_vort(abi._p(rel), abi._p(a), m.dualgrid.ptr) == 0, g.lib.game_gpu_last_error()
    _orc(o, "add_f_to_rel_vort", rel, b)
    assert rel_err(a, b) <= TOL
    assert _pointwise(a, b) <= 1e-12
