"""Pins the oracle to the reference: the reference's own C (compiled from its
sources into oracle/_ref by oracle/build_ref.py) and the oracle run the same
driver loop on identical host structs; every byte of State, Diagnostics,
Forcings and Irreversible_quantities must agree after every step.  Runs only
where the reference sources exist (this build container)."""
import numpy as np
import pytest

from game_archived_gb300 import driver
from helpers import clone, make_model
from oracle.bind import Oracle

refbind = pytest.importorskip("refbind")
pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference sources not present")

CASES = [
    (3, 0, "std_wind", False, 400.0, 4),
    (3, 1, "jet_moist", True, 300.0, 3),
    (4, 0, "std_wind_tpert", True, 200.0, 3),
    (4, 1, "tracers", False, 300.0, 2),
]


@pytest.mark.parametrize("cfg", CASES, ids=lambda c: f"R{c[0]}M{c[1]}-{c[2]}{'-oro' if c[3] else ''}")
def test_oracle_bitwise_equals_reference(cfg):
    res, moist, case, mountain, dt, steps = cfg
    _, m_ref = make_model(res, moist, case, mountain)
    m_orc = clone(m_ref)
    ref = refbind.Reference(m_ref)
    orc = Oracle(m_orc)
    driver.start(m_ref, ref.linear_combine_two_states)
    driver.start(m_orc, orc.linear_combine_two_states)
    for n in range(steps):
        driver.step(m_ref, ref.linear_combine_two_states, ref.manage_rkhevi, dt, n * dt)
        driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
        for k in ("state_old", "state_new", "state_tendency", "diagnostics", "forcings", "irrev"):
            a, b = getattr(m_ref, k).buf, getattr(m_orc, k).buf
            assert np.array_equal(a, b), f"step {n}: {k} differs in {np.count_nonzero(a != b)} bytes"


def test_reference_operators_equal_oracle():
    """single operators called on host arrays, as the reference's
    initialisation and output code call them"""
    _, m = make_model(3, 1, "tracers", True)
    ref = refbind.Reference(m)
    import ctypes
    vp = ctypes.c_void_p
    lib = ref.lib
    lay = m.layout
    orc = Oracle(m)
    rng = np.random.default_rng(11)
    s = m.state_old["exner_pert"] + 1e-3 * rng.standard_normal(lay.n_scalars)
    wind = m.state_old["wind"].copy()
    for name, args_ref, args_orc, out_len in [
        ("grad", None, None, lay.n_vectors),
        ("inner_product", None, None, lay.n_scalars),
        ("divv_h", None, None, lay.n_scalars),
    ]:
        a = np.zeros(out_len)
        b = np.zeros(out_len)
        if name == "grad":
            getattr(lib, name).argtypes = [vp] * 3
            lib.grad(s.ctypes.data, a.ctypes.data, m.grid.ptr)
            orc.grad(s, b)
        elif name == "inner_product":
            lib.inner_product.argtypes = [vp] * 4
            lib.inner_product(wind.ctypes.data, wind.ctypes.data, a.ctypes.data, m.grid.ptr)
            orc.inner_product(wind, wind, b)
        else:
            lib.divv_h.argtypes = [vp] * 3
            lib.divv_h(wind.ctypes.data, a.ctypes.data, m.grid.ptr)
            orc.divv_h(wind, b)
        assert np.array_equal(a, b), name


SWITCHES = ("momentum_diff_h", "momentum_diff_v", "temperature_diff_h", "temperature_diff_v", "mass_diff_h",
            "mass_diff_v")
DIFFUSION = [
    # (res, moist, case, mountain, dt, steps, switches on)
    (3, 1, "tracers", True, 300.0, 3, SWITCHES),
    (3, 0, "std_wind_tpert", True, 300.0, 3, ("momentum_diff_h",)),
    (3, 0, "std_wind_tpert", True, 300.0, 3, ("momentum_diff_v",)),
    (3, 1, "jet_moist", False, 300.0, 2, ("mass_diff_h", "mass_diff_v")),
    (4, 1, "tracers", True, 200.0, 2, ("momentum_diff_h", "temperature_diff_h", "temperature_diff_v")),
]


def with_diffusion(m, switches, seed=5):
    """switches on, and a seeded turbulent kinetic energy of 0.5-1 J/kg (the
    reference reads TKE from its initial-state file)"""
    for s in SWITCHES:
        m.config[s][0] = 1 if s in switches else 0
    rng = np.random.default_rng(seed)
    m.irrev["tke"][:] = 0.5 + 0.5 * rng.random(m.irrev["tke"].size)
    return m


@pytest.mark.parametrize("cfg", DIFFUSION, ids=lambda c: f"R{c[0]}M{c[1]}-{c[2]}-" + "+".join(
    s.replace("_diff_", "") for s in c[6]))
def test_oracle_bitwise_equals_reference_with_diffusion(cfg):
    res, moist, case, mountain, dt, steps, switches = cfg
    _, m_ref = make_model(res, moist, case, mountain)
    with_diffusion(m_ref, switches)
    m_orc = clone(m_ref)
    ref = refbind.Reference(m_ref)
    orc = Oracle(m_orc)
    driver.start(m_ref, ref.linear_combine_two_states)
    driver.start(m_orc, orc.linear_combine_two_states)
    for n in range(steps):
        driver.step(m_ref, ref.linear_combine_two_states, ref.manage_rkhevi, dt, n * dt)
        driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
        for k in ("state_old", "state_new", "state_tendency", "diagnostics", "forcings", "irrev"):
            a, b = getattr(m_ref, k).buf, getattr(m_orc, k).buf
            assert np.array_equal(a, b), f"step {n}: {k} differs in {np.count_nonzero(a != b)} bytes"
    assert np.any(m_orc.irrev["friction_acc"] != 0) or "momentum" not in "".join(switches)


@pytest.mark.parametrize("moist,case,mountain", [(0, "std_wind_tpert", True), (1, "tracers", False)],
                         ids=["dry-oro", "moist"])
def test_oracle_bitwise_equals_reference_held_suarez(moist, case, mountain):
    """the reference's Held-Suarez run configuration (run_scripts/held_suar.sh:
    rad_on = 2, pbl_scheme = 2, horizontal momentum diffusion), the radiation
    updated at every other step as the reference's driver does for a longer
    radiation time step.  RES_ID = 5: its 10242 cells per layer split into the
    reference's 18 radiation blocks exactly (on RES3/4/6 grids with 26 layers
    the reference's block loops write past the end of radiation_tendency)."""
    _, m_ref = make_model(5, moist, case, mountain)
    with_diffusion(m_ref, ("momentum_diff_h",))
    m_ref.config["rad_on"][0] = 2
    m_ref.config["pbl_scheme"][0] = 2
    m_orc = clone(m_ref)
    ref = refbind.Reference(m_ref)
    orc = Oracle(m_orc)
    driver.start(m_ref, ref.linear_combine_two_states)
    driver.start(m_orc, orc.linear_combine_two_states)
    for n in range(4):
        for m in (m_ref, m_orc):
            m.config["rad_update"][0] = 1 if n % 2 == 0 else 0
        driver.step(m_ref, ref.linear_combine_two_states, ref.manage_rkhevi, 300.0, n * 300.0)
        driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, 300.0, n * 300.0)
        for k in ("state_old", "state_new", "state_tendency", "diagnostics", "forcings", "irrev"):
            a, b = getattr(m_ref, k).buf, getattr(m_orc, k).buf
            assert np.array_equal(a, b), f"step {n}: {k} differs in {np.count_nonzero(a != b)} bytes"
    assert np.any(m_orc.forcings["radiation_tendency"] != 0)


def test_reference_operator_variants_equal_oracle():
    """the exported operator variants the reference's initialisation, output
    and subgrid code call on host arrays (gradient_operators.c:14-91,
    averaging.c:113-133, multiplications.c:45-117, divergences.c:66-148,
    vorticities.c:87-165), bit for bit, including the entries each leaves
    untouched"""
    import ctypes
    _, m = make_model(3, 1, "tracers", True)
    ref = refbind.Reference(m)
    lib = ref.lib
    lay = m.layout
    orc = Oracle(m)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(13)
    s = m.state_old["exner_pert"] + 1e-3 * rng.standard_normal(lay.n_scalars)
    rho = m.state_old["rho"][lay.n_cond * lay.n_scalars:(lay.n_cond + 1) * lay.n_scalars].copy()
    dens = rho * (1.0 + 0.1 * rng.standard_normal(lay.n_scalars))
    wind = m.state_old["wind"] + rng.standard_normal(lay.n_vectors)

    def orc_call(name, *arrays):
        fn = getattr(orc.lib, "orc_" + name)
        assert fn(ctypes.byref(orc.g), *[a.ctypes.data_as(dp) for a in arrays]) == 0, name

    for name in ("grad_hor_cov", "grad_vert_cov", "grad_cov", "grad_hor"):
        a, b = np.full(lay.n_vectors, 7.0), np.full(lay.n_vectors, 7.0)
        getattr(lib, name).argtypes = [vp] * 3
        assert getattr(lib, name)(s.ctypes.data, a.ctypes.data, m.grid.ptr) == 0
        orc_call(name, s, b)
        assert np.array_equal(a, b), name
    a, b = wind.copy(), wind.copy()
    lib.vector_field_hor_cov_to_con.argtypes = [vp] * 2
    assert lib.vector_field_hor_cov_to_con(a.ctypes.data, m.grid.ptr) == 0
    orc_call("vector_field_hor_cov_to_con", b)
    assert np.array_equal(a, b)
    for name in ("scalar_times_vector_h", "scalar_times_vector_h_upstream", "scalar_times_vector_v"):
        a, b = np.full(lay.n_vectors, -3.0), np.full(lay.n_vectors, -3.0)
        getattr(lib, name).argtypes = [vp] * 4
        assert getattr(lib, name)(rho.ctypes.data, wind.ctypes.data, a.ctypes.data, m.grid.ptr) == 0
        orc_call(name, rho, wind, b)
        assert np.array_equal(a, b), name
    flux = np.zeros(lay.n_vectors)
    orc_call("scalar_times_vector", dens, wind, flux)
    a, b = np.zeros(lay.n_scalars), np.zeros(lay.n_scalars)
    lib.divv_h_tracer.argtypes = [vp] * 5
    assert lib.divv_h_tracer(flux.ctypes.data, dens.ctypes.data, wind.ctypes.data, a.ctypes.data, m.grid.ptr) == 0
    orc_call("divv_h_tracer", flux, dens, wind, b)
    assert np.array_equal(a, b)
    # calc_rel_vort writes diagnostics->rel_vort and rel_vort_on_triangles
    lib.calc_rel_vort.argtypes = [vp] * 4
    assert lib.calc_rel_vort(wind.ctypes.data, m.diagnostics.ptr, m.grid.ptr, m.dualgrid.ptr) == 0
    rel_ref, tri_ref = m.diagnostics["rel_vort"].copy(), m.diagnostics["rel_vort_on_triangles"].copy()
    m.diagnostics["rel_vort"][:] = 0.0
    m.diagnostics["rel_vort_on_triangles"][:] = 0.0
    od = orc.diag()
    assert orc.lib.orc_calc_rel_vort(ctypes.byref(orc.g), wind.ctypes.data_as(dp), ctypes.byref(od)) == 0
    assert np.array_equal(rel_ref, m.diagnostics["rel_vort"])
    assert np.array_equal(tri_ref, m.diagnostics["rel_vort_on_triangles"])
    a, b = np.full(rel_ref.size, 5.0), np.full(rel_ref.size, 5.0)
    lib.add_f_to_rel_vort.argtypes = [vp] * 3
    assert lib.add_f_to_rel_vort(rel_ref.ctypes.data, a.ctypes.data, m.dualgrid.ptr) == 0
    orc_call("add_f_to_rel_vort", rel_ref, b)
    assert np.array_equal(a, b)
