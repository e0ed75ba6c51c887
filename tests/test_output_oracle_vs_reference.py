"""The oracle's output diagnostics against the reference's own write_out.

The reference's src/io/write_output.c and src/io/spatial_ops_for_output.c are
compiled into the reference harness (oracle/build_ref.py) against stand-ins
for the netCDF and ecCodes libraries that record every array handed to the
writers.  write_out runs with every output switch on; the oracle's restatement
(orc_write_out_fields, orc_interpolate_to_ll) runs on a clone of the same
model; every field must be identical to the last bit: the surface fields, the
pressure-level fields, the model-level fields, each of them interpolated to the
lat-lon grid as the GRIB path writes it, the Diagnostics members write_out
leaves behind, and the state's theta_v_pert, which write_out rounds in the top
layer.
"""
import numpy as np
import pytest

import refbind
from helpers import clone, output_scenario
from oracle import bind

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference sources not present")

SURFACE = [("mslp", "mslp"), ("surface_p", "surface_p"), ("t2", "t2"), ("tcdc", "tcdc"), ("rprate", "rprate"),
           ("sprate", "sprate"), ("cape", "cape"), ("sfc_sw_down", "sfc_sw_down"), ("10u", "u10"), ("10v", "v10"),
           ("10gusts", "gusts")]
PLEVELS = [("geopotential_height", "geopotential_height"), ("temperature", "t_pl"), ("relative_humidity", "rh_pl"),
           ("ertels_potential_vorticity", "epv_pl"), ("wind_u", "u_pl"), ("wind_v", "v_pl"),
           ("relative_vorticity", "rel_vort_pl")]
GRIB_SURFACE = ["surface_p", "mslp", "t2", "rprate", "cape", "sfc_sw_down", "sprate", "tcdc", "u10", "v10", "gusts"]
GRIB_PLEVELS = ["geopotential_height", "t_pl", "rh_pl", "rel_vort_pl", "epv_pl", "u_pl", "v_pl"]


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("res,moist,case,mountain,gusts", [
    (3, 0, "std_wind_tpert", True, False),
    (3, 1, "tracers", True, True),
    (4, 1, "jet_moist", False, False),
])
def test_write_out_fields_equal_reference(res, moist, case, mountain, gusts, tmp_path):
    m, wl, nw = output_scenario(res, moist, case, mountain, gust_scheme=gusts)
    lay = m.layout
    m_orc = clone(m)
    ref = refbind.Reference(m)
    got = refbind.write_out(ref, m.state_new, wl, nw, str(tmp_path))
    orc = bind.Oracle(m_orc)
    out = bind.write_out_fields(orc, m_orc.state_new, wl, nw)

    for ref_name, name in SURFACE:
        assert _same(got["surface"][ref_name], out[name]), name
    for ref_name, name in PLEVELS:
        assert _same(got["pressure_levels"][ref_name], out[name]), name
    ml = got["model_levels"]
    assert _same(ml["temperature"], m_orc.diagnostics["temperature"])
    assert _same(ml["rh"], out["rh"])
    assert _same(ml["rel_vort"], out["rel_vort"])
    assert _same(ml["divv_h_all_layers"], out["divv_h"])
    for f in ("u_at_edge", "v_at_edge", "u_at_cell", "v_at_cell", "rel_vort", "pot_vort", "temperature",
              "scalar_field_placeholder"):
        assert _same(m.diagnostics[f], m_orc.diagnostics[f]), f
    assert _same(m.state_new["theta_v_pert"], m_orc.state_new["theta_v_pert"])

    ll = lambda f: bind.interpolate_to_ll(orc, f)  # noqa: E731
    assert len(got["grib_surface"]) == len(GRIB_SURFACE)
    for arr, name in zip(got["grib_surface"], GRIB_SURFACE):
        assert _same(arr, ll(out[name])), name
    npl, nc, nl = bind.N_PRESSURE_LEVELS, lay.nc, lay.nl
    gp = got["grib_pressure_levels"]
    assert len(gp) == npl * len(GRIB_PLEVELS)
    for j in range(npl):
        for k, name in enumerate(GRIB_PLEVELS):
            assert _same(gp[j * len(GRIB_PLEVELS) + k], ll(out[name].reshape(nc, npl)[:, j])), (name, j)
    gm = got["grib_model_levels"]
    assert len(gm) == 7 * nl + nl + 1
    t = m_orc.diagnostics["temperature"]
    for layer in range(nl):
        sl = slice(layer * nc, (layer + 1) * nc)
        fields = [t[sl], out["pressure"][sl], out["rh"][sl], m_orc.diagnostics["u_at_cell"][sl],
                  m_orc.diagnostics["v_at_cell"][sl], out["rel_vort"][sl], out["divv_h"][sl]]
        for k, f in enumerate(fields):
            assert _same(gm[7 * layer + k], ll(f)), (layer, k)
    for level in range(nl + 1):
        w = m_orc.state_new["wind"][level * lay.vpl:level * lay.vpl + nc]
        assert _same(gm[7 * nl + level], ll(w)), level
    # the fields carry information (not all zero / all missing)
    assert np.ptp(out["t2"]) > 0 and np.ptp(out["epv"]) > 0 and np.any(out["t_pl"] != 9999)
    if moist:
        assert np.any(out["tcdc"] > 0) and np.any(out["tcdc"] == 0) and np.any(out["rprate"] > 0)
