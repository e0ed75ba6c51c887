"""Output diagnostics on the GPU (C ABI) against the oracle.

The oracle's output diagnostics are identical to the reference's own
write_out (tests/test_output_oracle_vs_reference.py).  Here the library's
game_gpu_write_out_fields and the output operators (interpolate_to_ll,
epv_diagnostics, calc_uv_at_edge, ...) run on the same inputs:
* every native-grid field within 1e-11 of the oracle relative to the field's
  largest magnitude (FP64 in the reference's operation order; CUDA's pow,
  log, exp, sin and cos differ from the C library's in the last bits), with
  the same missing values (9999) on the pressure levels;
* every lat-lon field (the GRIB path) within the same bound;
* the state's theta_v_pert rounded in the top layer exactly as the oracle
  rounds it;
* device-resident output with the lowest-layer winds recorded on the device
  gives the same bits as host-in/host-out output.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi
from helpers import clone, output_scenario
from oracle import bind

pytestmark = pytest.mark.gpu

TOL = 1e-11
NATIVE = {  # library name -> oracle name (None: compared separately)
    "mslp": "mslp", "surface_p": "surface_p", "t2": "t2", "tcdc": "tcdc", "rprate": "rprate", "sprate": "sprate",
    "cape": "cape", "sfc_sw_down": "sfc_sw_down", "u10": "u10", "v10": "v10", "gusts": "gusts",
    "pressure": "pressure", "rh": "rh", "rel_vort": "rel_vort", "divv_h": "divv_h", "epv": "epv",
    "geopotential_height": "geopotential_height", "t_pl": "t_pl", "rh_pl": "rh_pl", "epv_pl": "epv_pl",
    "u_pl": "u_pl", "v_pl": "v_pl", "rel_vort_pl": "rel_vort_pl"}
PLEVEL = {"geopotential_height", "t_pl", "rh_pl", "epv_pl", "u_pl", "v_pl", "rel_vort_pl"}


def close(a, b, tol=TOL):
    """max |a - b| / max |b| <= tol, 9999 (missing) at the same places"""
    miss_a, miss_b = a == 9999, b == 9999
    if not np.array_equal(miss_a, miss_b):
        return False, "missing values differ"
    a, b = a[~miss_b], b[~miss_b]
    if b.size == 0:
        return True, 0.0
    scale = np.max(np.abs(b))
    err = float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a - b)))
    return err <= tol, err


def oracle_fields(m, wl, nw):
    m_orc = clone(m)
    orc = bind.Oracle(m_orc)
    out = bind.write_out_fields(orc, m_orc.state_new, wl, nw)
    out["temperature"] = m_orc.diagnostics["temperature"].copy()
    out["u"] = m_orc.diagnostics["u_at_cell"].copy()
    out["v"] = m_orc.diagnostics["v_at_cell"].copy()
    return orc, m_orc, out


CASES = [(3, 0, "std_wind_tpert", True, False), (3, 1, "tracers", True, True), (4, 1, "jet_moist", False, False),
         (5, 0, "std_wind_tpert", True, False)]


@pytest.mark.parametrize("res,moist,case,mountain,gusts", CASES,
                         ids=[f"R{c[0]}M{c[1]}-{c[2]}{'-gusts' if c[4] else ''}" for c in CASES])
def test_write_out_fields_match_oracle(res, moist, case, mountain, gusts):
    m, wl, nw = output_scenario(res, moist, case, mountain, gust_scheme=gusts)
    orc, m_orc, ref = oracle_fields(m, wl, nw)
    g = abi.GpuModel(m, abi.FP64)
    try:
        got = g.output_fields(m.state_new, wl, nw, native=True, latlon=True)
    finally:
        g.close()
    lay = m.layout
    nc, nl = lay.nc, lay.nl
    errs = {}
    for name, oname in list(NATIVE.items()) + [("temperature", "temperature"), ("u", "u"), ("v", "v")]:
        ok, err = close(got["native"][name], ref[oname])
        errs[name] = err
        assert ok, (name, err)
    # the GRIB path: every horizontal slice interpolated to the lat-lon grid
    ll = lambda f: bind.interpolate_to_ll(orc, f)  # noqa: E731
    for name, kind in abi.OUTPUT_FIELDS:
        a = got["latlon"][name]
        if kind == 0:
            want = [ll(ref[name])]
        elif kind == 1:
            want = [ll(ref[name][k * nc:(k + 1) * nc]) for k in range(nl)]
        elif kind == 2:
            want = [ll(ref[name].reshape(nc, 6)[:, j]) for j in range(6)]
        else:
            w = m_orc.state_new["wind"]
            want = [ll(w[k * lay.vpl:k * lay.vpl + nc]) for k in range(nl + 1)]
        ok, err = close(a, np.concatenate(want))
        errs["ll_" + name] = err
        assert ok, ("latlon", name, err)
    assert np.array_equal(m.state_new["theta_v_pert"], m_orc.state_new["theta_v_pert"])
    print(f"R{res}M{moist} {case}: worst native {max(v for k, v in errs.items() if not k.startswith('ll_')):.3g}, "
          f"worst lat-lon {max(v for k, v in errs.items() if k.startswith('ll_')):.3g}")


def test_resident_output_with_recorded_winds_equals_host_mode():
    m0, wl, nw = output_scenario(3, 1, "tracers", True)
    lay = m0.layout
    ne, lo = lay.ne, lay.n_vectors - lay.vpl
    results = []
    for resident in (False, True):
        m = clone(m0)
        g = abi.GpuModel(m, abi.FP64, resident=resident)
        try:
            if resident:
                # the driver's wind bookkeeping on the device: one slot per step
                for t in range(nw):
                    m.state_old["wind"][:] = m0.state_new["wind"]
                    m.state_old["wind"][lo:lo + ne] = wl[t * ne:(t + 1) * ne]
                    g.sync_to_device(m.state_old)
                    g.record_wind_lowest(m.state_old, t)
                g.sync_to_device(m.state_new)
                out = g.output_fields(m.state_new, None, nw, native=True, latlon=True)
                g.sync_to_host(m.state_new)
            else:
                out = g.output_fields(m.state_new, wl, nw, native=True, latlon=True)
        finally:
            g.close()
        results.append((out, m.state_new["theta_v_pert"].copy()))
    (a, ta), (b, tb) = results
    for kind in ("native", "latlon"):
        for name in a[kind]:
            assert np.array_equal(a[kind][name], b[kind][name]), (kind, name)
    assert np.array_equal(ta, tb)


def test_output_operators_match_oracle():
    m, _, _ = output_scenario(4, 1, "jet_moist", False)
    lay = m.layout
    m_orc = clone(m)
    orc = bind.Oracle(m_orc)
    rng = np.random.default_rng(3)
    wind = m.state_new["wind"].copy()
    g = abi.GpuModel(m, abi.FP64)
    try:
        f = rng.standard_normal(lay.nc)
        f[7] = 9999.0   # a missing value spreads to the lat-lon points next to it
        ok, err = close(g.interpolate_to_ll(f), bind.interpolate_to_ll(orc, f))
        assert ok, ("interpolate_to_ll", err)
        e = rng.standard_normal(lay.ne)
        ok, err = close(g.edges_to_cells_lowest_layer(e),
                        bind.output_op(orc, "edges_to_cells_lowest_layer", e, out_len=lay.nc))
        assert ok, ("edges_to_cells_lowest_layer", err)
        ok, err = close(g.edges_to_cells(wind), bind.output_op(orc, "edges_to_cells", wind))
        assert ok, ("edges_to_cells", err)
        u = rng.standard_normal(lay.n_vectors)
        v = u.copy()
        u_o, v_o = u.copy(), v.copy()
        g.calc_uv_at_edge(wind, u, v)
        orc.lib.orc_calc_uv_at_edge(bind.ctypes.byref(orc.g), bind._d(wind), bind._d(u_o), bind._d(v_o))
        for a, b, n in ((u, u_o, "u"), (v, v_o, "v")):
            ok, err = close(a, b)
            assert ok, ("calc_uv_at_edge", n, err)
        # the vertical entries keep what the caller had there
        for k in range(lay.nl + 1):
            assert np.array_equal(u[k * lay.vpl:k * lay.vpl + lay.nc], u_o[k * lay.vpl:k * lay.vpl + lay.nc])
        curl = rng.standard_normal(lay.n_curl)
        ok, err = close(g.curl_field_to_cells(curl), bind.output_op(orc, "curl_field_to_cells", curl))
        assert ok, ("curl_field_to_cells", err)
        a = rng.standard_normal(lay.n_vectors)
        ok, err = close(g.inner_product_tangential(a, wind), bind.output_op(orc, "inner_product_tangential", a, wind))
        assert ok, ("inner_product_tangential", err)
        g.calc_pot_vort(wind, m.state_new["rho"][lay.n_cond * lay.n_scalars:(lay.n_cond + 1) * lay.n_scalars].copy())
        pv = m.diagnostics["pot_vort"].copy()
        epv = g.epv_diagnostics(pv, m.state_new)
        epv_o = bind.epv_diagnostics(orc, pv, m_orc.state_new)
        ok, err = close(epv, epv_o)
        assert ok, ("epv_diagnostics", err)
        assert np.array_equal(m.state_new["theta_v_pert"], m_orc.state_new["theta_v_pert"])
    finally:
        g.close()


def test_output_argument_errors():
    m, wl, nw = output_scenario(3, 0, "std_wind")
    g = abi.GpuModel(m, abi.FP64)
    try:
        with pytest.raises(abi.GpuError, match="wind slots"):
            g.output_fields(m.state_new, None, 2)
        with pytest.raises(abi.GpuError, match="at least 1"):
            g.output_fields(m.state_new, wl, 0)
        with pytest.raises(abi.GpuError, match="slot"):
            g.record_wind_lowest(m.state_new, 5000)
    finally:
        g.close()
