"""ctypes binding of the oracle (test infrastructure only).

Builds the oracle's field-pointer structs from host structs laid out as the
reference's (game_archived_gb300.structs.Model), and exposes the oracle
operators and step with the reference's argument meaning.
"""
import ctypes

import numpy as np

from . import build_oracle

_lib = None
P = ctypes.POINTER
dp = P(ctypes.c_double)
ip = P(ctypes.c_int)


DIAG_FIELDS = ("flux_density", "flux_density_divv", "rel_vort_on_triangles", "rel_vort", "pot_vort", "temperature",
               "v_squared", "scalar_field_placeholder", "wind_divv", "curl_of_vorticity", "vector_field_placeholder",
               "n_squared", "dv_hdz", "u_at_edge", "v_at_edge", "u_at_cell", "v_at_cell", "monin_obukhov_length",
               "roughness_velocity")
IRREV_FIELDS = ("temperature_diffusion_heating", "friction_acc", "heating_diss", "pressure_gradient_decel_factor",
                "condensates_sediment_heat", "mass_diff_tendency", "phase_trans_rates", "phase_trans_heating_rate",
                "molecular_diffusion_coeff", "mass_diffusion_coeff_numerical_h", "mass_diffusion_coeff_numerical_v",
                "temp_diffusion_coeff_numerical_h", "temp_diffusion_coeff_numerical_v", "viscosity", "viscosity_rhombi",
                "viscosity_triangles", "vert_hor_viscosity", "tke")


class OrcGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nc", "ne", "nt", "nl", "n_oro", "moisture_on", "n_const", "n_cond")] + [
        ("radius", ctypes.c_double)] + [(n, dp) for n in (
            "normal_distance", "volume", "area", "z_scalar", "z_vector", "gravity_m", "slope", "theta_v_bg",
            "exner_bg", "exner_bg_grad", "ipw", "trsk_weights", "rhombi_weights")] + [(n, ip) for n in (
                "trsk_indices", "trsk_mci", "from_", "to", "adj", "adj_sign", "rhombi_idx", "is_land")] + [
        (n, dp) for n in ("dual_area", "dual_z_vector", "f_vec")] + [
        (n, ip) for n in ("dual_from", "dual_to", "vort_idx", "vort_sign")] + [("gravity_potential", dp)] + [
        (n, dp) for n in ("layer_thickness", "dual_normal_distance")] + [
        (n, ctypes.c_double) for n in ("eff_hor_res", "mean_velocity_area")] + [("latitude_scalar", dp)] + [
        (n, dp) for n in ("direction", "roughness_length", "sfc_albedo", "latlon_weights")] + [
        ("latlon_indices", ip), ("n_latlon", ctypes.c_long)]

# the fields of orc_output, in its order: surface [Nc], model layers [S],
# pressure levels [Nc][6]
OUTPUT_SURFACE = ("mslp", "surface_p", "t2", "tcdc", "rprate", "sprate", "cape", "sfc_sw_down", "u10", "v10", "gusts")
OUTPUT_LAYERS = ("pressure", "rh", "rel_vort", "divv_h", "epv")
OUTPUT_PLEVELS = ("geopotential_height", "t_pl", "rh_pl", "epv_pl", "u_pl", "v_pl", "rel_vort_pl")
N_PRESSURE_LEVELS = 6


class OrcOutput(ctypes.Structure):
    _fields_ = [(n, dp) for n in OUTPUT_SURFACE + OUTPUT_LAYERS + OUTPUT_PLEVELS]


class OrcState(ctypes.Structure):
    _fields_ = [(n, dp) for n in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")]


class OrcDiag(ctypes.Structure):
    _fields_ = [(n, dp) for n in DIAG_FIELDS]


class OrcForcings(ctypes.Structure):
    _fields_ = [(n, dp) for n in ("pgrad_acc_old", "pgrad_nl", "pgrad_l", "pgrad_condensates_v",
                                  "v_squared_grad", "pot_vort_tend", "radiation_tendency", "sfc_sw_in",
                                  "sfc_lw_out")]


class OrcIrrev(ctypes.Structure):
    _fields_ = [(n, dp) for n in IRREV_FIELDS]


class OrcConfig(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "totally_first_step_bool", "temperature_diff_h", "temperature_diff_v", "momentum_diff_h",
        "momentum_diff_v", "mass_diff_h", "mass_diff_v", "rad_on", "prog_soil_temp", "sfc_phase_trans",
        "sfc_sensible_heat_flux", "rad_update", "time_to_next_analysis", "pbl_scheme", "total_run_span")] + [
        (n, ctypes.c_double) for n in ("damping_start_height_over_toa", "damping_coeff_max",
                                       "impl_thermo_weight", "cloud_droplets_velocity", "rain_velocity",
                                       "snow_velocity", "radiation_delta_t")]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        vp = ctypes.c_void_p
        for name in ("orc_manage_rkhevi",):
            getattr(_lib, name).argtypes = [vp] * 8 + [ctypes.c_double, ctypes.c_double]
        _lib.orc_global_scalar_integrator.restype = ctypes.c_double
        _lib.orc_global_scalar_integrator.argtypes = [vp, vp]
    return _lib


def _d(a):
    return a.ctypes.data_as(dp)


def _i(a):
    return a.ctypes.data_as(ip)


class Oracle:
    """The oracle bound to one Model (host structs in the reference layout)."""

    def __init__(self, model):
        self.m = model
        lay = model.layout
        g, dg = model.grid, model.dualgrid
        self.g = OrcGrid(lay.nc, lay.ne, lay.nt, lay.nl, int(g["no_of_oro_layers"][0]), lay.moisture_on,
                         lay.n_const, lay.n_cond, float(g["radius"][0]),
                         _d(g["normal_distance"]), _d(g["volume"]), _d(g["area"]), _d(g["z_scalar"]),
                         _d(g["z_vector"]), _d(g["gravity_m"]), _d(g["slope"]), _d(g["theta_v_bg"]),
                         _d(g["exner_bg"]), _d(g["exner_bg_grad"]), _d(g["inner_product_weights"]),
                         _d(g["trsk_weights"]), _d(g["density_to_rhombi_weights"]), _i(g["trsk_indices"]),
                         _i(g["trsk_modified_curl_indices"]), _i(g["from_index"]), _i(g["to_index"]),
                         _i(g["adjacent_vector_indices_h"]), _i(g["adjacent_signs_h"]),
                         _i(g["density_to_rhombi_indices"]), _i(g["is_land"]), _d(dg["area"]), _d(dg["z_vector"]),
                         _d(dg["f_vec"]), _i(dg["from_index"]), _i(dg["to_index"]),
                         _i(dg["vorticity_indices_triangles"]), _i(dg["vorticity_signs_triangles"]),
                         _d(g["gravity_potential"]), _d(g["layer_thickness"]), _d(dg["normal_distance"]),
                         float(g["eff_hor_res"][0]), float(g["mean_velocity_area"][0]), _d(g["latitude_scalar"]),
                         _d(g["direction"]), _d(g["roughness_length"]), _d(g["sfc_albedo"]),
                         _d(g["latlon_interpol_weights"]), _i(g["latlon_interpol_indices"]), lay.n_latlon)
        self.lib = lib()

    def state(self, s):
        return OrcState(_d(s["rho"]), _d(s["rhotheta_v"]), _d(s["theta_v_pert"]), _d(s["exner_pert"]), _d(s["wind"]))

    def diag(self):
        d = self.m.diagnostics
        return OrcDiag(*[_d(d[n]) for n in DIAG_FIELDS])

    def forcings(self):
        f = self.m.forcings
        return OrcForcings(*[_d(f[n]) for n in ("pgrad_acc_old", "pressure_gradient_acc_neg_nl",
                                                "pressure_gradient_acc_neg_l", "pressure_grad_condensates_v",
                                                "v_squared_grad", "pot_vort_tend", "radiation_tendency",
                                                "sfc_sw_in", "sfc_lw_out")])

    def irrev(self):
        r = self.m.irrev
        return OrcIrrev(*[_d(r[n]) for n in IRREV_FIELDS])

    def config(self):
        c = self.m.config
        ints = [int(c[n][0]) for n, t in OrcConfig._fields_ if t is ctypes.c_int]
        dbls = [float(c[n][0]) for n, t in OrcConfig._fields_ if t is ctypes.c_double]
        return OrcConfig(*(ints + dbls))

    # ---- operators on host arrays (reference argument meaning)
    def scalar_times_vector(self, s, v, out):
        self.lib.orc_scalar_times_vector(ctypes.byref(self.g), _d(s), _d(v), _d(out))

    def calc_pot_vort(self, wind, rho):
        d = self.diag()
        self.lib.orc_calc_pot_vort(ctypes.byref(self.g), _d(wind), _d(rho), ctypes.byref(d))

    def vorticity_flux(self, flux, pv, out):
        self.lib.orc_vorticity_flux(ctypes.byref(self.g), _d(flux), _d(pv), _d(out))

    def inner_product(self, a, b, out):
        self.lib.orc_inner_product(ctypes.byref(self.g), _d(a), _d(b), _d(out))

    def grad(self, s, out):
        self.lib.orc_grad(ctypes.byref(self.g), _d(s), _d(out))

    def divv_h(self, v, out):
        self.lib.orc_divv_h(ctypes.byref(self.g), _d(v), _d(out))

    def linear_combine_two_states(self, s0, s1, out, c0, c1):
        a, b, o = self.state(s0), self.state(s1), self.state(out)
        self.lib.orc_linear_combine_two_states(ctypes.byref(self.g), ctypes.byref(a), ctypes.byref(b),
                                               ctypes.byref(o), ctypes.c_double(c0), ctypes.c_double(c1))

    # ---- the sub-steps of manage_rkhevi (reference argument meaning)
    def step_prelude(self, state, dt):
        """temperature diagnostics and phase-transition rates of a State, as
        manage_rkhevi computes them first (manage_rkhevi.c:29-41)"""
        m = self.m
        s, d, r, c = self.state(state), self.diag(), self.irrev(), self.config()
        self.lib.orc_temperature_diagnostics(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(d))
        if m.layout.moisture_on:
            self.lib.orc_calc_h2otracers_source_rates(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(d),
                                                      ctypes.byref(c), ctypes.byref(r), ctypes.c_double(dt))

    def manage_pressure_gradient(self, state):
        s, d, f, r, c = self.state(state), self.diag(), self.forcings(), self.irrev(), self.config()
        self.lib.orc_manage_pressure_gradient(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(d), ctypes.byref(f),
                                              ctypes.byref(r), ctypes.byref(c))

    def calc_pressure_grad_condensates_v(self, state):
        s, f, r = self.state(state), self.forcings(), self.irrev()
        self.lib.orc_calc_pressure_grad_condensates_v(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(f),
                                                      ctypes.byref(r))

    def vector_tendencies_expl(self, state, tend, rk, dt):
        s, t, d, f, r, c = (self.state(state), self.state(tend), self.diag(), self.forcings(), self.irrev(),
                            self.config())
        self.lib.orc_vector_tendencies_expl(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(t), ctypes.byref(d),
                                            ctypes.byref(f), ctypes.byref(r), ctypes.byref(c), int(rk),
                                            ctypes.c_double(dt))

    def scalar_tendencies_expl(self, s_old, s_new, tend, dt, rk):
        so, sn, t = self.state(s_old), self.state(s_new), self.state(tend)
        d, f, r, c = self.diag(), self.forcings(), self.irrev(), self.config()
        rc = self.lib.orc_scalar_tendencies_expl(ctypes.byref(self.g), ctypes.byref(so), ctypes.byref(sn),
                                                 ctypes.byref(t), ctypes.c_double(dt), ctypes.byref(d),
                                                 ctypes.byref(f), ctypes.byref(r), ctypes.byref(c), int(rk))
        if rc != 0:
            raise RuntimeError(f"oracle scalar_tendencies_expl returned {rc}")

    def three_band_solver_ver_waves(self, s_old, s_new, tend, dt, rk):
        so, sn, t, c = self.state(s_old), self.state(s_new), self.state(tend), self.config()
        rc = self.lib.orc_three_band_solver_ver_waves(ctypes.byref(self.g), ctypes.byref(so), ctypes.byref(sn),
                                                      ctypes.byref(t), ctypes.byref(c), ctypes.c_double(dt), int(rk))
        if rc != 0:
            raise RuntimeError(f"oracle three_band_solver_ver_waves returned {rc}")

    def three_band_solver_gen_densities(self, s_old, s_new, tend, dt, rk):
        so, sn, t = self.state(s_old), self.state(s_new), self.state(tend)
        d, r, c = self.diag(), self.irrev(), self.config()
        self.lib.orc_three_band_solver_gen_densities(ctypes.byref(self.g), ctypes.byref(so), ctypes.byref(sn),
                                                     ctypes.byref(t), ctypes.byref(d), ctypes.byref(r),
                                                     ctypes.byref(c), ctypes.c_double(dt), int(rk))

    def manage_rkhevi(self, dt, t=0.0):
        m = self.m
        so, sn, st = self.state(m.state_old), self.state(m.state_new), self.state(m.state_tendency)
        d, f, r, c = self.diag(), self.forcings(), self.irrev(), self.config()
        rc = self.lib.orc_manage_rkhevi(ctypes.byref(self.g), ctypes.byref(so), ctypes.byref(sn), ctypes.byref(st),
                                        ctypes.byref(d), ctypes.byref(f), ctypes.byref(r), ctypes.byref(c),
                                        ctypes.c_double(dt), ctypes.c_double(t))
        if rc != 0:
            raise RuntimeError(f"oracle manage_rkhevi returned {rc}")

    def surface_pressure(self, state, temperature, with_mslp=False):
        out = np.zeros(self.m.layout.nc)
        ms = np.zeros(self.m.layout.nc) if with_mslp else None
        s = self.state(state)
        self.lib.orc_surface_pressure(ctypes.byref(self.g), ctypes.byref(s), _d(temperature), _d(out),
                                      _d(ms) if with_mslp else None)
        return (out, ms) if with_mslp else out

    def temperature(self, state):
        """temperature_diagnostics of a State (derived_quantities.c:15-40)"""
        t = np.zeros(self.m.layout.n_scalars)
        d = OrcDiag()
        d.temperature = _d(t)
        s = self.state(state)
        self.lib.orc_temperature_diagnostics(ctypes.byref(self.g), ctypes.byref(s), ctypes.byref(d))
        return t

    def integral(self, field):
        return self.lib.orc_global_scalar_integrator(ctypes.byref(self.g), _d(field))

    def write_out_integral(self, state, integral_id, temperature):
        """the numbers write_out_integral (src/io/write_output.c:1515-1596)
        writes: serial sums as in the reference"""
        lay = self.m.layout
        ns = lay.n_scalars
        rho = state["rho"]
        if integral_id == 0:
            return np.array([self.integral(np.ascontiguousarray(rho[k * ns:(k + 1) * ns]))
                             for k in range(lay.n_const)])
        if integral_id == 1:
            return np.array([self.integral(np.ascontiguousarray(state["rhotheta_v"]))])
        rho_g = np.ascontiguousarray(rho[lay.n_cond * ns:(lay.n_cond + 1) * ns])
        ekin = np.zeros(ns)
        self.inner_product(state["wind"], state["wind"], ekin)
        ekin = rho_g * ekin
        pot = rho_g * self.m.grid["gravity_potential"]
        internal = rho_g * temperature
        return np.array([0.5 * self.integral(ekin), self.integral(pot), 717.942189 * self.integral(internal)])


def _output_arrays(lay):
    out = {n: np.zeros(lay.nc) for n in OUTPUT_SURFACE}
    out.update({n: np.zeros(lay.n_scalars) for n in OUTPUT_LAYERS})
    out.update({n: np.zeros(lay.nc * N_PRESSURE_LEVELS) for n in OUTPUT_PLEVELS})
    return out


def write_out_fields(orc, state, wind_lowest, n_wind_steps):
    """the fields write_out (src/io/write_output.c:51-1513) computes from
    state, as a dict of arrays (surface [Nc], model layers [S], pressure
    levels [Nc][6]); also writes the Diagnostics members write_out writes
    and rounds the top layer of state's theta_v_pert as the reference does"""
    m = orc.m
    lay = m.layout
    out = _output_arrays(lay)
    o = OrcOutput(*[_d(out[n]) for n, _ in OrcOutput._fields_])
    s = orc.state(state)
    d = orc.diag()
    c = orc.config()
    wl = np.ascontiguousarray(wind_lowest, dtype=np.float64)
    rc = orc.lib.orc_write_out_fields(ctypes.byref(orc.g), ctypes.byref(s), _d(state["temperature_soil"]), _d(wl),
                                      ctypes.c_int(n_wind_steps), ctypes.byref(d), _d(m.forcings["sfc_sw_in"]),
                                      ctypes.byref(c), ctypes.byref(o))
    if rc != 0:
        raise RuntimeError("oracle write_out_fields failed")
    return out


def interpolate_to_ll(orc, field):
    """interpolate_to_ll (src/io/spatial_ops_for_output.c:168-197)"""
    f = np.ascontiguousarray(field, dtype=np.float64)
    out = np.zeros(orc.m.layout.n_latlon)
    orc.lib.orc_interpolate_to_ll(ctypes.byref(orc.g), _d(f), _d(out))
    return out


def output_op(orc, name, *arrays, out_len=None, extra_out=None):
    """calls one of the oracle's output operators (orc_calc_uv_at_edge,
    orc_curl_field_to_cells, orc_edges_to_cells, orc_edges_to_cells_lowest_layer,
    orc_inner_product_tangential) on host arrays; returns the output array"""
    lay = orc.m.layout
    out = np.zeros(out_len if out_len is not None else lay.n_scalars)
    args = [_d(np.ascontiguousarray(a, dtype=np.float64)) for a in arrays] + [_d(out)]
    getattr(orc.lib, "orc_" + name)(ctypes.byref(orc.g), *args)
    return out


def epv_diagnostics(orc, pot_vort, state):
    """orc_epv_diagnostics; rounds state's theta_v_pert top layer in place"""
    out = np.zeros(orc.m.layout.n_scalars)
    s = orc.state(state)
    rc = orc.lib.orc_epv_diagnostics(ctypes.byref(orc.g), _d(np.ascontiguousarray(pot_vort)), ctypes.byref(s), _d(out))
    if rc != 0:
        raise RuntimeError("oracle epv_diagnostics failed")
    return out
