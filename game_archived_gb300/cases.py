"""Initial states for the benchmark and test cases.

The recipe follows the reference's idealised initialisation
(src/io/set_initial_state.c:23-242): temperature and pressure fields, an
edge-normal wind projected from (u, v) with the edge direction
(set_initial_state.c:132), w = 0, and a hydrostatic balance that integrates the
Exner pressure upward with the quadratic formula including the kinetic-energy
and generalised-Coriolis terms (set_initial_state.c:155-206).  The operators
that balance needs (scalar_times_vector, calc_pot_vort, vorticity_flux,
inner_product) are taken from an ``ops`` object, so the same recipe runs on
the GPU library's C ABI, on the reference build or on the oracle.

Cases (inputs are synthetic; seeds are fixed per case):

* ``std_wind``    ICAO standard atmosphere (the reference's standard_temp /
                  standard_pres, grid_generator/src/vertical_grid.c:350-392),
                  u = 20 m/s cos(lat) + N(0, 1 m/s) on edge-normal winds, dry.
* ``std_wind_tpert``  as ``std_wind`` plus N(0, 1 K) i.i.d. temperature noise.
* ``jet_moist``   barotropic jet u = 35 m/s sin^2(2 lat) (T(z)/T_sfc) in
                  gradient-wind balance with the surface pressure, standard
                  temperature profile, N(0, 0.5 m/s) wind noise, water vapour at
                  70 % relative humidity below 8 km and none above, condensates 0.
* ``baroclinic_moist``  the baroclinic jet u = 35 m/s cos^(3/2)(eta_v) sin^2(2 lat)
                  with its thermal-wind-balanced temperature, the steady state
                  of Jablonowski and Williamson (2006, QJRMS 132, 2943-2975,
                  their eqs. 2-10), evaluated at each grid point's height by
                  solving their geopotential for the pressure; N(0, 0.5 m/s)
                  wind noise; water vapour at 70 % relative humidity below
                  8 km and none above, condensates 0.
* ``tracers``     as ``std_wind_tpert`` with every non-main constituent set to a
                  log-normal (sigma 0.5) field times exp(-z / 3 km).
"""
import numpy as np

# src/game_constants.h:10-27
T_0 = 273.15
P_0 = 100000.0
C_D_P = 1005.0
R_D = 287.057811
R_V = 461.524879
N_A = 6.02214076e23
M_D = N_A * 0.004810e-23
M_V = N_A * 0.002991e-23
OMEGA = 7.292115e-5
G_MEAN_SFC_ABS = 9.80616

CASE_SEEDS = {"std_wind": 1001, "std_wind_tpert": 1002, "jet_moist": 1003, "tracers": 1005,
              "baroclinic_moist": 1003}


def standard_temp(z):
    """grid_generator/src/vertical_grid.c:350-369"""
    t_sfc, grad, tropo, inv, grad_inv = 273.15 + 15, -0.65 / 100, 11e3, 20e3, 0.1 / 100
    tropo_temp = t_sfc + tropo * grad
    return np.where(z < tropo, t_sfc + z * grad,
                    np.where(z < inv, tropo_temp, tropo_temp + grad_inv * (z - inv)))


def standard_pres(z):
    """grid_generator/src/vertical_grid.c:371-392"""
    t_sfc, grad, tropo, inv, p0 = 273.15 + 15, -0.65 / 100, 11e3, 20e3, 101325.0
    tropo_temp = t_sfc + tropo * grad
    expo = -G_MEAN_SFC_ABS / (R_D * grad)
    p_tropo = p0 * (1 + grad * tropo / t_sfc) ** expo
    p_inv = p_tropo * np.exp(-G_MEAN_SFC_ABS * (inv - tropo) / (R_D * tropo_temp))
    return np.where(z < tropo, p0 * (1 + grad * z / t_sfc) ** expo,
                    np.where(z < inv, p_tropo * np.exp(-G_MEAN_SFC_ABS * (z - tropo) / (R_D * tropo_temp)),
                             p_inv * (1 + grad * (z - inv) / t_sfc) ** expo))


def saturation_pressure(t):
    """over water above T_0, over ice below (src/constituents/dictionary.c:281-372)"""
    tc = t - T_0
    tw = np.minimum(tc, 100.0)
    water = np.exp(34.494 - 4924.99 / (tw + 237.1)) / (tw + 105.0) ** 1.57
    ti = np.clip(tc, -80.0, 0.0)
    ice = np.exp(43.494 - 6545.8 / (ti + 278.0)) / (ti + 868.0) ** 2
    return np.where(t > T_0, water, ice)


# Jablonowski and Williamson (2006): parameters of their baroclinic steady state
JW_U0, JW_T0, JW_GAMMA, JW_DT, JW_ETA_T, JW_ETA_0, JW_P0 = 35.0, 288.0, 0.005, 4.8e5, 0.2, 0.252, 1.0e5


def _jw_terms(eta, lat, a):
    """the latitude-dependent brackets shared by their temperature and
    geopotential (eqs. 6 and 9)"""
    s, c = np.sin(lat), np.cos(lat)
    eta_v = (eta - JW_ETA_0) * np.pi / 2
    cv = np.cos(eta_v)
    b1 = -2.0 * s ** 6 * (c ** 2 + 1.0 / 3.0) + 10.0 / 63.0
    b2 = (8.0 / 5.0 * c ** 3 * (s ** 2 + 2.0 / 3.0) - np.pi / 4.0) * a * OMEGA
    return eta_v, cv, b1, b2


def jw_temperature(eta, lat, a):
    """eqs. 4-6: horizontal-mean profile plus the balanced perturbation"""
    expo = R_D * JW_GAMMA / G_MEAN_SFC_ABS
    t_mean = JW_T0 * eta ** expo + np.where(eta < JW_ETA_T, JW_DT * np.clip(JW_ETA_T - eta, 0.0, None) ** 5, 0.0)
    eta_v, cv, b1, b2 = _jw_terms(eta, lat, a)
    return t_mean + 0.75 * eta * np.pi * JW_U0 / R_D * np.sin(eta_v) * np.sqrt(cv) * (
        b1 * 2.0 * JW_U0 * cv ** 1.5 + b2)


def jw_geopotential(eta, lat, a):
    """eqs. 7-9"""
    expo = R_D * JW_GAMMA / G_MEAN_SFC_ABS
    phi_mean = JW_T0 * G_MEAN_SFC_ABS / JW_GAMMA * (1.0 - eta ** expo)
    et = JW_ETA_T
    strat = R_D * JW_DT * ((np.log(np.minimum(eta, et) / et) + 137.0 / 60.0) * et ** 5 - 5.0 * et ** 4 * eta
                           + 5.0 * et ** 3 * eta ** 2 - 10.0 / 3.0 * et ** 2 * eta ** 3 + 1.25 * et * eta ** 4
                           - 0.2 * eta ** 5)
    phi_mean = phi_mean - np.where(eta < et, strat, 0.0)
    eta_v, cv, b1, b2 = _jw_terms(eta, lat, a)
    return phi_mean + JW_U0 * cv ** 1.5 * (b1 * JW_U0 * cv ** 1.5 + b2)


def jw_eta(z, lat, a, iterations=60):
    """the pressure coordinate eta = p / p0 at height z: Newton iterations on
    Phi(eta) = g z with dPhi / d ln(eta) = -R_d T (their hydrostatic
    relation)"""
    eta = np.full(np.shape(z), 1.0)
    target = G_MEAN_SFC_ABS * np.asarray(z)
    for _ in range(iterations):
        f = jw_geopotential(eta, lat, a) - target
        eta_new = eta * np.exp(f / (R_D * jw_temperature(eta, lat, a)))
        if np.max(np.abs(eta_new / eta - 1.0)) < 1e-15:
            eta = eta_new
            break
        eta = eta_new
    return eta


def jw_wind(eta, lat):
    """eq. 2"""
    return JW_U0 * np.cos((eta - JW_ETA_0) * np.pi / 2) ** 1.5 * np.sin(2.0 * lat) ** 2


def _wind_field(layout, tables, u_of):
    """edge-normal wind in reference layout from a zonal wind u(lat, z) (v = 0)"""
    nc, ne, nl, vpl = layout.nc, layout.ne, layout.nl, layout.vpl
    wind = np.zeros(layout.n_vectors)
    lat_e = tables["latitude_vector"]
    direction = tables["direction"]
    z = tables["z_vector"]
    for l in range(nl):
        zl = z[nc + l * vpl: nc + l * vpl + ne]
        u = u_of(lat_e, zl)
        wind[nc + l * vpl: nc + l * vpl + ne] = u * np.cos(direction)
    return wind


def build_initial_state(model, tables, case, ops, seed=None):
    """Fills model.state_old / state_new (identical) and leaves diagnostics/forcings
    as the reference leaves them after initialisation.  ``ops`` provides the four
    operators on host arrays (see module docstring)."""
    lay = model.layout
    nc, ne, nl, vpl, ns = lay.nc, lay.ne, lay.nl, lay.vpl, lay.n_scalars
    rng = np.random.default_rng(CASE_SEEDS[case] if seed is None else seed)
    zs = tables["z_scalar"]
    lat_c = np.tile(tables["latitude_scalar"], nl)
    temperature = standard_temp(zs)
    pressure = standard_pres(zs)
    vapour = np.zeros(ns)
    if case in ("std_wind", "std_wind_tpert", "tracers"):
        wind = _wind_field(lay, tables, lambda lat, z: 20.0 * np.cos(lat))
        noise = 1.0
    elif case == "jet_moist":
        if not lay.moisture_on:
            raise ValueError("jet_moist needs the moist build")
        t_sfc = 288.15
        # gradient-wind balanced surface pressure for u0(lat) = 35 sin^2(2 lat)
        lat_grid = np.linspace(-np.pi / 2, np.pi / 2, 20001)
        u0 = 35.0 * np.sin(2 * lat_grid) ** 2
        a = tables.radius
        dlnp = -(a / (R_D * t_sfc)) * (2 * OMEGA * np.sin(lat_grid) * u0 + u0 ** 2 * np.tan(
            np.clip(lat_grid, -1.5, 1.5)) / a)
        lnp = np.concatenate([[0.0], np.cumsum(0.5 * (dlnp[1:] + dlnp[:-1]) * np.diff(lat_grid))])
        lnp -= np.average(lnp, weights=np.cos(lat_grid))
        pressure = pressure * np.exp(np.interp(lat_c, lat_grid, lnp))
        wind = _wind_field(lay, tables, lambda lat, z: 35.0 * np.sin(2 * lat) ** 2 * standard_temp(z) / t_sfc)
        noise = 0.5
    elif case == "baroclinic_moist":
        if not lay.moisture_on:
            raise ValueError("baroclinic_moist needs the moist build")
        a = tables.radius
        eta = jw_eta(zs, lat_c, a)
        pressure = JW_P0 * eta
        temperature = jw_temperature(eta, lat_c, a)
        wind = _wind_field(lay, tables, lambda lat, z: jw_wind(jw_eta(z, lat, a), lat))
        noise = 0.5
    else:
        raise ValueError(f"unknown case {case}")
    # seeded noise on the edge-normal winds
    for l in range(nl):
        wind[nc + l * vpl: nc + l * vpl + ne] += noise * rng.standard_normal(ne)
    if case in ("std_wind_tpert", "tracers"):
        temperature = temperature + rng.standard_normal(ns)
    temperature_v = temperature.copy()
    if case in ("jet_moist", "baroclinic_moist"):
        rh = np.where(zs < 8000.0, 0.7, 0.0)
        vapour = rh * saturation_pressure(temperature) / (R_V * temperature)
        rho_moist = pressure / (R_D * temperature)
        for _ in range(3):
            temperature_v = temperature * (1.0 + vapour / rho_moist * (M_D / M_V - 1.0))
            rho_moist = pressure / (R_D * temperature_v)
    st = model.state_old
    st["wind"] = wind
    # unbalanced moist-air density and the operators of the balance equation
    diag, forc = model.diagnostics, model.forcings
    diag["scalar_field_placeholder"] = pressure / (R_D * temperature_v)
    ops.scalar_times_vector(diag["scalar_field_placeholder"], st["wind"], diag["flux_density"])
    ops.calc_pot_vort(st["wind"], diag["scalar_field_placeholder"])
    ops.vorticity_flux(diag["flux_density"], diag["pot_vort"], forc["pot_vort_tend"])
    ops.inner_product(st["wind"], st["wind"], diag["v_squared"])
    v2 = diag["v_squared"].copy()
    pvt = forc["pot_vort_tend"]
    gp = tables["gravity_potential"]
    exner = np.zeros(ns)
    theta_v = np.zeros(ns)
    rho = np.zeros(ns)
    for l in range(nl - 1, -1, -1):
        s = slice(l * nc, (l + 1) * nc)
        if l == nl - 1:
            exner[s] = (pressure[s] / P_0) ** (R_D / C_D_P)
        else:
            b_ = slice((l + 1) * nc, (l + 2) * nc)
            b = -0.5 * exner[b_] / temperature_v[b_] * (
                temperature_v[s] - temperature_v[b_] + 2.0 / C_D_P * (
                    gp[s] - gp[b_] + 0.5 * v2[s] - 0.5 * v2[b_]
                    - (zs[s] - zs[b_]) * pvt[(l + 1) * vpl: (l + 1) * vpl + nc]))
            c = exner[b_] ** 2 * temperature_v[s] / temperature_v[b_]
            exner[s] = b + np.sqrt(b ** 2 + c)
        theta_v[s] = temperature_v[s] / exner[s]
        rho[s] = P_0 * exner[s] ** (C_D_P / R_D) / (R_D * temperature_v[s])
    rhotheta = rho * theta_v
    g = model.grid
    st["exner_pert"] = exner - g["exner_bg"]
    st["theta_v_pert"] = theta_v - g["theta_v_bg"]
    st["rhotheta_v"] = rhotheta
    r = st["rho"]
    r[:] = 0.0
    cond = lay.n_cond
    r[cond * ns:(cond + 1) * ns] = rho
    if lay.moisture_on:
        r[(cond + 1) * ns:(cond + 2) * ns] = vapour
    if case == "tracers":
        for k in range(lay.n_const):
            if k == cond:
                continue
            f = np.exp(0.5 * rng.standard_normal(ns)) * np.exp(-zs / 3000.0) * 1e-3
            r[k * ns:(k + 1) * ns] = f
    model.state_new.copy_from(model.state_old)
    return model


def default_config(model, first_step=True):
    """The run configuration of every benchmark case: radiation, diffusion,
    PBL, soil and surface fluxes off; the reference's hard-wired constants
    (src/coordinator.c:54-57, 221-223)."""
    c = model.config
    c.buf[...] = 0
    c["totally_first_step_bool"] = 1 if first_step else 0
    c["impl_thermo_weight"] = 0.75
    c["damping_start_height_over_toa"] = 0.53
    c["damping_coeff_max"] = 0.25
    c["cloud_droplets_velocity"] = 0.01
    c["rain_velocity"] = 10.0
    c["snow_velocity"] = 5.0
    c["radiation_delta_t"] = 3600.0
    return c
