"""ctypes declarations of include/game_gb300.h and a thin host-side wrapper.

``GpuModel`` binds the C library to one ``structs.Model`` (host structs in the
reference layout) and exposes the reference's calls with the reference's
argument meaning, so tests and the benchmark drive the library exactly as the
reference's own driver (src/coordinator.c) would.
"""
import ctypes

from . import native

vp, dbl, cint = ctypes.c_void_p, ctypes.c_double, ctypes.c_int

SIGNATURES = {
    "game_gpu_init": ([cint, cint, cint, vp, vp], cint),
    "game_gpu_finalize": ([], cint),
    "game_gpu_set_precision": ([cint], cint),
    "game_gpu_set_resident": ([cint], cint),
    "game_gpu_set_graphs": ([cint], cint),
    "game_gpu_set_column_solver": ([cint], cint),
    "game_gpu_set_double_float": ([cint], cint),
    "game_gpu_set_checkpoint_stride": ([cint], cint),
    "game_gpu_sync_to_device": ([vp], cint),
    "game_gpu_sync_to_host": ([vp], cint),
    "game_gpu_sync_aux_to_host": ([vp, vp, vp], cint),
    "game_gpu_synchronize": ([], cint),
    "game_gpu_last_error": ([], ctypes.c_char_p),
    "game_gpu_host_alloc": ([ctypes.POINTER(vp), ctypes.c_size_t], cint),
    "game_gpu_host_free": ([vp], cint),
    "game_gpu_kernel_launches": ([cint], ctypes.c_longlong),
    "game_gpu_set_device": ([cint], cint),
    "game_gpu_event_record": ([cint], cint),
    "game_gpu_event_elapsed": ([cint, cint, ctypes.POINTER(ctypes.c_float)], cint),
    "game_gpu_profile": ([cint], cint),
    "game_gpu_profile_count": ([], cint),
    "game_gpu_profile_get": ([cint, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_longlong)], cint),
    "game_gpu_transfer_bytes": ([ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), cint], cint),
    "manage_rkhevi": ([vp] * 9 + [dbl, dbl], cint),
    "linear_combine_two_states": ([vp, vp, vp, dbl, dbl, vp], cint),
    "manage_pressure_gradient": ([vp] * 7, cint),
    "calc_pressure_grad_condensates_v": ([vp] * 4, cint),
    "vector_tendencies_expl": ([vp] * 8 + [cint, dbl], cint),
    "scalar_tendencies_expl": ([vp] * 5 + [dbl] + [vp] * 4 + [cint], cint),
    "three_band_solver_ver_waves": ([vp] * 6 + [dbl, vp, cint], cint),
    "three_band_solver_gen_densities": ([vp] * 6 + [dbl, cint, vp], cint),
    "grad_hor_cov": ([vp] * 3, cint),
    "grad_vert_cov": ([vp] * 3, cint),
    "vector_field_hor_cov_to_con": ([vp] * 2, cint),
    "grad_cov": ([vp] * 3, cint),
    "grad": ([vp] * 3, cint),
    "grad_hor": ([vp] * 3, cint),
    "calc_pot_vort": ([vp] * 5, cint),
    "add_f_to_rel_vort": ([vp] * 3, cint),
    "calc_rel_vort": ([vp] * 4, cint),
    "vorticity_flux": ([vp] * 5, cint),
    "divv_h": ([vp] * 3, cint),
    "divv_h_tracer": ([vp] * 5, cint),
    "scalar_times_vector": ([vp] * 4, cint),
    "scalar_times_vector_h": ([vp] * 4, cint),
    "scalar_times_vector_h_upstream": ([vp] * 4, cint),
    "scalar_times_vector_v": ([vp] * 4, cint),
    "inner_product": ([vp] * 4, cint),
    "scalar_times_scalar": ([vp] * 3, cint),
    "vector_times_vector": ([vp] * 3, cint),
    "add_vertical_divv": ([vp] * 3, cint),
    "global_scalar_integrator": ([vp, vp], dbl),
    "game_gpu_write_out_integral": ([vp, cint, vp], cint),
    "game_gpu_surface_pressure": ([vp, vp, vp], cint),
    "game_gpu_weighted_sums_noalloc": ([vp, cint, ctypes.c_longlong, vp, vp, vp], cint),
    "game_gpu_numerics": ([cint, vp, vp, ctypes.c_longlong], cint),
    "game_gpu_check_state": ([vp, vp], cint),
    "game_gpu_set_health_check": ([cint], cint),
    "game_gpu_write_checkpoint": ([ctypes.c_char_p, vp, vp, vp, vp, vp], cint),
    "game_gpu_read_checkpoint": ([ctypes.c_char_p, vp, vp, vp, vp, vp], cint),
    "grad_adj": ([vp] * 3, cint),
    "divv_h_adj": ([vp] * 3, cint),
    "divv_h_tracer_adj": ([vp] * 8, cint),
    "manage_rkhevi_adj": ([vp] * 9 + [dbl, dbl, vp, vp], cint),
    "three_band_solver_gen_densities_adj": ([vp] * 6 + [dbl, cint] + [vp] * 6, cint),
    "scalar_times_vector_adj": ([vp] * 6, cint),
    "inner_product_adj": ([vp] * 6, cint),
    "calc_pot_vort_adj": ([vp] * 7, cint),
    "vorticity_flux_adj": ([vp] * 7, cint),
    "three_band_solver_ver_waves_adj": ([vp] * 6 + [dbl, vp, cint, vp, vp, vp], cint),
    "rkhevi_window_forward": ([vp] * 8 + [dbl, cint], cint),
    "rkhevi_window_tl": ([vp, vp], cint),
    "rkhevi_window_backward": ([vp, vp], cint),
    "game_gpu_sfc_pressure_objective": ([vp, vp, ctypes.POINTER(ctypes.c_double), vp], cint),
    "interpolate_to_ll": ([vp] * 3, cint),
    "edges_to_cells_lowest_layer": ([vp] * 3, cint),
    "epv_diagnostics": ([vp] * 5, cint),
    "inner_product_tangential": ([vp] * 5, cint),
    "calc_uv_at_edge": ([vp] * 4, cint),
    "curl_field_to_cells": ([vp] * 3, cint),
    "edges_to_cells": ([vp] * 3, cint),
    "game_gpu_write_out_fields": ([vp, vp, cint, vp, vp, vp, vp, vp, vp], cint),
    "game_gpu_record_wind_lowest": ([vp, cint], cint),
    "write_out": ([vp, vp, cint, dbl, dbl, vp, vp, vp, vp, vp, vp, vp], cint),
    "write_out_integral": ([vp, dbl, vp, vp, vp, cint], cint),
    "interpolation_t": ([vp, vp, vp, dbl, dbl, dbl, vp], cint),
}

# struct game_gpu_output_fields (include/game_gb300.h), in declaration order,
# with each field's kind: 0 surface, 1 model layers, 2 pressure levels,
# 3 vertical wind at the levels (lat-lon only)
OUTPUT_FIELDS = (("mslp", 0), ("surface_p", 0), ("t2", 0), ("tcdc", 0), ("rprate", 0), ("sprate", 0), ("cape", 0),
                 ("sfc_sw_down", 0), ("u10", 0), ("v10", 0), ("gusts", 0), ("temperature", 1), ("pressure", 1),
                 ("rh", 1), ("u", 1), ("v", 1), ("rel_vort", 1), ("divv_h", 1), ("epv", 1),
                 ("geopotential_height", 2), ("t_pl", 2), ("rh_pl", 2), ("epv_pl", 2), ("u_pl", 2), ("v_pl", 2),
                 ("rel_vort_pl", 2), ("w", 3))
N_PRESSURE_LEVELS = 6


class OutputFields(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(dbl)) for n, _ in OUTPUT_FIELDS]

FP64, MIXED = 0, 1
UNHEALTHY = 2


class Health(ctypes.Structure):
    """struct game_gpu_health (include/game_gb300.h)"""
    _fields_ = [(n, ctypes.c_longlong) for n in ("nonfinite", "negative_density", "first_nonfinite",
                                                 "first_negative_density")]


def declare(lib):
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class GpuError(RuntimeError):
    pass


class GpuModel:
    """The CUDA library bound to a Model."""

    def __init__(self, model, precision=FP64, resident=False, graphs=True, device=None, column_solver=0,
                 double_float=1):
        self.lib = native.gpu()
        self.m = model
        lay = model.layout
        if device is not None:
            self._check(self.lib.game_gpu_set_device(device), "game_gpu_set_device")
        self._check(self.lib.game_gpu_init(lay.res_id, lay.n_layers, lay.moisture_on, model.grid.ptr,
                                           model.dualgrid.ptr), "game_gpu_init")
        try:
            self._check(self.lib.game_gpu_set_precision(precision), "set_precision")
            self._check(self.lib.game_gpu_set_resident(1 if resident else 0), "set_resident")
            self._check(self.lib.game_gpu_set_graphs(1 if graphs else 0), "set_graphs")
            self._check(self.lib.game_gpu_set_column_solver(column_solver), "set_column_solver")
            self._check(self.lib.game_gpu_set_double_float(double_float), "set_double_float")
        except GpuError:
            self.lib.game_gpu_finalize()
            raise
        self.resident = resident

    def _check(self, rc, what):
        if rc != 0:
            raise GpuError(f"{what}: {self.lib.game_gpu_last_error().decode()}")

    def close(self):
        self.lib.game_gpu_finalize()

    # -- the reference's calls
    def manage_rkhevi(self, dt, t=0.0):
        m = self.m
        self._check(self.lib.manage_rkhevi(m.state_old.ptr, m.state_new.ptr, m.grid.ptr, m.dualgrid.ptr,
                                           m.state_tendency.ptr, m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr,
                                           m.config.ptr, dt, t), "manage_rkhevi")

    def linear_combine_two_states(self, s0, s1, out, c0, c1):
        self._check(self.lib.linear_combine_two_states(s0.ptr, s1.ptr, out.ptr, c0, c1, self.m.grid.ptr),
                    "linear_combine_two_states")

    # -- the sub-steps of manage_rkhevi (reference argument order)
    def manage_pressure_gradient(self, state):
        m = self.m
        self._check(self.lib.manage_pressure_gradient(state.ptr, m.grid.ptr, m.dualgrid.ptr, m.diagnostics.ptr,
                                                      m.forcings.ptr, m.irrev.ptr, m.config.ptr),
                    "manage_pressure_gradient")

    def calc_pressure_grad_condensates_v(self, state):
        m = self.m
        self._check(self.lib.calc_pressure_grad_condensates_v(state.ptr, m.grid.ptr, m.forcings.ptr, m.irrev.ptr),
                    "calc_pressure_grad_condensates_v")

    def vector_tendencies_expl(self, state, tend, rk, dt):
        m = self.m
        self._check(self.lib.vector_tendencies_expl(state.ptr, tend.ptr, m.grid.ptr, m.dualgrid.ptr, m.diagnostics.ptr,
                                                    m.forcings.ptr, m.irrev.ptr, m.config.ptr, rk, dt),
                    "vector_tendencies_expl")

    def scalar_tendencies_expl(self, s_old, s_new, tend, dt, rk):
        m = self.m
        self._check(self.lib.scalar_tendencies_expl(s_old.ptr, s_new.ptr, tend.ptr, m.grid.ptr, m.dualgrid.ptr, dt,
                                                    m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr, m.config.ptr, rk),
                    "scalar_tendencies_expl")

    def three_band_solver_ver_waves(self, s_old, s_new, tend, dt, rk):
        m = self.m
        self._check(self.lib.three_band_solver_ver_waves(s_old.ptr, s_new.ptr, tend.ptr, m.diagnostics.ptr,
                                                         m.forcings.ptr, m.config.ptr, dt, m.grid.ptr, rk),
                    "three_band_solver_ver_waves")

    def three_band_solver_gen_densities(self, s_old, s_new, tend, dt, rk):
        m = self.m
        self._check(self.lib.three_band_solver_gen_densities(s_old.ptr, s_new.ptr, tend.ptr, m.diagnostics.ptr,
                                                             m.irrev.ptr, m.config.ptr, dt, rk, m.grid.ptr),
                    "three_band_solver_gen_densities")

    def sync_to_device(self, s):
        self._check(self.lib.game_gpu_sync_to_device(s.ptr), "sync_to_device")

    def sync_to_host(self, s):
        self._check(self.lib.game_gpu_sync_to_host(s.ptr), "sync_to_host")

    def sync_aux_to_host(self):
        m = self.m
        self._check(self.lib.game_gpu_sync_aux_to_host(m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr), "sync_aux")

    def synchronize(self):
        self._check(self.lib.game_gpu_synchronize(), "synchronize")

    # -- health check and checkpoints
    def check_state(self, s):
        """(status, report): status 0 healthy, UNHEALTHY (2) otherwise"""
        r = Health()
        rc = self.lib.game_gpu_check_state(s.ptr, ctypes.byref(r))
        if rc not in (0, UNHEALTHY):
            raise GpuError(f"check_state: {self.lib.game_gpu_last_error().decode()}")
        return rc, {k: getattr(r, k) for k, _ in Health._fields_}

    def set_health_check(self, every):
        self._check(self.lib.game_gpu_set_health_check(every), "set_health_check")

    def write_checkpoint(self, path, state):
        m = self.m
        self._check(self.lib.game_gpu_write_checkpoint(str(path).encode(), state.ptr, m.diagnostics.ptr,
                                                       m.forcings.ptr, m.irrev.ptr, m.config.ptr), "write_checkpoint")

    def read_checkpoint(self, path, state):
        m = self.m
        self._check(self.lib.game_gpu_read_checkpoint(str(path).encode(), state.ptr, m.diagnostics.ptr,
                                                      m.forcings.ptr, m.irrev.ptr, m.config.ptr), "read_checkpoint")

    def kernel_launches(self, reset=False):
        return int(self.lib.game_gpu_kernel_launches(1 if reset else 0))

    def event_record(self, slot):
        self._check(self.lib.game_gpu_event_record(slot), "event_record")

    def event_elapsed_ms(self, a, b):
        ms = ctypes.c_float()
        self._check(self.lib.game_gpu_event_elapsed(a, b, ctypes.byref(ms)), "event_elapsed")
        return float(ms.value)

    def profile(self, on):
        self._check(self.lib.game_gpu_profile(1 if on else 0), "profile")

    def profile_results(self):
        out = {}
        name, ms, n = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_longlong()
        for i in range(self.lib.game_gpu_profile_count()):
            self._check(self.lib.game_gpu_profile_get(i, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(n)),
                        "profile_get")
            out[name.value.decode()] = (ms.value, n.value)
        return out

    def transfer_bytes(self, reset=False):
        h, d = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(self.lib.game_gpu_transfer_bytes(ctypes.byref(h), ctypes.byref(d), 1 if reset else 0),
                    "transfer_bytes")
        return h.value, d.value

    # -- single operators on host arrays
    def grad(self, s, out):
        self._check(self.lib.grad(_p(s), _p(out), self.m.grid.ptr), "grad")

    def divv_h(self, v, out):
        self._check(self.lib.divv_h(_p(v), _p(out), self.m.grid.ptr), "divv_h")

    def divv_h_tracer(self, v, dens, wind, out):
        self._check(self.lib.divv_h_tracer(_p(v), _p(dens), _p(wind), _p(out), self.m.grid.ptr), "divv_h_tracer")

    def scalar_times_vector(self, s, v, out, variant=""):
        f = getattr(self.lib, "scalar_times_vector" + variant)
        self._check(f(_p(s), _p(v), _p(out), self.m.grid.ptr), "scalar_times_vector" + variant)

    def inner_product(self, a, b, out):
        self._check(self.lib.inner_product(_p(a), _p(b), _p(out), self.m.grid.ptr), "inner_product")

    def calc_pot_vort(self, wind, rho):
        m = self.m
        self._check(self.lib.calc_pot_vort(_p(wind), _p(rho), m.diagnostics.ptr, m.grid.ptr, m.dualgrid.ptr),
                    "calc_pot_vort")

    def vorticity_flux(self, flux, pv, out):
        m = self.m
        self._check(self.lib.vorticity_flux(_p(flux), _p(pv), _p(out), m.grid.ptr, m.dualgrid.ptr), "vorticity_flux")

    # -- operator adjoints (bars of inputs accumulated)
    def grad_adj(self, out_bar, in_bar):
        self._check(self.lib.grad_adj(_p(out_bar), _p(in_bar), self.m.grid.ptr), "grad_adj")

    def divv_h_adj(self, out_bar, in_bar):
        self._check(self.lib.divv_h_adj(_p(out_bar), _p(in_bar), self.m.grid.ptr), "divv_h_adj")

    def divv_h_tracer_adj(self, v, dens, wind, out_bar, v_bar, dens_bar, wind_bar):
        self._check(self.lib.divv_h_tracer_adj(_p(v), _p(dens), _p(wind), _p(out_bar), _p(v_bar), _p(dens_bar),
                                               _p(wind_bar), self.m.grid.ptr), "divv_h_tracer_adj")

    def scalar_times_vector_adj(self, s, v, out_bar, s_bar, v_bar):
        self._check(self.lib.scalar_times_vector_adj(_p(s), _p(v), _p(out_bar), _p(s_bar), _p(v_bar),
                                                     self.m.grid.ptr), "scalar_times_vector_adj")

    def inner_product_adj(self, a, b, out_bar, a_bar, b_bar):
        self._check(self.lib.inner_product_adj(_p(a), _p(b), _p(out_bar), _p(a_bar), _p(b_bar), self.m.grid.ptr),
                    "inner_product_adj")

    def calc_pot_vort_adj(self, wind, rho, pv_bar, wind_bar, rho_bar):
        m = self.m
        self._check(self.lib.calc_pot_vort_adj(_p(wind), _p(rho), _p(pv_bar), _p(wind_bar), _p(rho_bar), m.grid.ptr,
                                               m.dualgrid.ptr), "calc_pot_vort_adj")

    def vorticity_flux_adj(self, flux, pv, out_bar, flux_bar, pv_bar):
        m = self.m
        self._check(self.lib.vorticity_flux_adj(_p(flux), _p(pv), _p(out_bar), _p(flux_bar), _p(pv_bar), m.grid.ptr,
                                                m.dualgrid.ptr), "vorticity_flux_adj")

    def three_band_solver_ver_waves_adj(self, s_old, s_new, tend, dt, rk, so_bar, sn_bar, st_bar):
        m = self.m
        self._check(self.lib.three_band_solver_ver_waves_adj(s_old.ptr, s_new.ptr, tend.ptr, m.diagnostics.ptr,
                                                             m.forcings.ptr, m.config.ptr, dt, m.grid.ptr, rk,
                                                             so_bar.ptr, sn_bar.ptr, st_bar.ptr),
                    "three_band_solver_ver_waves_adj")

    def three_band_solver_gen_densities_adj(self, s_old, s_new, tend, dt, rk, so_bar, sn_bar, st_bar, diag_bar,
                                            irrev_bar):
        m = self.m
        self._check(self.lib.three_band_solver_gen_densities_adj(s_old.ptr, s_new.ptr, tend.ptr, m.diagnostics.ptr,
                                                                 m.irrev.ptr, m.config.ptr, dt, rk, m.grid.ptr,
                                                                 so_bar.ptr, sn_bar.ptr, st_bar.ptr, diag_bar.ptr,
                                                                 irrev_bar.ptr),
                    "three_band_solver_gen_densities_adj")

    def manage_rkhevi_adj(self, dt, t, s_new_bar, s_old_bar):
        m = self.m
        self._check(self.lib.manage_rkhevi_adj(m.state_old.ptr, m.state_new.ptr, m.grid.ptr, m.dualgrid.ptr,
                                               m.state_tendency.ptr, m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr,
                                               m.config.ptr, dt, t, s_new_bar.ptr, s_old_bar.ptr),
                    "manage_rkhevi_adj")

    # -- adjoint / tangent-linear windows (dry and moist builds; forward in the library's precision)
    def window_forward(self, s_init, s_final, dt, n_steps):
        m = self.m
        self._check(self.lib.rkhevi_window_forward(s_init.ptr, s_final.ptr, m.grid.ptr, m.dualgrid.ptr,
                                                   m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr, m.config.ptr,
                                                   dt, n_steps), "rkhevi_window_forward")

    def set_checkpoint_stride(self, every):
        self._check(self.lib.game_gpu_set_checkpoint_stride(every), "set_checkpoint_stride")

    def window_tl(self, s_dot, s_final_dot):
        self._check(self.lib.rkhevi_window_tl(s_dot.ptr, s_final_dot.ptr), "rkhevi_window_tl")

    def window_backward(self, s_final_bar, s_init_bar):
        self._check(self.lib.rkhevi_window_backward(s_final_bar.ptr, s_init_bar.ptr), "rkhevi_window_backward")

    def sfc_pressure_objective(self, state, weights, state_bar=None):
        import numpy as np
        w = np.ascontiguousarray(weights, dtype=np.float64)
        J = ctypes.c_double()
        self._check(self.lib.game_gpu_sfc_pressure_objective(state.ptr, _p(w), ctypes.byref(J),
                                                             state_bar.ptr if state_bar is not None else None),
                    "sfc_pressure_objective")
        return J.value

    # -- integrals and surface pressure
    def global_scalar_integrator(self, field):
        import math
        r = self.lib.global_scalar_integrator(_p(field), self.m.grid.ptr)
        if math.isnan(r):
            err = self.lib.game_gpu_last_error().decode()
            if err:
                raise GpuError(f"global_scalar_integrator: {err}")
        return r

    def write_out_integral(self, state, integral_id):
        """masses (id 0), rho*theta_v (id 1) or (0.5 kinetic, potential,
        c_v internal) energy (id 2) of a State"""
        import numpy as np
        n = {0: self.m.layout.n_const, 1: 1, 2: 3}[integral_id]
        out = np.zeros(max(n, 1))
        self._check(self.lib.game_gpu_write_out_integral(state.ptr, integral_id, _p(out)), "write_out_integral")
        return out[:n]

    def surface_pressure(self, state, with_mslp=False):
        """surface pressure (and MSLP) per column, reference column order"""
        import numpy as np
        nc = self.m.layout.nc
        ps = np.zeros(nc)
        ms = np.zeros(nc) if with_mslp else None
        self._check(self.lib.game_gpu_surface_pressure(state.ptr, _p(ps), _p(ms) if with_mslp else None),
                    "surface_pressure")
        return (ps, ms) if with_mslp else ps


    # -- output diagnostics
    def output_fields(self, state, wind_lowest, n_wind_steps, native=True, latlon=False, names=None, buffers=None):
        """the fields write_out computes (game_gpu_write_out_fields): a dict
        {"native": {name: array}, "latlon": {name: array}}; wind_lowest None
        takes the recorded device slots; buffers: a dict of that shape from an
        earlier call, reused instead of new arrays"""
        import numpy as np
        lay = self.m.layout
        nc, nl, nll = lay.nc, lay.nl, lay.n_latlon
        want = [n for n, _ in OUTPUT_FIELDS] if names is None else list(names)
        out = {}
        structs_ = []
        for grid_kind, on in (("native", native), ("latlon", latlon)):
            if not on:
                structs_.append(None)
                continue
            arrs = {}
            fs = OutputFields()
            for n, kind in OUTPUT_FIELDS:
                if n not in want or (grid_kind == "native" and kind == 3):
                    continue
                if grid_kind == "native":
                    size = {0: nc, 1: nl * nc, 2: nc * N_PRESSURE_LEVELS}[kind]
                else:
                    size = {0: 1, 1: nl, 2: N_PRESSURE_LEVELS, 3: nl + 1}[kind] * nll
                a = buffers[grid_kind][n] if buffers is not None else np.zeros(size)
                arrs[n] = a
                setattr(fs, n, a.ctypes.data_as(ctypes.POINTER(dbl)))
            out[grid_kind] = arrs
            structs_.append(fs)
        wl = None if wind_lowest is None else np.ascontiguousarray(wind_lowest, dtype=np.float64)
        m = self.m
        rc = self.lib.game_gpu_write_out_fields(state.ptr, _p(wl) if wl is not None else None, n_wind_steps,
                                                m.diagnostics.ptr, m.forcings.ptr, m.grid.ptr, m.config.ptr,
                                                ctypes.byref(structs_[0]) if structs_[0] is not None else None,
                                                ctypes.byref(structs_[1]) if structs_[1] is not None else None)
        self._check(rc, "write_out_fields")
        return out

    def record_wind_lowest(self, state, slot):
        self._check(self.lib.game_gpu_record_wind_lowest(state.ptr, slot), "record_wind_lowest")

    def interpolate_to_ll(self, field):
        import numpy as np
        out = np.zeros(self.m.layout.n_latlon)
        self._check(self.lib.interpolate_to_ll(_p(np.ascontiguousarray(field)), _p(out), self.m.grid.ptr),
                    "interpolate_to_ll")
        return out

    def edges_to_cells_lowest_layer(self, field):
        import numpy as np
        out = np.zeros(self.m.layout.nc)
        self._check(self.lib.edges_to_cells_lowest_layer(_p(np.ascontiguousarray(field)), _p(out), self.m.grid.ptr),
                    "edges_to_cells_lowest_layer")
        return out

    def epv_diagnostics(self, pot_vort, state):
        import numpy as np
        out = np.zeros(self.m.layout.n_scalars)
        self._check(self.lib.epv_diagnostics(_p(pot_vort), state.ptr, _p(out), self.m.grid.ptr,
                                             self.m.dualgrid.ptr), "epv_diagnostics")
        return out

    def inner_product_tangential(self, a, b):
        import numpy as np
        out = np.zeros(self.m.layout.n_scalars)
        self._check(self.lib.inner_product_tangential(_p(a), _p(b), _p(out), self.m.grid.ptr, self.m.dualgrid.ptr),
                    "inner_product_tangential")
        return out

    def calc_uv_at_edge(self, wind, u, v):
        self._check(self.lib.calc_uv_at_edge(_p(wind), _p(u), _p(v), self.m.grid.ptr), "calc_uv_at_edge")

    def curl_field_to_cells(self, curl):
        import numpy as np
        out = np.zeros(self.m.layout.n_scalars)
        self._check(self.lib.curl_field_to_cells(_p(curl), _p(out), self.m.grid.ptr), "curl_field_to_cells")
        return out

    def edges_to_cells(self, vec):
        import numpy as np
        out = np.zeros(self.m.layout.n_scalars)
        self._check(self.lib.edges_to_cells(_p(vec), _p(out), self.m.grid.ptr), "edges_to_cells")
        return out


def pinned_model(layout):
    """A Model whose structs live in pinned host memory (fast asynchronous
    copies), allocated through the library."""
    from .structs import Model
    lib = native.gpu()
    bufs = {}
    keep = []
    for k in Model.KINDS:
        kind = "state" if k.startswith("state") else k
        size = layout.sizes[kind]
        p = ctypes.c_void_p()
        if lib.game_gpu_host_alloc(ctypes.byref(p), size) != 0:
            raise GpuError(lib.game_gpu_last_error().decode())
        arr = (ctypes.c_uint8 * size).from_address(p.value)
        keep.append(p)
        import numpy as np
        bufs[k] = np.frombuffer(arr, dtype=np.uint8)
    m = Model(layout, bufs)
    m._pinned = keep
    return m
