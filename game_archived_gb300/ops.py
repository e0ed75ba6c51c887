"""Operator calls through the reference's C signatures.

``CAbiOps`` calls scalar_times_vector, calc_pot_vort, vorticity_flux and
inner_product (src/spatial_operators/spatial_operators.h:6-36) on host arrays
through any shared library that exports them with the reference's signatures:
libgame_gb300.so (this project's CUDA library) or a build of the reference.
It is what the initial-state recipe in cases.py runs on.
"""
import ctypes

import numpy as np


def ptr(a):
    assert isinstance(a, np.ndarray) and a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


class CAbiOps:
    def __init__(self, lib, model):
        self.lib, self.model = lib, model
        vp = ctypes.c_void_p
        for name, n in (("scalar_times_vector", 4), ("calc_pot_vort", 5), ("vorticity_flux", 5),
                        ("inner_product", 4), ("grad", 3), ("divv_h", 3)):
            f = getattr(lib, name)
            f.argtypes = [vp] * n
            f.restype = ctypes.c_int

    def _check(self, rc, name):
        if rc != 0:
            raise RuntimeError(f"{name} returned {rc}")

    def scalar_times_vector(self, s, v, out):
        self._check(self.lib.scalar_times_vector(ptr(s), ptr(v), ptr(out), self.model.grid.ptr), "scalar_times_vector")

    def calc_pot_vort(self, wind, rho):
        m = self.model
        self._check(self.lib.calc_pot_vort(ptr(wind), ptr(rho), m.diagnostics.ptr, m.grid.ptr, m.dualgrid.ptr),
                    "calc_pot_vort")

    def vorticity_flux(self, flux, pv, out):
        m = self.model
        self._check(self.lib.vorticity_flux(ptr(flux), ptr(pv), ptr(out), m.grid.ptr, m.dualgrid.ptr),
                    "vorticity_flux")

    def inner_product(self, a, b, out):
        self._check(self.lib.inner_product(ptr(a), ptr(b), ptr(out), self.model.grid.ptr), "inner_product")
