"""Binding of the reference's own C build in oracle/_ref (this container only)."""
import ctypes
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402


def available():
    return build_ref.available()


class Reference:
    """The reference library for one (RES_ID, MOISTURE_ON), driven on a Model."""

    def __init__(self, model):
        lay = model.layout
        self.lib = ctypes.CDLL(build_ref.build(lay.res_id, lay.moisture_on, lay.n_layers))
        vp, dbl = ctypes.c_void_p, ctypes.c_double
        self.lib.manage_rkhevi.argtypes = [vp] * 9 + [dbl, dbl]
        self.lib.linear_combine_two_states.argtypes = [vp, vp, vp, dbl, dbl, vp]
        self.lib.ref_offsetof.restype = ctypes.c_long
        self.lib.ref_offsetof.argtypes = [ctypes.c_int, ctypes.c_char_p]
        self.lib.ref_sizeof.restype = ctypes.c_long
        self.lib.global_scalar_integrator = None
        self.m = model

    def manage_rkhevi(self, dt, t=0.0):
        m = self.m
        rc = self.lib.manage_rkhevi(m.state_old.ptr, m.state_new.ptr, m.grid.ptr, m.dualgrid.ptr,
                                    m.state_tendency.ptr, m.diagnostics.ptr, m.forcings.ptr, m.irrev.ptr,
                                    m.config.ptr, dt, t)
        assert rc == 0

    def linear_combine_two_states(self, s0, s1, out, c0, c1):
        self.lib.linear_combine_two_states(s0.ptr, s1.ptr, out.ptr, c0, c1, self.m.grid.ptr)
