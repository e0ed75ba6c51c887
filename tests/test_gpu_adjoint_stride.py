"""Adjoint windows that store only every k-th step start
(game_gpu_set_checkpoint_stride): the backward sweep recomputes the other
starts in FP64 from the checkpoint before them, the tangent-linear model
re-linearises only at stored starts.

* FP64 windows (dry and moist, 7 steps, stride 3): the gradient of the
  surface-pressure objective equals the all-checkpoint window's to 1e-12
  (norm-relative per field; the two differ only by the adjoint's atomic
  summation order), and the dot-product test holds to 1e-10;
* mixed-precision forward of record (moist, stride 3): the dot-product test
  holds to 1e-10 (between checkpoints TL and adjoint both follow the FP64
  recomputation).
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, structs
from helpers import clone, make_model, state_errors

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")
N_STEPS, STRIDE = 7, 3


def _dot(a, b):
    return sum(float(np.dot(a[f], b[f])) for f in FIELDS)


def _state_like(lay):
    return structs.HostStruct(lay, "state")


def _cap_weights(m, lat0=45.0, lon0=0.0, radius_deg=20.0):
    lay = m.layout
    lat, lon = m.grid["latitude_scalar"][:lay.nc], m.grid["longitude_scalar"][:lay.nc]
    p0, l0 = np.radians(lat0), np.radians(lon0)
    cosd = np.sin(lat) * np.sin(p0) + np.cos(lat) * np.cos(p0) * np.cos(lon - l0)
    area_sfc = m.grid["area"][lay.n_vectors - lay.nc:lay.n_vectors]
    return np.where(cosd >= np.cos(np.radians(radius_deg)), area_sfc, 0.0)


def _random(m, rng, scale_bar):
    s = _state_like(m.layout)
    so = m.state_old
    lay = m.layout
    ns = lay.n_scalars
    for k in range(lay.n_const):
        sl = slice(k * ns, (k + 1) * ns)
        sd = max(np.std(so["rho"][sl]), 1e-30)
        s["rho"][sl] = rng.standard_normal(ns) * (1.0 / sd if scale_bar else 1e-3 * sd)
    for f in ("rhotheta_v", "exner_pert", "wind"):
        sd = max(np.std(so[f]), 1e-30) if f != "wind" else 1.0
        s[f][:] = rng.standard_normal(s[f].size) * (1.0 / sd if scale_bar else 1e-3 * sd)
    return s


def _window(m0, precision, stride, dt):
    """(gradient of the objective, <TL dx, ybar>, <dx, AD ybar>)"""
    m = clone(m0)
    rng = np.random.default_rng(77)
    g = abi.GpuModel(m, precision)
    try:
        g.set_checkpoint_stride(stride)
        m.config["totally_first_step_bool"][0] = 1
        out = _state_like(m.layout)
        g.window_forward(m.state_old, out, dt, N_STEPS)
        jb = _state_like(m.layout)
        g.sfc_pressure_objective(out, _cap_weights(m), jb)
        grad = _state_like(m.layout)
        g.window_backward(jb, grad)
        dx, yb = _random(m, rng, False), _random(m, rng, True)
        dy, xb = _state_like(m.layout), _state_like(m.layout)
        g.window_tl(dx, dy)
        g.window_backward(yb, xb)
    finally:
        g.close()
    return grad, _dot(dy, yb), _dot(dx, xb)


CASES = {"dry": (0, "std_wind_tpert", 200.0), "moist": (1, "tracers", 300.0)}


@pytest.mark.parametrize("label", sorted(CASES))
def test_strided_checkpoints_give_the_same_gradient(label):
    moist, case, dt = CASES[label]
    _, m0 = make_model(3, moist, case, mountain=True)
    g1, _, _ = _window(m0, abi.FP64, 1, dt)
    g3, lhs, rhs = _window(m0, abi.FP64, STRIDE, dt)
    e = {k: v for k, v in state_errors(g3, g1, m0.layout).items() if np.isfinite(v)}
    print(f"\n{label}: {N_STEPS}-step window, stride {STRIDE} vs 1: gradient max {max(e.values()):.3g}; dot product "
          f"{lhs:.17g} vs {rhs:.17g} ({abs(lhs - rhs) / abs(lhs):.3g})")
    assert max(e.values()) <= 1e-12, e
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_strided_checkpoints_mixed_forward_dot_product():
    _, m0 = make_model(3, 1, "tracers", mountain=True)
    _, lhs, rhs = _window(m0, abi.MIXED, STRIDE, 300.0)
    print(f"\nmixed forward of record, stride {STRIDE}: dot product {lhs:.17g} vs {rhs:.17g} "
          f"({abs(lhs - rhs) / abs(lhs):.3g})")
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)
