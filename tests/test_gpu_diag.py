"""Global integrals and surface pressure on the GPU (C ABI) against the oracle.

global_scalar_integrator: the device sum carries the exact rounding error of
every product and addition, so it must equal the exactly rounded sum of the
exact products (computed here with fractions) to within 1 ulp, and the
reference's serial FP64 loop (the oracle) to within 1e-12 relative.
write_out_integral values: the same bounds against the oracle's serial sums.
Surface pressure / MSLP: pointwise FP64 with pow, within 1e-13 relative.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from game_archived_gb300 import abi, driver
from helpers import clone, make_model
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu


def exact_weighted_sum(a, b):
    s = Fraction(0)
    for x, y in zip(a.tolist(), b.tolist()):
        s += Fraction(x) * Fraction(y)
    return float(s)


@pytest.fixture(scope="module")
def moist_model():
    return make_model(3, 1, "jet_moist", mountain=True)


def test_integrator_exact_and_deterministic(moist_model):
    _, m = moist_model
    ns = m.layout.n_scalars
    rng = np.random.default_rng(7)
    # signed values with cancellation: the serial sum loses digits, the exact one does not
    field = rng.normal(size=ns) * np.exp(rng.uniform(-20, 20, size=ns))
    gpu = abi.GpuModel(clone(m), abi.FP64)
    try:
        r1 = gpu.global_scalar_integrator(field)
        r2 = gpu.global_scalar_integrator(field)
    finally:
        gpu.close()
    exact = exact_weighted_sum(field, m.grid["volume"])
    assert r1 == r2
    assert abs(r1 - exact) <= math.ulp(exact), (r1, exact)


def test_integrator_matches_serial_sum(moist_model):
    _, m = moist_model
    ns = m.layout.n_scalars
    orc = Oracle(m)
    gpu = abi.GpuModel(clone(m), abi.FP64)
    try:
        for k in range(m.layout.n_const):
            f = np.ascontiguousarray(m.state_old["rho"][k * ns:(k + 1) * ns])
            ref = orc.integral(f)
            got = gpu.global_scalar_integrator(f)
            assert abs(got - ref) <= 1e-12 * max(abs(ref), 1e-300), (k, got, ref)
        # a field of zeros integrates to exactly zero
        assert gpu.global_scalar_integrator(np.zeros(ns)) == 0.0
    finally:
        gpu.close()


@pytest.mark.parametrize("resident", [False, True], ids=["sync", "resident"])
def test_write_out_integrals_before_and_after_steps(moist_model, resident):
    _, m0 = moist_model
    m_orc, m_gpu = clone(m0), clone(m0)
    orc = Oracle(m_orc)
    gpu = abi.GpuModel(m_gpu, abi.FP64, resident=resident)
    dt = 300.0
    try:
        driver.start(m_orc, orc.linear_combine_two_states)
        driver.start(m_gpu, gpu.linear_combine_two_states)
        if resident:
            for s in (m_gpu.state_old, m_gpu.state_new, m_gpu.state_tendency):
                gpu.sync_to_device(s)
        # before the first step: temperature of the state itself (coordinator.c:250, :280-284)
        t0 = orc.temperature(m_orc.state_old)
        for iid in (0, 1, 2):
            ref = orc.write_out_integral(m_orc.state_old, iid, t0)
            got = gpu.write_out_integral(m_gpu.state_old, iid)
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, err_msg=f"id {iid} before stepping")
        for n in range(2):
            t_old = orc.temperature(m_orc.state_new)  # state_old of the coming step
            driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
            driver.step(m_gpu, gpu.linear_combine_two_states, gpu.manage_rkhevi, dt, n * dt)
            for iid in (0, 1, 2):
                ref = orc.write_out_integral(m_orc.state_new, iid, t_old)
                got = gpu.write_out_integral(m_gpu.state_new, iid)
                np.testing.assert_allclose(got, ref, rtol=1e-11, atol=0, err_msg=f"id {iid} after step {n}")
    finally:
        gpu.close()


@pytest.mark.parametrize("moist", [0, 1])
def test_surface_pressure_and_mslp(moist):
    _, m = make_model(3, moist, "std_wind_tpert" if not moist else "jet_moist", mountain=True)
    orc = Oracle(m)
    t = orc.temperature(m.state_old)
    ps_ref, ms_ref = orc.surface_pressure(m.state_old, t, with_mslp=True)
    gpu = abi.GpuModel(clone(m), abi.FP64)
    try:
        ps, ms = gpu.surface_pressure(gpu.m.state_old, with_mslp=True)
        ps_only = gpu.surface_pressure(gpu.m.state_old)
    finally:
        gpu.close()
    np.testing.assert_allclose(ps, ps_ref, rtol=1e-13, atol=0)
    np.testing.assert_allclose(ms, ms_ref, rtol=1e-13, atol=0)
    assert np.array_equal(ps, ps_only)
    assert np.all(ps > 5e4) and np.all(ps < 1.2e5)
    # over the mountain the surface pressure is below the MSLP, elsewhere (z_sfc = 0) they agree
    assert np.all(ps <= ms * (1 + 1e-12))
