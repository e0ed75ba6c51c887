"""Checkpoints and the device health check, through the C ABI.

* A run stopped after k steps, written to a checkpoint
  (game_gpu_write_checkpoint), and resumed in a new library context from
  fresh host structs (game_gpu_read_checkpoint) ends bit for bit where the
  uninterrupted run ends -- FP64 and mixed precision, resident and
  host-in/host-out.  The reference's own restart reads a State only
  (src/io/set_initial_state.c:244-336) and would not.
* game_gpu_check_state counts NaN/Inf values and negative densities planted
  in a host State (also after moving it to the device), reports the first of
  each in the reference's State layout, and passes a clean State (-0.0 is
  not negative); with game_gpu_set_health_check(1) manage_rkhevi returns
  GAME_GPU_UNHEALTHY after a step from a State with a planted NaN.  Nothing
  here faults the GPU: the bad values are ordinary doubles in host memory.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model

pytestmark = pytest.mark.gpu

DT, N, K = 300.0, 6, 3


@pytest.fixture(scope="module")
def moist_model():
    return make_model(4, 1, "tracers", True)[1]


def _fresh_like(m0):
    """new host structs with only the grid of m0 (as a new process would
    have them before reading a checkpoint)"""
    m = structs.Model(m0.layout)
    m.grid.copy_from(m0.grid)
    m.dualgrid.copy_from(m0.dualgrid)
    return m


def _sync_all(g, m):
    for s in (m.state_old, m.state_new, m.state_tendency):
        g.sync_to_device(s)


@pytest.mark.parametrize("precision,resident", [(abi.FP64, True), (abi.MIXED, False), (abi.MIXED, True)],
                         ids=["fp64-resident", "mixed-host", "mixed-resident"])
def test_resume_from_checkpoint_is_bit_identical(moist_model, tmp_path, precision, resident):
    m_a = clone(moist_model)
    g = abi.GpuModel(m_a, precision, resident=resident)
    try:
        if resident:
            _sync_all(g, m_a)
        driver.run(m_a, N, DT, g.linear_combine_two_states, g.manage_rkhevi)
        if resident:
            g.sync_to_host(m_a.state_new)
    finally:
        g.close()

    path = tmp_path / "run.ckpt"
    m_b = clone(moist_model)
    g = abi.GpuModel(m_b, precision, resident=resident)
    try:
        if resident:
            _sync_all(g, m_b)
        driver.run(m_b, K, DT, g.linear_combine_two_states, g.manage_rkhevi)
        g.write_checkpoint(path, m_b.state_new)
    finally:
        g.close()

    m_c = _fresh_like(moist_model)
    g = abi.GpuModel(m_c, precision, resident=resident)
    try:
        if resident:
            _sync_all(g, m_c)
        g.read_checkpoint(path, m_c.state_new)
        assert m_c.config["totally_first_step_bool"][0] == 0
        for n in range(K, N):
            driver.step(m_c, g.linear_combine_two_states, g.manage_rkhevi, DT, n * DT)
        if resident:
            g.sync_to_host(m_c.state_new)
    finally:
        g.close()
    for f in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        assert np.array_equal(m_c.state_new[f], m_a.state_new[f]), f


def test_checkpoint_is_refused_when_corrupted_or_for_another_grid(moist_model, tmp_path):
    path = tmp_path / "a.ckpt"
    m = clone(moist_model)
    g = abi.GpuModel(m, abi.FP64)
    try:
        g.write_checkpoint(path, m.state_new)
        raw = bytearray(path.read_bytes())
        raw[-12] ^= 0x40
        bad = tmp_path / "b.ckpt"
        bad.write_bytes(bytes(raw))
        with pytest.raises(abi.GpuError, match="digest"):
            g.read_checkpoint(bad, m.state_new)
    finally:
        g.close()
    _, m3 = make_model(3, 1, "tracers", True)
    g = abi.GpuModel(m3, abi.FP64)
    try:
        with pytest.raises(abi.GpuError, match="RES_ID"):
            g.read_checkpoint(path, m3.state_new)
    finally:
        g.close()


def test_health_check_counts_planted_values(moist_model):
    m = clone(moist_model)
    lay = m.layout
    ns = lay.n_scalars
    g = abi.GpuModel(m, abi.FP64)
    try:
        rc, r = g.check_state(m.state_old)
        assert rc == 0 and r["nonfinite"] == 0 and r["negative_density"] == 0
        s = m.state_old
        off_rho = lay.members["state"]["rho"][2] // 8
        off_wind = lay.members["state"]["wind"][2] // 8
        s["rho"][3 * ns + 17] = -0.0          # not negative
        rc, r = g.check_state(s)
        assert rc == 0, r
        s["rho"][2 * ns + 5] = -1e-9
        s["rho"][4 * ns + 9] = -2e-3
        s["wind"][123] = np.nan
        s["exner_pert"][7] = np.inf
        rc, r = g.check_state(s)
        assert rc == abi.UNHEALTHY
        assert r["nonfinite"] == 2 and r["negative_density"] == 2
        assert r["first_negative_density"] == off_rho + 2 * ns + 5
        off_ep = lay.members["state"]["exner_pert"][2] // 8
        assert r["first_nonfinite"] == min(off_wind + 123, off_ep + 7)
        assert "non-finite" in g.lib.game_gpu_last_error().decode()
    finally:
        g.close()
    # the same State as a device copy of a resident run
    g = abi.GpuModel(m, abi.FP64, resident=True)
    try:
        g.sync_to_device(m.state_old)
        rc, r = g.check_state(m.state_old)
        assert rc == abi.UNHEALTHY and r["nonfinite"] == 2 and r["negative_density"] == 2
    finally:
        g.close()


def test_manage_rkhevi_reports_an_unhealthy_step(moist_model):
    m = clone(moist_model)
    g = abi.GpuModel(m, abi.MIXED)
    try:
        g.set_health_check(1)
        driver.start(m, g.linear_combine_two_states)
        driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, DT, 0.0)   # healthy
        m.state_new["rhotheta_v"][1000] = np.nan
        with pytest.raises(abi.GpuError, match="non-finite"):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, DT, DT)
        g.set_health_check(0)
        driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, DT, 2 * DT)  # no check: returns 0
    finally:
        g.close()
