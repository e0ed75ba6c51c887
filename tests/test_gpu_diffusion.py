"""Diffusion branch of the step on the GPU (C ABI) against the oracle.

The oracle's diffusion branch is itself byte-identical to the reference's C
(tests/test_oracle_vs_reference.py).  Here the GPU step runs with the same
switch combinations and a seeded turbulent kinetic energy:
* FP64: every prognostic field within 1e-12 relative of the oracle after
  each of the first steps (both trajectories run freely, so the bound also
  covers the TKE, viscosity, friction and heating fields the step carries
  from one call to the next), and after game_gpu_sync_aux_to_host those
  carried fields within 1e-11;
* device-resident steps with CUDA graphs give the same bits as host-in/host-out
  steps;
* the mixed path stays as close to FP64 as without diffusion;
* the Held-Suarez configuration (radiation relaxation and boundary-layer
  friction with horizontal momentum diffusion) within 1e-12 of the oracle at
  RES_ID = 5, where the reference's radiation blocks tile the grid, and
  refused where they would overrun radiation_tendency;
* RTE+RRTMGP radiation and the sub-step entry points without a diffusion
  branch are refused on the host.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver
from helpers import clone, make_model, rel_err, state_errors
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

SWITCHES = ("momentum_diff_h", "momentum_diff_v", "temperature_diff_h", "temperature_diff_v", "mass_diff_h",
            "mass_diff_v")
CASES = [
    # (res, moist, case, mountain, dt, steps, switches on)
    (3, 1, "tracers", True, 300.0, 4, SWITCHES),
    (3, 0, "std_wind_tpert", True, 300.0, 4, ("momentum_diff_h",)),
    (3, 0, "std_wind_tpert", True, 300.0, 3, ("momentum_diff_v",)),
    (3, 1, "jet_moist", False, 300.0, 3, ("mass_diff_h", "mass_diff_v")),
    (4, 1, "tracers", True, 200.0, 3, ("momentum_diff_h", "temperature_diff_h", "temperature_diff_v")),
    (4, 0, "std_wind_tpert", True, 200.0, 3, SWITCHES),
]
CARRIED = ("tke", "viscosity", "heating_diss", "friction_acc", "temperature_diffusion_heating", "mass_diff_tendency")


def with_diffusion(m, switches, seed=5):
    for s in SWITCHES:
        m.config[s][0] = 1 if s in switches else 0
    rng = np.random.default_rng(seed)
    m.irrev["tke"][:] = 0.5 + 0.5 * rng.random(m.irrev["tke"].size)
    return m


def _ids(c):
    return f"R{c[0]}M{c[1]}-{c[2]}-" + "+".join(s.replace("_diff_", "") for s in c[6])


@pytest.mark.parametrize("cfg", CASES, ids=_ids)
def test_diffusion_step_fp64_matches_oracle(cfg):
    res, moist, case, mountain, dt, steps, switches = cfg
    _, m_orc = make_model(res, moist, case, mountain)
    with_diffusion(m_orc, switches)
    m_gpu = clone(m_orc)
    orc = Oracle(m_orc)
    g = abi.GpuModel(m_gpu, abi.FP64)
    worst = 0.0
    try:
        driver.start(m_orc, orc.linear_combine_two_states)
        driver.start(m_gpu, g.linear_combine_two_states)
        for n in range(steps):
            driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
            driver.step(m_gpu, g.linear_combine_two_states, g.manage_rkhevi, dt, n * dt)
            e = state_errors(m_gpu.state_new, m_orc.state_new, m_gpu.layout)
            worst = max(worst, max(e.values()))
            assert max(e.values()) <= 1e-12, f"step {n}: {e}"
        g.sync_aux_to_host()
    finally:
        g.close()
    carried = {f: rel_err(m_gpu.irrev[f], m_orc.irrev[f]) for f in CARRIED if np.any(m_orc.irrev[f] != 0)}
    print(f"{_ids(cfg)}: worst state error {worst:.3g}; carried fields {carried}")
    assert max(carried.values(), default=0.0) <= 1e-11, carried
    assert rel_err(m_gpu.diagnostics["n_squared"], m_orc.diagnostics["n_squared"]) <= 1e-11


def test_diffusion_resident_graph_equals_host_mode():
    _, m0 = make_model(3, 1, "tracers", True)
    with_diffusion(m0, SWITCHES)
    out = []
    for resident in (False, True):
        m = clone(m0)
        g = abi.GpuModel(m, abi.FP64, resident=resident, graphs=resident)
        try:
            # the start-up combination (which rediagnoses theta_v') runs on
            # the device in both modes
            if resident:
                for s in (m.state_old, m.state_tendency):
                    g.sync_to_device(s)
            driver.start(m, g.linear_combine_two_states)
            for n in range(3):
                driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, 300.0, n * 300.0)
            if resident:
                g.sync_to_host(m.state_new)
        finally:
            g.close()
        out.append(m.state_new)
    for f in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        assert np.array_equal(out[0][f], out[1][f]), f


def test_diffusion_mixed_close_to_fp64():
    _, m64 = make_model(4, 1, "jet_moist", False)
    with_diffusion(m64, SWITCHES)
    m32 = clone(m64)
    for m, prec in ((m64, abi.FP64), (m32, abi.MIXED)):
        g = abi.GpuModel(m, prec)
        try:
            driver.run(m, 4, 300.0, g.linear_combine_two_states, g.manage_rkhevi)
        finally:
            g.close()
    e = state_errors(m32.state_new, m64.state_new, m64.layout)
    print(f"diffusion on, mixed vs FP64 after 4 steps: {e}")
    assert e["rho[4]"] < 1e-5 and e["rhotheta_v"] < 1e-5 and e["exner_pert"] < 1e-3, e
    assert e["wind_h"] < 1e-3, e


def test_out_of_scope_switches_refused():
    _, m = make_model(3, 0, "std_wind")
    with_diffusion(m, SWITCHES)
    m.config["rad_on"][0] = 1
    g = abi.GpuModel(m, abi.FP64)
    try:
        driver.start(m, g.linear_combine_two_states)
        with pytest.raises(abi.GpuError, match="rad_on"):
            g.manage_rkhevi(300.0)
        m.config["rad_on"][0] = 0
        with pytest.raises(abi.GpuError, match="diffusion branch"):
            g.three_band_solver_ver_waves(m.state_old, m.state_new, m.state_tendency, 300.0, 0)
    finally:
        g.close()


def held_suarez(m):
    """the reference's Held-Suarez run configuration (run_scripts/held_suar.sh):
    Held-Suarez radiation and boundary-layer friction, horizontal momentum
    diffusion"""
    with_diffusion(m, ("momentum_diff_h",))
    m.config["rad_on"][0] = 2
    m.config["pbl_scheme"][0] = 2
    return m


@pytest.mark.parametrize("moist,case,mountain", [(0, "std_wind_tpert", True), (1, "tracers", False)],
                         ids=["dry-oro", "moist"])
def test_held_suarez_fp64_matches_oracle(moist, case, mountain):
    """RES_ID = 5 (the reference's 18 radiation blocks tile its 10242 cells);
    the radiation is updated at every other step, as the reference's driver
    does for a radiation time step of two model steps"""
    _, m_orc = make_model(5, moist, case, mountain)
    held_suarez(m_orc)
    m_gpu = clone(m_orc)
    orc = Oracle(m_orc)
    g = abi.GpuModel(m_gpu, abi.FP64)
    worst = 0.0
    try:
        driver.start(m_orc, orc.linear_combine_two_states)
        driver.start(m_gpu, g.linear_combine_two_states)
        for n in range(4):
            for m in (m_orc, m_gpu):
                m.config["rad_update"][0] = 1 if n % 2 == 0 else 0
            driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, 200.0, n * 200.0)
            driver.step(m_gpu, g.linear_combine_two_states, g.manage_rkhevi, 200.0, n * 200.0)
            e = state_errors(m_gpu.state_new, m_orc.state_new, m_gpu.layout)
            worst = max(worst, max(e.values()))
            assert max(e.values()) <= 1e-12, f"step {n}: {e}"
        g.sync_aux_to_host()
    finally:
        g.close()
    rad = rel_err(m_gpu.forcings["radiation_tendency"], m_orc.forcings["radiation_tendency"])
    fric = rel_err(m_gpu.irrev["friction_acc"], m_orc.irrev["friction_acc"])
    print(f"Held-Suarez, {case}: worst state error {worst:.3g}, radiation_tendency {rad:.3g}, friction {fric:.3g}")
    assert rad <= 1e-11 and fric <= 1e-11
    assert np.all(m_gpu.forcings["sfc_sw_in"] == 0.0)


def test_held_suarez_mixed_close_to_fp64():
    _, m64 = make_model(5, 0, "std_wind_tpert", True)
    held_suarez(m64)
    m64.config["rad_update"][0] = 1
    m32 = clone(m64)
    for m, prec in ((m64, abi.FP64), (m32, abi.MIXED)):
        g = abi.GpuModel(m, prec)
        try:
            driver.run(m, 4, 200.0, g.linear_combine_two_states, g.manage_rkhevi)
        finally:
            g.close()
    e = state_errors(m32.state_new, m64.state_new, m64.layout)
    print(f"Held-Suarez, mixed vs FP64 after 4 steps: {e}")
    assert e["rho[0]"] < 1e-5 and e["rhotheta_v"] < 1e-5 and e["exner_pert"] < 1e-3 and e["wind_h"] < 1e-3, e


def test_held_suarez_refused_where_the_reference_overruns():
    """RES_ID = 3 with 26 layers: NO_OF_SCALARS / 18 = 927 is not a multiple of
    26, so the reference's radiation-block loops write past the end of
    radiation_tendency; the library refuses instead.  rad_on = 1 (RTE+RRTMGP)
    is refused on every grid."""
    _, m = make_model(3, 0, "std_wind")
    held_suarez(m)
    m.config["rad_update"][0] = 1
    g = abi.GpuModel(m, abi.FP64)
    try:
        driver.start(m, g.linear_combine_two_states)
        with pytest.raises(abi.GpuError, match="radiation blocks"):
            g.manage_rkhevi(200.0)
        m.config["rad_on"][0] = 1
        with pytest.raises(abi.GpuError, match="RTE"):
            g.manage_rkhevi(200.0)
    finally:
        g.close()
