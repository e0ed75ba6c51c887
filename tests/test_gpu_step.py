"""RKHEVI step on the GPU (C ABI, FP64) against the oracle, step by step.

Tolerance: every prognostic field within 1e-12 relative (max |gpu - oracle| /
max |oracle|) after every step, starting each comparison from the state both
reached; the FP64 path is compiled without FMA contraction and follows the
reference's operation order, so the remaining differences come only from
CUDA's exp/pow/sin versus the host libm.
"""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver
from helpers import clone, make_model, state_errors, state_errors_pointwise
from oracle.bind import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
# pointwise relative error |gpu - oracle| / |oracle| over the entries whose
# magnitude is at least 1e-6 of the field's largest (the perturbation fields
# theta_v' and Pi' and the vertical wind pass through zero, where a relative
# error has no meaning)
POINTWISE_TOL = 1e-9

CONFIGS = [
    # (res, moist, case, mountain, dt, steps)
    (3, 0, "std_wind", False, 400.0, 6),
    (4, 0, "std_wind_tpert", True, 200.0, 5),
    (4, 1, "jet_moist", False, 300.0, 5),
    (3, 1, "tracers", True, 300.0, 4),
    # the benchmark configurations at their own sizes: RES_ID=4 standard
    # atmosphere with wind noise (400 s, 10 steps), RES_ID=5 with the
    # mountain and 1 K noise (200 s), RES_ID=6 moist jet (100 s)
    (4, 0, "std_wind", False, 400.0, 10),
    (5, 0, "std_wind_tpert", True, 200.0, 72),
    (6, 1, "jet_moist", False, 100.0, 2),
]


def _run_pair(res, moist, case, mountain, dt, steps, resident=False, graphs=True):
    tab, m_orc = make_model(res, moist, case, mountain)
    m_gpu = clone(m_orc)
    orc = Oracle(m_orc)
    gpu = abi.GpuModel(m_gpu, abi.FP64, resident=resident, graphs=graphs)
    try:
        driver.start(m_orc, orc.linear_combine_two_states)
        driver.start(m_gpu, gpu.linear_combine_two_states)
        if resident:
            for s in (m_gpu.state_old, m_gpu.state_new, m_gpu.state_tendency):
                gpu.sync_to_device(s)
        errs = []
        for n in range(steps):
            driver.step(m_orc, orc.linear_combine_two_states, orc.manage_rkhevi, dt, n * dt)
            driver.step(m_gpu, gpu.linear_combine_two_states, gpu.manage_rkhevi, dt, n * dt)
            if resident:
                gpu.sync_to_host(m_gpu.state_new)
            errs.append({"norm": state_errors(m_gpu.state_new, m_orc.state_new, m_gpu.layout),
                         "pointwise": state_errors_pointwise(m_gpu.state_new, m_orc.state_new, m_gpu.layout)})
            # continue both from the oracle's state so that every step is compared from identical inputs
            m_gpu.state_new.copy_from(m_orc.state_new)
            if resident:
                gpu.sync_to_device(m_gpu.state_new)
        return errs, m_gpu, m_orc, gpu
    finally:
        gpu.close()


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: f"R{c[0]}M{c[1]}-{c[2]}{'-oro' if c[3] else ''}-{c[5]}")
def test_step_fp64_matches_oracle(cfg):
    errs, *_ = _run_pair(*cfg)
    for n, e in enumerate(errs):
        worst = max(e["norm"].values())
        assert worst <= TOL, f"step {n}: {e['norm']}"
        worst_pw = max(e["pointwise"].values())
        assert worst_pw <= POINTWISE_TOL, f"step {n}: {e['pointwise']}"
    norm = {k: max(e["norm"][k] for e in errs) for k in errs[0]["norm"]}
    pw = {k: max(e["pointwise"][k] for e in errs) for k in errs[0]["pointwise"]}
    print(f"\n{cfg}: worst over {len(errs)} steps, norm-relative {max(norm.values()):.3g} {norm}; "
          f"pointwise {max(pw.values()):.3g} {pw}")


def test_resident_graph_equals_sync():
    """device-resident mode with CUDA graphs gives the same bits as the
    host-in/host-out mode"""
    cfg = (3, 1, "jet_moist", False, 300.0, 3)
    _, m_sync, _, _ = _run_pair(*cfg, resident=False, graphs=False)
    _, m_res, _, _ = _run_pair(*cfg, resident=True, graphs=True)
    for f in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        assert np.array_equal(m_sync.state_new[f], m_res.state_new[f]), f


def test_mixed_precision_close_to_fp64():
    """mixed path (FP32 horizontal operators) stays close to FP64 over a few steps"""
    res, moist, case, dt, steps = 4, 1, "jet_moist", 300.0, 4
    _, m64 = make_model(res, moist, case)
    m32 = clone(m64)
    g64 = abi.GpuModel(m64, abi.FP64)
    try:
        driver.run(m64, steps, dt, g64.linear_combine_two_states, g64.manage_rkhevi)
    finally:
        g64.close()
    g32 = abi.GpuModel(m32, abi.MIXED)
    try:
        driver.run(m32, steps, dt, g32.linear_combine_two_states, g32.manage_rkhevi)
    finally:
        g32.close()
    e = state_errors(m32.state_new, m64.state_new, m64.layout)
    assert e["rho[4]"] < 1e-5 and e["rhotheta_v"] < 1e-5 and e["exner_pert"] < 1e-3, e
    assert e["wind_h"] < 1e-3, e


@pytest.mark.parametrize("case,mountain", [("tracers", True), ("jet_moist", False)])
def test_double_float_eliminations_keep_the_mixed_error(case, mountain):
    """the mixed path with its vertical eliminations in double-float (the
    default) and in FP64 (game_gpu_set_double_float(0)) stays as close to
    the FP64 path: per field, the double-float run's error is within 1.5
    times the FP64-elimination run's, plus 1e-12; and the two mixed runs
    differ far less than either differs from FP64"""
    res, moist, dt, steps = 4, 1, 300.0, 4
    _, m0 = make_model(res, moist, case, mountain)
    runs = {}
    for name, prec, dfl in (("fp64", abi.FP64, 1), ("mixed_f64elim", abi.MIXED, 0), ("mixed_df", abi.MIXED, 1)):
        m = clone(m0)
        g = abi.GpuModel(m, prec, double_float=dfl)
        try:
            driver.run(m, steps, dt, g.linear_combine_two_states, g.manage_rkhevi)
        finally:
            g.close()
        runs[name] = m
    lay = m0.layout
    e_ref = state_errors(runs["mixed_f64elim"].state_new, runs["fp64"].state_new, lay)
    e_df = state_errors(runs["mixed_df"].state_new, runs["fp64"].state_new, lay)
    e_between = state_errors(runs["mixed_df"].state_new, runs["mixed_f64elim"].state_new, lay)
    print(f"\n{case}: mixed (FP64 eliminations) vs FP64 {e_ref}\nmixed (double-float) vs FP64 {e_df}\n"
          f"between the two mixed runs {e_between}")
    for k in e_ref:
        assert e_df[k] <= 1.5 * e_ref[k] + 1e-12, (k, e_df[k], e_ref[k])
    assert max(e_between.values()) <= 0.1 * max(e_ref.values()) + 1e-12
