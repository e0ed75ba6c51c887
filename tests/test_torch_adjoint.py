"""The PyTorch restatement of the dry step (the CPU adjoint's forward model)
against the oracle, on CPU: three steps from the model's first step, RES_ID=3
with the 2 km mountain, every prognostic field within 1e-12 relative."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from game_archived_gb300 import driver, structs  # noqa: E402
from helpers import clone, make_model, state_errors  # noqa: E402
from oracle.bind import Oracle  # noqa: E402
import torch_dry_step as tds  # noqa: E402


def test_torch_dry_step_matches_the_oracle():
    _, m = make_model(3, 0, "std_wind_tpert", mountain=True)
    n, dt = 3, 300.0
    m_o = clone(m)
    orc = Oracle(m_o)
    driver.run(m_o, n, dt, orc.linear_combine_two_states, orc.manage_rkhevi)
    step = tds.make_step(m, dt)
    with torch.no_grad():
        out = step.window(tds.state_tensors(m, m.state_old), n)
    got = structs.HostStruct(m.layout, "state")
    tds.tensors_to_state(m, out, got)
    e = state_errors(got, m_o.state_new, m.layout)
    assert max(e.values()) <= 1e-12, e


def test_torch_surface_pressure_matches_the_oracle():
    _, m = make_model(3, 0, "std_wind_tpert", mountain=True)
    orc = Oracle(m)
    ref = orc.surface_pressure(m.state_old, orc.temperature(m.state_old))
    step = tds.make_step(m, 300.0)
    s = step.rediag(tds.state_tensors(m, m.state_old))
    got = step.sfc_pressure(s).numpy()
    assert np.max(np.abs(got - ref) / ref) <= 1e-14
