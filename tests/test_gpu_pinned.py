"""States in the library's own pinned allocations (game_gpu_host_alloc) are
copied by kernels that read and write host memory directly; everywhere else
the copies are staged.  Both give the same bits: host-in/host-out steps and
state blends on a pinned model equal those on an ordinary one, in both
precisions, and a device-resident run synchronised through pinned structs
equals one synchronised through ordinary ones."""
import numpy as np
import pytest

from game_archived_gb300 import abi, driver, structs
from helpers import clone, make_model

pytestmark = pytest.mark.gpu
FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


def pinned_clone(m0):
    m = abi.pinned_model(m0.layout)
    for k in structs.Model.KINDS:
        getattr(m, k).copy_from(getattr(m0, k))
    return m


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED], ids=["fp64", "mixed"])
def test_pinned_host_mode_equals_staged(precision):
    _, m0 = make_model(4, 1, "jet_moist", False)
    out = []
    for pinned in (False, True):
        m = pinned_clone(m0) if pinned else clone(m0)
        g = abi.GpuModel(m, precision)
        try:
            driver.run(m, 3, 200.0, g.linear_combine_two_states, g.manage_rkhevi)
            g.linear_combine_two_states(m.state_old, m.state_new, m.state_tendency, 0.25, 0.75)
        finally:
            g.close()
        out.append(m)
    a, b = out
    for s in ("state_old", "state_new", "state_tendency"):
        for f in FIELDS:
            assert np.array_equal(getattr(a, s)[f], getattr(b, s)[f]), (s, f)


def test_pinned_resident_sync_equals_staged():
    _, m0 = make_model(3, 0, "std_wind_tpert", True)
    out = []
    for pinned in (False, True):
        m = pinned_clone(m0) if pinned else clone(m0)
        g = abi.GpuModel(m, abi.FP64, resident=True)
        try:
            for s in (m.state_old, m.state_new, m.state_tendency):
                g.sync_to_device(s)
            driver.start(m, g.linear_combine_two_states)
            for n in range(3):
                driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, 300.0, n * 300.0)
            g.sync_to_host(m.state_new)
        finally:
            g.close()
        out.append(m.state_new)
    for f in FIELDS:
        assert np.array_equal(out[0][f], out[1][f]), f
