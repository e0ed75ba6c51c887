"""The oracle against golden fixtures produced by the reference itself
(tests/golden/make_golden.py).  On the machine that generated them the grid
tables and the results agree bit for bit; elsewhere (another libm) the grid
fingerprint may differ in the last bits, so values are compared with a
relative tolerance of 1e-11."""
import os

import numpy as np
import pytest

from game_archived_gb300 import driver
from golden.make_golden import CASES, FIELDS, STRIDE, grid_fingerprint
from helpers import make_model
from oracle.bind import Oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_fixtures(name):
    path = os.path.join(HERE, f"{name}.npz")
    assert os.path.exists(path), "golden fixture missing"
    gold = np.load(path)
    res, moist, case, mountain, dt, steps = CASES[name]
    tab, m = make_model(res, moist, case, mountain)
    fp = grid_fingerprint(tab)
    exact = np.array_equal(fp, gold["grid"])
    assert np.allclose(fp, gold["grid"], rtol=1e-12, atol=0), "grid tables differ from the fixture's"
    o = Oracle(m)
    for f in FIELDS:
        a, b = m.state_old[f][::STRIDE], gold[f"init_{f}"]
        assert np.array_equal(a, b) if exact else np.allclose(a, b, rtol=1e-11, atol=1e-11 * np.abs(b).max())
    driver.start(m, o.linear_combine_two_states)
    for n in range(int(steps)):
        driver.step(m, o.linear_combine_two_states, o.manage_rkhevi, dt, n * dt)
        for f in FIELDS:
            a, b = m.state_new[f][::STRIDE], gold[f"step{n}_{f}"]
            if exact:
                assert np.array_equal(a, b), (n, f)
                assert float(np.sum(m.state_new[f])) == float(gold[f"step{n}_{f}_sum"]), (n, f)
            else:
                scale = np.abs(b).max()
                assert np.max(np.abs(a - b)) <= 1e-11 * scale, (n, f)
