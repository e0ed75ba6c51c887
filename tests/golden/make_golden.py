"""Generates the golden fixtures in this directory from the reference itself.

The reference's own C (oracle/_ref, compiled from the reference sources by
oracle/build_ref.py) runs the reference time loop on the grid tables of
game_archived_gb300.tables and the initial states of game_archived_gb300.cases;
after every step a fixed sample of every prognostic field (every 37th element)
and the full-field sums are stored, together with a fingerprint of the grid
tables.  tests/test_golden.py checks the oracle against these files on any
machine.  Run here, where the reference sources exist:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from game_archived_gb300 import driver  # noqa: E402

CASES = {
    "R3_dry_flat_std_wind": (3, 0, "std_wind", False, 400.0, 4),
    "R3_moist_oro_tracers": (3, 1, "tracers", True, 300.0, 3),
    "R4_dry_oro_tpert": (4, 0, "std_wind_tpert", True, 200.0, 2),
}
STRIDE = 37
FIELDS = ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind")


def grid_fingerprint(tab):
    keys = ("normal_distance", "area", "volume", "trsk_weights", "inner_product_weights", "z_vector",
            "density_to_rhombi_weights", "f_vec")
    return np.array([float(np.sum(tab[k])) for k in keys] + [float(np.sum(tab["trsk_indices"])),
                                                             float(np.sum(tab["adjacent_vector_indices_h"]))])


def sample(state):
    return {f: state[f][::STRIDE].copy() for f in FIELDS}, {f: float(np.sum(state[f])) for f in FIELDS}


def main():
    from helpers import make_model
    import refbind
    if not refbind.available():
        raise SystemExit("reference sources not present")
    for name, (res, moist, case, mountain, dt, steps) in CASES.items():
        tab, m = make_model(res, moist, case, mountain)
        ref = refbind.Reference(m)
        out = {"grid": grid_fingerprint(tab), "config": np.array([res, moist, int(mountain), dt, steps])}
        init, _ = sample(m.state_old)
        for f in FIELDS:
            out[f"init_{f}"] = init[f]
        driver.start(m, ref.linear_combine_two_states)
        for n in range(steps):
            driver.step(m, ref.linear_combine_two_states, ref.manage_rkhevi, dt, n * dt)
            smp, sums = sample(m.state_new)
            for f in FIELDS:
                out[f"step{n}_{f}"] = smp[f]
                out[f"step{n}_{f}_sum"] = np.array(sums[f])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name)


if __name__ == "__main__":
    main()
