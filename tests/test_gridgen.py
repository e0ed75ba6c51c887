"""Grid-table builder: counts, ranges and the invariants the reference's grid
generator checks (grid_generator/src/*.c sanity checks), plus the discrete
identities the step relies on."""
import numpy as np
import pytest

from helpers import MOUNTAIN
from game_archived_gb300 import tables


@pytest.fixture(scope="module", params=[(2, False), (3, True)], ids=["R2-flat", "R3-oro"])
def tab(request):
    res, mountain = request.param
    return tables.GridTables(res, n_lloyd=100, mountain=MOUNTAIN if mountain else None)


def test_counts_and_ranges(tab):
    nc, ne, nt, nl = tab.nc, tab.ne, tab.nt, tab.n_layers
    assert nc == 10 * 4 ** tab.res_id + 2 and ne == 30 * 4 ** tab.res_id and nt == 20 * 4 ** tab.res_id
    assert nc - ne + nt == 2  # Euler characteristic of the sphere
    for k in ("from_index", "to_index"):
        assert tab[k].min() >= 0 and tab[k].max() < nc
    adj = tab["adjacent_vector_indices_h"].reshape(nc, 6)
    sign = tab["adjacent_signs_h"].reshape(nc, 6)
    assert np.all(sign[:12, 5] == 0) and np.all(np.abs(sign[12:]) == 1)
    # each edge is adjacent to exactly two cells, once with +1 and once with -1
    cnt = np.zeros(ne, int)
    ssum = np.zeros(ne, int)
    for j in range(6):
        m = sign[:, j] != 0
        np.add.at(cnt, adj[m, j], 1)
        np.add.at(ssum, adj[m, j], sign[m, j])
    assert np.all(cnt == 2) and np.all(ssum == 0)
    assert tab["trsk_indices"].max() < ne and tab["vorticity_indices_triangles"].max() < ne


def test_areas_and_weights(tab):
    assert abs(tab["pent_hex_face_unity_sphere"].sum() / (4 * np.pi) - 1) < 1e-10
    assert abs(tab["triangle_face_unit_sphere"].sum() / (4 * np.pi) - 1) < 1e-10
    w = tab["density_to_rhombi_weights"].reshape(-1, 4)
    assert np.allclose(w.sum(axis=1), 1.0, atol=1e-10) and np.all(w > 0)
    assert np.all(tab["volume"] > 0) and np.all(tab["normal_distance"] > 0)


def test_divergence_of_constant_flux_sums_to_zero(tab):
    """sum over cells of the horizontal divergence times volume vanishes for any
    edge field (each edge enters two cells with opposite signs)"""
    nc, ne, nl = tab.nc, tab.ne, tab.n_layers
    vpl = nc + ne
    adj = tab["adjacent_vector_indices_h"].reshape(nc, 6)
    sign = tab["adjacent_signs_h"].reshape(nc, 6)
    area = tab["area"]
    rng = np.random.default_rng(0)
    f = rng.standard_normal(ne)
    l = nl - 1
    a = area[nc + l * vpl: (l + 1) * vpl]
    tot = 0.0
    for j in range(6):
        tot += np.sum(f[adj[:, j]] * sign[:, j] * a[adj[:, j]])
    assert abs(tot) < 1e-9 * np.sum(np.abs(f * a))


def test_background_state_hydrostatic(tab):
    """the background Exner pressure satisfies the discrete hydrostatic
    balance it was integrated with (vertical_grid.c:311-348)"""
    nc, nl = tab.nc, tab.n_layers
    pi = tab["exner_bg"].reshape(nl, nc)
    th = tab["theta_v_bg"].reshape(nl, nc)
    phi = tab["gravity_potential"].reshape(nl, nc)
    lhs = 1005.0 * 0.5 * (th[:-1] + th[1:]) * (pi[:-1] - pi[1:])
    rhs = -(phi[:-1] - phi[1:])
    assert np.max(np.abs(lhs - rhs) / np.abs(rhs)) < 1e-2
