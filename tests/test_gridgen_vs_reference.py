"""The grid-table builder against the reference's own grid generator.

The reference's generator (grid_generator/src/*.c, its main) is compiled into
the reference harness with a netCDF stand-in that records the tables it would
write to its grid file (oracle/build_ref.py: build_gridgen), and runs
in-process on a flat grid.  The table builder numbers cells, edges and
triangles its own way, so the two grids are matched first: cells and
triangles by position, edges by their pair of cells, with the edge's
orientation (from/to) recorded; every table is then compared in the
reference's numbering, signs corrected for reversed edges:
* geometry (positions, heights, distances, areas, volumes, the background
  state, directions, Coriolis vector, inner-product and rhombus weights) to
  1e-12 of each table's largest magnitude, the TRSK weights to 1e-11 (five
  times both at RES_ID 5): both follow the same formulas, summed in
  different orders; the share of entries that differ and the largest
  difference in ulps are printed per table (heights, gravity potential and
  the background state are bit-identical; positions, distances, areas and
  volumes are not);
* topology (cell-edge incidence and signs, triangle-edge incidence and signs,
  the dual orientation, TRSK and modified-curl index pairs) exactly;
* TRSK weights that are zero up to rounding (|w| < 1e-9 of the largest: the
  Gassmann slots whose two kite areas cancel) are compared as zero;
* the lat-lon interpolation: identical cells and weights at every point
  except where two cells are equally far from it, where the reference's
  index-order tie rule picks by numbering.
The reference's generator parses its stretching parameter with strtof, so its
grids use float(1.3); GridTables does the same.
"""
import math

import numpy as np
import pytest

import refbind
from game_archived_gb300 import tables

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference sources not present")
L = 26


def xyz(lat, lon):
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s else float(np.max(np.abs(a - b)))


def ulps(a, b, floor=1e-9):
    """(share of entries that differ, largest difference in units in the last
    place of the reference value) over the entries with |b| above floor of
    the table's largest magnitude"""
    a, b = np.asarray(a, dtype=np.float64).ravel(), np.asarray(b, dtype=np.float64).ravel()
    m = np.abs(b) > floor * np.max(np.abs(b)) if np.max(np.abs(b)) > 0 else np.ones(b.shape, bool)
    d = np.abs(a[m] - b[m]) / np.spacing(np.abs(b[m]))
    return float(np.mean(a[m] != b[m])), float(np.max(d)) if d.size else 0.0


def match(T, ref):
    from scipy.spatial import cKDTree
    o_c = xyz(T["latitude_scalar"], T["longitude_scalar"])
    d, cmap = cKDTree(xyz(ref["latitude_scalar"], ref["longitude_scalar"])).query(o_c)
    assert d.max() < 1e-12 and len(set(cmap)) == len(cmap)
    rf, rt = ref["from_index"].astype(int), ref["to_index"].astype(int)
    key = {(min(a, b), max(a, b)): e for e, (a, b) in enumerate(zip(rf, rt))}
    ne = len(T["from_index"])
    emap, esign = np.zeros(ne, int), np.zeros(ne, int)
    for e in range(ne):
        a, b = cmap[T["from_index"][e]], cmap[T["to_index"][e]]
        emap[e] = key[(min(a, b), max(a, b))]
        esign[e] = 1 if rf[emap[e]] == a else -1
    d, tmap = cKDTree(xyz(ref["latitude_scalar_dual"], ref["longitude_scalar_dual"])).query(
        xyz(T["latitude_scalar_dual"], T["longitude_scalar_dual"]))
    assert d.max() < 1e-12 and len(set(tmap)) == len(tmap)
    return cmap, emap, esign, tmap


@pytest.mark.parametrize("res,n_iter", [(3, 0), (3, 10), (4, 3), (5, 1)])
def test_tables_match_reference_generator(res, n_iter, tmp_path):
    ref = refbind.run_gridgen(res, n_iter, str(tmp_path))
    T = tables.GridTables(res, n_layers=L, n_lloyd=n_iter)
    cmap, emap, esign, tmap = match(T, ref)
    nc, ne, nt = len(cmap), len(emap), len(tmap)
    vpl, dpl = nc + ne, ne + nt
    errs = {}
    # cells
    dlon = np.angle(np.exp(1j * (T["longitude_scalar"] - ref["longitude_scalar"][cmap])))
    errs["latitude_scalar"] = rel(T["latitude_scalar"], ref["latitude_scalar"][cmap])
    # (the longitude of a cell at a pole is whatever atan2 makes of rounding)
    off_pole = np.cos(T["latitude_scalar"]) > 1e-9
    errs["longitude_scalar"] = float(np.max(np.abs(dlon[off_pole])))
    ulp = {}
    for name in ("z_scalar", "volume", "gravity_potential", "theta_v_bg", "exner_bg"):
        errs[name] = rel(T[name].reshape(L, nc), ref[name].reshape(L, nc)[:, cmap])
        ulp[name] = ulps(T[name].reshape(L, nc), ref[name].reshape(L, nc)[:, cmap])
    # primal vector fields: vertical at the cells, horizontal at the edges
    for name in ("z_vector", "normal_distance", "area"):
        a, b = T[name], ref[name]
        errs[name + "_v"] = rel(np.stack([a[k * vpl:k * vpl + nc] for k in range(L + 1)]),
                                np.stack([b[k * vpl:k * vpl + nc][cmap] for k in range(L + 1)]))
        errs[name + "_h"] = rel(np.stack([a[k * vpl + nc:(k + 1) * vpl] for k in range(L)]),
                                np.stack([b[k * vpl + nc:(k + 1) * vpl][emap] for k in range(L)]))
        ulp[name + "_v"] = ulps(np.stack([a[k * vpl:k * vpl + nc] for k in range(L + 1)]),
                                np.stack([b[k * vpl:k * vpl + nc][cmap] for k in range(L + 1)]))
        ulp[name + "_h"] = ulps(np.stack([a[k * vpl + nc:(k + 1) * vpl] for k in range(L)]),
                                np.stack([b[k * vpl + nc:(k + 1) * vpl][emap] for k in range(L)]))
    # dual vector fields: horizontal at the edges, vertical at the triangles
    for name in ("area_dual", "z_vector_dual", "normal_distance_dual"):
        a, b = T[name], ref[name]
        errs[name + "_h"] = rel(np.stack([a[k * dpl:k * dpl + ne] for k in range(L + 1)]),
                                np.stack([b[k * dpl:k * dpl + ne][emap] for k in range(L + 1)]))
        errs[name + "_t"] = rel(np.stack([a[k * dpl + ne:(k + 1) * dpl] for k in range(L)]),
                                np.stack([b[k * dpl + ne:(k + 1) * dpl][tmap] for k in range(L)]))
    # edges
    errs["latitude_vector"] = rel(T["latitude_vector"], ref["latitude_vector"][emap])
    flip = np.where(esign < 0, math.pi, 0.0)
    errs["direction"] = float(np.max(np.abs(np.angle(np.exp(1j * (T["direction"] - ref["direction"][emap] - flip))))))
    errs["f_vec_h"] = rel(T["f_vec"][:ne] * esign, ref["f_vec"][:ne][emap])
    errs["f_vec_v"] = rel(T["f_vec"][ne:], ref["f_vec"][ne:][emap])
    # cell-edge incidence and inner-product weights
    adj_o, sgn_o = T["adjacent_vector_indices_h"].reshape(nc, 6), T["adjacent_signs_h"].reshape(nc, 6)
    adj_r = ref["adjacent_vector_indices_h"].astype(int).reshape(nc, 6)
    sgn_r = ref["adjacent_signs_h"].astype(int).reshape(nc, 6)
    ipw_o, ipw_r = T["inner_product_weights"].reshape(L, nc, 8), ref["inner_product_weights"].reshape(L, nc, 8)
    ipw_err, scale = 0.0, np.abs(ipw_r).max()
    for i in range(nc):
        I, n = cmap[i], 5 if i < 12 else 6
        assert {(emap[adj_o[i, j]], sgn_o[i, j] * esign[adj_o[i, j]]) for j in range(n)} == \
            {(adj_r[I, j], sgn_r[I, j]) for j in range(n)}, i
        slot = {emap[adj_o[i, j]]: j for j in range(n)}
        for j in range(n):
            ipw_err = max(ipw_err, float(np.max(np.abs(ipw_o[:, i, slot[adj_r[I, j]]] - ipw_r[:, I, j]))) / scale)
        ipw_err = max(ipw_err, float(np.max(np.abs(ipw_o[:, i, 6:] - ipw_r[:, I, 6:]))) / scale)
    errs["inner_product_weights"] = ipw_err
    # triangles: incidence, signs, dual orientation
    nt_ = len(T["latitude_scalar_dual"])
    vi_o, vs_o = T["vorticity_indices_triangles"].reshape(nt_, 3), T["vorticity_signs_triangles"].reshape(nt_, 3)
    vi_r = ref["vorticity_indices_triangles"].astype(int).reshape(nt_, 3)
    vs_r = ref["vorticity_signs_triangles"].astype(int).reshape(nt_, 3)
    for t in range(nt_):
        assert {(emap[vi_o[t, j]], vs_o[t, j] * esign[vi_o[t, j]]) for j in range(3)} == \
            {(vi_r[tmap[t], j], vs_r[tmap[t], j]) for j in range(3)}, t
    fd_r, td_r = ref["from_index_dual"].astype(int)[emap], ref["to_index_dual"].astype(int)[emap]
    fd_o, td_o = tmap[T["from_index_dual"]], tmap[T["to_index_dual"]]
    assert np.array_equal(np.where(esign > 0, fd_o, td_o), fd_r)
    assert np.array_equal(np.where(esign > 0, td_o, fd_o), td_r)
    # rhombus interpolation
    ri_o, rw_o = T["density_to_rhombi_indices"].reshape(ne, 4), T["density_to_rhombi_weights"].reshape(ne, 4)
    ri_r = ref["density_to_rhombi_indices"].astype(int).reshape(ne, 4)
    rw_r = ref["density_to_rhombi_weights"].reshape(ne, 4)
    r_err = 0.0
    for e in range(ne):
        do = {cmap[ri_o[e, j]]: rw_o[e, j] for j in range(4)}
        dr = {ri_r[emap[e], j]: rw_r[emap[e], j] for j in range(4)}
        assert set(do) == set(dr), e
        r_err = max(r_err, max(abs(do[k] - dr[k]) for k in do))
    errs["density_to_rhombi_weights"] = r_err
    # TRSK: (edge, modified-curl edge) -> signed weight
    tw_o, ti_o = T["trsk_weights"].reshape(ne, 10), T["trsk_indices"].reshape(ne, 10)
    tm_o = T["trsk_modified_curl_indices"].reshape(ne, 10)
    tw_r, ti_r = ref["trsk_weights"].reshape(ne, 10), ref["trsk_indices"].astype(int).reshape(ne, 10)
    tm_r = ref["trsk_modified_curl_indices"].astype(int).reshape(ne, 10)
    w_scale = np.abs(tw_r).max()
    tiny = 1e-9 * w_scale  # regular weights are above 1e-4 of the largest
    t_err = 0.0
    for e in range(ne):
        E = emap[e]
        do, dr = {}, {}
        for k in range(10):
            if abs(tw_o[e, k]) > tiny:
                kk = (emap[ti_o[e, k]], emap[tm_o[e, k]])
                do[kk] = do.get(kk, 0.0) + tw_o[e, k] * esign[e] * esign[ti_o[e, k]]
            if abs(tw_r[E, k]) > tiny:
                kk = (ti_r[E, k], tm_r[E, k])
                dr[kk] = dr.get(kk, 0.0) + tw_r[E, k]
        assert set(do) == set(dr), e
        t_err = max(t_err, max(abs(do[k] - dr[k]) for k in do) / w_scale)
    errs["trsk_weights"] = t_err
    ulp["latitude_scalar"] = ulps(T["latitude_scalar"], ref["latitude_scalar"][cmap])
    ulp["latitude_vector"] = ulps(T["latitude_vector"], ref["latitude_vector"][emap])
    worst = max(errs, key=errs.get)
    print(f"RES{res}, {n_iter} Lloyd iterations: worst {worst} {errs[worst]:.3g}")
    print(f"RES{res}, {n_iter} Lloyd iterations: (share of entries that differ, max ulps): " +
          ", ".join(f"{k} ({v[0]:.3f}, {v[1]:.3g})" for k, v in sorted(ulp.items())))
    # the TRSK weights sum kite areas; the reference's own zero weights carry
    # up to 2e-12 of its rounding, so they are held to 1e-11.  The positions
    # come out of the Lloyd iterations with the two builders' different
    # summation orders, so the differences grow with the number of cells:
    # the bounds at RES_ID 5 are five times those of RES_ID 3 and 4 (measured
    # there: 2.7e-12 for volumes and areas, 1.3e-11 for the TRSK weights)
    scale = 5.0 if res >= 5 else 1.0
    bad = {k: v for k, v in errs.items() if v > scale * (1e-11 if k == "trsk_weights" else 1e-12)}
    assert not bad, bad
    # lat-lon interpolation: equal except at distance ties
    lat_c, lon_c = ref["latitude_scalar"], ref["longitude_scalar"]
    li_o, lw_o = T["latlon_interpol_indices"].reshape(-1, 5), T["latlon_interpol_weights"].reshape(-1, 5)
    li_r, lw_r = ref["interpol_indices"].astype(int).reshape(-1, 5), ref["interpol_weights"].reshape(-1, 5)
    n_lat, n_lon = 2 << res, 4 << res
    ties = 0
    for p in range(len(li_o)):
        do = {cmap[li_o[p, j]]: lw_o[p, j] for j in range(5)}
        dr = {li_r[p, j]: lw_r[p, j] for j in range(5)}
        if set(do) == set(dr):
            assert max(abs(do[k] - dr[k]) for k in do) < scale * 1e-12
            continue
        # the cells picked by one side only must be as far from the point as
        # a cell picked by the other side only
        la = math.pi / 2 - 0.5 * math.pi / n_lat - (p // n_lon) * math.pi / n_lat
        lo = (p % n_lon) * 2 * math.pi / n_lon

        def dist(c):
            return 2 * math.asin(math.sqrt(0.5 - 0.5 * (math.cos(la) * math.cos(lat_c[c]) * math.cos(lon_c[c] - lo)
                                                        + math.sin(la) * math.sin(lat_c[c]))))
        only_o = sorted(dist(c) for c in set(do) - set(dr))
        only_r = sorted(dist(c) for c in set(dr) - set(do))
        assert len(only_o) == len(only_r) and np.allclose(only_o, only_r, rtol=1e-12, atol=0), p
        ties += 1
    assert ties <= len(li_o) // 50, ties
