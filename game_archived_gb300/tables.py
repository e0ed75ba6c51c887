"""Grid tables for the RKHEVI step.

``GridTables`` runs the C table builder (csrc/tables/gridgen.c) and keeps its
arrays as numpy arrays in the reference layout.  ``fill_grid`` writes them into
host Grid/Dualgrid structs exactly where the reference's set_grid_properties
(src/io/set_grid_properties.c:21-255) would have put them after reading the
grid file, including the quantities it derives on loading.
"""
import ctypes
import math

import numpy as np

from . import native

# grid_generator/run_script.sh:16-18 defaults
DEFAULT_TOA = 41152.0
DEFAULT_STRETCHING = 1.3
DEFAULT_ORO_LAYERS = 23


def as_float32(x):
    """the value the reference's generator sees for a command-line argument
    it parses with strtof (grid_generator/src/coordinator.c:51-56): x rounded
    to single precision"""
    return float(np.float32(x))


class GridTables:
    def __init__(self, res_id, n_layers=26, n_oro_layers=DEFAULT_ORO_LAYERS, toa=DEFAULT_TOA,
                 stretching=DEFAULT_STRETCHING, radius_rescale=1.0, n_lloyd=None, mountain=None, n_threads=0):
        """mountain: None (flat) or (height_m, half_width_m, lat_deg, lon_deg).
        toa, stretching and radius_rescale are rounded to single precision
        first, as the reference's generator reads them."""
        toa, stretching, radius_rescale = as_float32(toa), as_float32(stretching), as_float32(radius_rescale)
        if n_lloyd is None:
            n_lloyd = 2000 if res_id <= 6 else 500
        lib = native.tables()
        params = None
        kind = 0
        if mountain is not None:
            kind = 1
            h, hw, lat, lon = mountain
            params = (ctypes.c_double * 4)(h, hw, math.radians(lat), math.radians(lon))
        handle = lib.gt_build(res_id, n_layers, n_oro_layers, toa, stretching, radius_rescale, n_lloyd, kind,
                              ctypes.cast(params, ctypes.c_void_p) if params is not None else None, n_threads)
        if not handle:
            raise RuntimeError("grid table builder failed: " + lib.gt_last_error().decode())
        self.arrays = {}
        try:
            name = ctypes.c_char_p()
            typ, n, ptr = ctypes.c_int(), ctypes.c_long(), ctypes.c_void_p()
            for i in range(lib.gt_count(handle)):
                lib.gt_info(handle, i, ctypes.byref(name), ctypes.byref(typ), ctypes.byref(n), ctypes.byref(ptr))
                ct = ctypes.c_int if typ.value == 1 else ctypes.c_double
                buf = (ct * n.value).from_address(ptr.value)
                self.arrays[name.value.decode()] = np.array(buf, copy=True)
        finally:
            lib.gt_free(handle)
        self.res_id, self.n_layers, self.n_oro_layers = res_id, n_layers, n_oro_layers
        self.toa, self.stretching, self.radius_rescale, self.n_lloyd = toa, stretching, radius_rescale, n_lloyd
        self.radius = radius_rescale * 6371000.789927
        self.mountain = mountain
        self.nc = len(self.arrays["latitude_scalar"])
        self.ne = len(self.arrays["from_index"])
        self.nt = len(self.arrays["latitude_scalar_dual"])

    def __getitem__(self, k):
        return self.arrays[k]


GRID_MEMBERS = ["normal_distance", "volume", "area", "z_scalar", "z_vector", "gravity_potential", "gravity_m",
                "slope", "theta_v_bg", "exner_bg", "exner_bg_grad", "layer_thickness", "trsk_indices",
                "trsk_modified_curl_indices", "from_index", "to_index", "adjacent_vector_indices_h",
                "adjacent_signs_h", "density_to_rhombi_indices", "latitude_scalar", "longitude_scalar",
                "inner_product_weights", "direction", "density_to_rhombi_weights", "trsk_weights",
                "latlon_interpol_indices", "latlon_interpol_weights"]


def fill_grid(tables, grid, dualgrid):
    """Writes the tables into host Grid / Dualgrid structs (reference layout)."""
    for k in GRID_MEMBERS:
        grid[k] = tables[k]
    grid["no_of_oro_layers"] = tables.n_oro_layers
    grid["toa"] = tables.toa
    grid["radius"] = tables.radius
    grid["stretching_parameter"] = tables.stretching
    grid["oro_id"] = 0 if tables.mountain is None else 1
    # surface properties: sea everywhere, the values the reference's grid
    # generator gives sea cells (grid_generator/src/phys_sfc_properties.c:155-
    # 199: albedo of water, rho*c_p of water, sea roughness length, thermal
    # conductivity of water) and the soil grid (set_grid_properties.c:224-252)
    grid["is_land"] = 0
    grid["sfc_albedo"] = 0.06
    grid["sfc_rho_c"] = 1024.0 * 4184.0
    grid["roughness_length"] = max(0.0001, 0.08)
    grid["t_conduc_soil"] = 1.4e-7
    grid["z_t_const"] = -10.0
    grid["t_const_soil"] = 273.15 + 25.0 * np.cos(2.0 * tables["latitude_scalar"])
    sigma_soil = 0.352
    n_soil = len(grid["z_soil_center"])
    zi = np.zeros(n_soil + 1)
    for i in range(1, n_soil + 1):
        zi[i] = zi[i - 1] + sigma_soil ** (n_soil - i)
    zi[1:] = (-10.0 / zi[n_soil]) * zi[1:]
    grid["z_soil_interface"] = zi
    grid["z_soil_center"] = 0.5 * (zi[:-1] + zi[1:])
    nc, nl = tables.nc, tables.n_layers
    area = tables["area"]
    # mean cell area -> effective horizontal resolution (src/coordinator.c:160-170)
    cell_area_sum = 0.0
    vpl = tables.nc + tables.ne
    for lev in range(nl + 1):
        cell_area_sum += area[lev * vpl: lev * vpl + nc].sum()
    grid["mean_velocity_area"] = 2.0 / 3.0 * cell_area_sum / ((nl + 1) * nc)
    grid["eff_hor_res"] = math.sqrt(cell_area_sum / ((nl + 1) * nc))
    n_dv = len(tables["area_dual"])
    dualgrid["area"][:n_dv] = tables["area_dual"]
    dualgrid["z_vector"] = tables["z_vector_dual"]
    dualgrid["normal_distance"] = tables["normal_distance_dual"]
    dualgrid["from_index"] = tables["from_index_dual"]
    dualgrid["to_index"] = tables["to_index_dual"]
    dualgrid["vorticity_indices_triangles"] = tables["vorticity_indices_triangles"]
    dualgrid["vorticity_signs_triangles"] = tables["vorticity_signs_triangles"]
    dualgrid["f_vec"] = tables["f_vec"]
