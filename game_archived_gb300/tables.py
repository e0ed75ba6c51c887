"""Grid tables for the RKHEVI step.

``GridTables`` runs the C table builder (csrc/tables/gridgen.c) and keeps its
arrays as numpy arrays in the reference layout.  ``fill_grid`` writes them into
host Grid/Dualgrid structs exactly where the reference's set_grid_properties
(src/io/set_grid_properties.c:21-255) would have put them after reading the
grid file, including the quantities it derives on loading.

On-disk format (``GridTables.save`` / ``load``; the reference keeps its grid
in a netCDF file, src/io/set_grid_properties.c:21-255, which this image cannot
write).  A table file is

    8 bytes   magic b"GAMEGT01"
    8 bytes   little-endian uint64: length H of the header
    H bytes   UTF-8 JSON header: the build parameters (res_id, n_layers,
              n_oro_layers, toa, stretching, radius_rescale, n_lloyd,
              mountain), the array directory [name, dtype ("<i4" or "<f8"),
              element count, byte offset from the start of the payload] and
              "sha256", the SHA-256 digest of the payload
    payload   the arrays, each 64-byte aligned, in directory order

``load`` verifies the digest and refuses a file whose payload does not match
it; reading needs numpy only (no native library).  ``cached`` returns the
tables for a parameter set from a directory of such files, building and
saving them on the first request.
"""
import ctypes
import hashlib
import json
import math
import os

import numpy as np

from . import native

TABLE_MAGIC = b"GAMEGT01"

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

    # ------------------------------------------------------------ file format
    def params(self):
        return {"res_id": self.res_id, "n_layers": self.n_layers, "n_oro_layers": self.n_oro_layers,
                "toa": self.toa, "stretching": self.stretching, "radius_rescale": self.radius_rescale,
                "n_lloyd": self.n_lloyd, "mountain": list(self.mountain) if self.mountain is not None else None}

    def save(self, path):
        """writes the tables in the format of the module docstring (atomically:
        a temporary file renamed into place)"""
        directory, offset = [], 0
        for name, a in self.arrays.items():
            a = np.ascontiguousarray(a)
            dt = "<i4" if a.dtype.kind == "i" else "<f8"
            directory.append([name, dt, int(a.size), offset])
            nbytes = a.size * (4 if dt == "<i4" else 8)
            offset += (nbytes + 63) // 64 * 64
        payload = bytearray(offset)
        for (name, dt, count, off) in directory:
            b = np.ascontiguousarray(self.arrays[name], dtype=np.dtype(dt)).tobytes()
            payload[off:off + len(b)] = b
        header = dict(self.params(), arrays=directory, sha256=hashlib.sha256(payload).hexdigest())
        hb = json.dumps(header, sort_keys=True).encode()
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "wb") as f:
            f.write(TABLE_MAGIC)
            f.write(len(hb).to_bytes(8, "little"))
            f.write(hb)
            f.write(payload)
        os.replace(tmp, path)
        return header["sha256"]

    @classmethod
    def load(cls, path):
        """reads a table file; raises ValueError if it is not one or if its
        payload does not match its digest"""
        with open(path, "rb") as f:
            if f.read(8) != TABLE_MAGIC:
                raise ValueError(f"{path}: not a grid table file")
            hlen = int.from_bytes(f.read(8), "little")
            header = json.loads(f.read(hlen).decode())
            payload = f.read()
        if hashlib.sha256(payload).hexdigest() != header["sha256"]:
            raise ValueError(f"{path}: payload does not match its SHA-256 digest")
        t = cls.__new__(cls)
        t.arrays = {}
        for name, dt, count, off in header["arrays"]:
            t.arrays[name] = np.frombuffer(payload, dtype=np.dtype(dt), count=count, offset=off).astype(
                np.int32 if dt == "<i4" else np.float64)
        t.res_id, t.n_layers, t.n_oro_layers = header["res_id"], header["n_layers"], header["n_oro_layers"]
        t.toa, t.stretching, t.radius_rescale = header["toa"], header["stretching"], header["radius_rescale"]
        t.n_lloyd = header["n_lloyd"]
        t.mountain = tuple(header["mountain"]) if header["mountain"] is not None else None
        t.radius = t.radius_rescale * 6371000.789927
        t.nc = len(t.arrays["latitude_scalar"])
        t.ne = len(t.arrays["from_index"])
        t.nt = len(t.arrays["latitude_scalar_dual"])
        t.sha256 = header["sha256"]
        return t


def table_file_name(res_id, n_layers=26, n_oro_layers=DEFAULT_ORO_LAYERS, toa=DEFAULT_TOA,
                    stretching=DEFAULT_STRETCHING, radius_rescale=1.0, n_lloyd=None, mountain=None):
    """the file name of a parameter set: RES, layers and Lloyd iterations,
    plus a digest of every parameter"""
    if n_lloyd is None:
        n_lloyd = 2000 if res_id <= 6 else 500
    key = json.dumps([res_id, n_layers, n_oro_layers, as_float32(toa), as_float32(stretching),
                      as_float32(radius_rescale), n_lloyd, list(mountain) if mountain is not None else None])
    return f"R{res_id}_L{n_layers}_lloyd{n_lloyd}_{hashlib.sha256(key.encode()).hexdigest()[:16]}.gtab"


def cached(directory, res_id, **kw):
    """the tables of this parameter set from directory, built and saved there
    on the first request"""
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, table_file_name(res_id, **kw))
    if os.path.exists(path):
        try:
            return GridTables.load(path)
        except ValueError:
            os.remove(path)
    t = GridTables(res_id, **kw)
    t.sha256 = t.save(path)
    return t


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
