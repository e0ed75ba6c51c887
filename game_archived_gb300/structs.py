"""Host-side mirrors of GAME's data structures.

``Layout`` gives, for one (RES_ID, NO_OF_LAYERS, MOISTURE_ON) configuration,
the byte offset, element type and count of every member of Grid, Dualgrid,
State, Diagnostics, Forcings, Irreversible_quantities and Config
(src/game_types.h:62-238), computed by the same C code the GPU library uses.
``HostStruct`` is one such struct in host memory, with numpy views of its
members; its address is what the C ABI (include/game_gb300.h) takes.
"""
import ctypes

import numpy as np

from . import native

STRUCT_IDS = {"grid": 0, "dualgrid": 1, "state": 2, "diagnostics": 3, "forcings": 4, "irrev": 5, "config": 6}


class Layout:
    def __init__(self, res_id, n_layers=26, moisture_on=0):
        lib = native.tables()
        self.dims = native.GameDims()
        if lib.game_dims_init(ctypes.byref(self.dims), res_id, n_layers, moisture_on) != 0:
            raise ValueError("invalid grid configuration")
        self.res_id, self.n_layers, self.moisture_on = res_id, n_layers, moisture_on
        d = self.dims
        self.nc, self.ne, self.nt, self.nl = d.n_cells, d.n_edges, d.n_triangles, n_layers
        self.n_scalars, self.n_vectors, self.n_dual_vectors = d.n_scalars, d.n_vectors, d.n_dual_vectors
        self.vpl, self.dpl, self.n_curl = d.vpl, d.dpl, d.n_curl
        self.n_const, self.n_cond = d.n_constituents, d.n_condensed
        self.n_latlon = d.n_latlon
        self.members = {}
        self.sizes = {}
        for name, sid in STRUCT_IDS.items():
            mem = {}
            m = native.GameMember()
            for i in range(lib.game_layout_count(sid)):
                lib.game_layout_member(ctypes.byref(self.dims), sid, i, ctypes.byref(m))
                mem[m.name.decode()] = (bool(m.is_int), int(m.count), int(m.offset))
            self.members[name] = mem
            self.sizes[name] = int(lib.game_layout_sizeof(ctypes.byref(self.dims), sid))

    LAYOUT_KEYS = ("res_id", "n_layers", "moisture_on", "nc", "ne", "nt", "nl", "n_scalars", "n_vectors",
                   "n_dual_vectors", "vpl", "dpl", "n_curl", "n_const", "n_cond", "n_latlon")

    def to_dict(self):
        """the layout as plain data (sizes, and every member's type, count and
        offset), for a process that reads it without the native library"""
        d = {k: getattr(self, k) for k in self.LAYOUT_KEYS}
        d["members"] = {kind: {n: list(v) for n, v in mem.items()} for kind, mem in self.members.items()}
        d["sizes"] = dict(self.sizes)
        return d

    @classmethod
    def from_dict(cls, d):
        lay = cls.__new__(cls)
        for k in cls.LAYOUT_KEYS:
            setattr(lay, k, d[k])
        lay.members = {kind: {n: (bool(v[0]), int(v[1]), int(v[2])) for n, v in mem.items()}
                       for kind, mem in d["members"].items()}
        lay.sizes = {k: int(v) for k, v in d["sizes"].items()}
        lay.dims = None
        return lay


class HostStruct:
    """One reference struct in host memory.  ``buffer`` may be supplied (for
    example pinned memory); otherwise a zeroed, 4 KiB-aligned numpy buffer is
    allocated, as the reference calloc()s its structs (src/coordinator.c:36-46)."""

    def __init__(self, layout, kind, buffer=None):
        self.layout, self.kind = layout, kind
        size = layout.sizes[kind]
        if buffer is None:
            raw = np.zeros(size + 4096, dtype=np.uint8)
            off = (-raw.ctypes.data) % 4096
            self._raw = raw
            self.buf = raw[off:off + size]
        else:
            self._raw = buffer
            self.buf = np.frombuffer(buffer, dtype=np.uint8, count=size) if not isinstance(buffer, np.ndarray) \
                else buffer[:size]
        self._views = {}

    @property
    def ptr(self):
        return self.buf.ctypes.data

    def __getitem__(self, name):
        v = self._views.get(name)
        if v is None:
            is_int, count, off = self.layout.members[self.kind][name]
            dt = np.int32 if is_int else np.float64
            v = self.buf[off:off + count * dt().itemsize].view(dt)
            self._views[name] = v
        return v

    def __setitem__(self, name, value):
        v = self[name]
        v[...] = value

    def copy_from(self, other):
        self.buf[...] = other.buf

    def clone(self):
        s = HostStruct(self.layout, self.kind)
        s.buf[...] = self.buf
        return s


class Model:
    """The set of structs one manage_rkhevi call takes (src/coordinator.c:36-46)."""

    KINDS = ("grid", "dualgrid", "state_old", "state_new", "state_tendency", "diagnostics", "forcings",
             "irrev", "config")

    def __init__(self, layout, buffers=None):
        self.layout = layout
        buffers = buffers or {}
        for k in self.KINDS:
            kind = "state" if k.startswith("state") else k
            setattr(self, k, HostStruct(layout, kind, buffers.get(k)))


class ConfigIo(ctypes.Structure):
    """the reference's Config_io (src/game_types.h:240-258): output switches
    and the run id of write_out; its layout does not depend on the grid"""
    _fields_ = [(n, ctypes.c_int) for n in (
        "grib_output_switch", "netcdf_output_switch", "pressure_level_output_switch", "model_level_output_switch",
        "surface_output_switch", "write_out_interval", "write_out_integrals", "year", "month", "day", "hour")] + [
        ("run_id", ctypes.c_char * 100), ("month_string", ctypes.c_char * 3), ("day_string", ctypes.c_char * 3),
        ("hour_string", ctypes.c_char * 3), ("ideal_input_id", ctypes.c_int)]
