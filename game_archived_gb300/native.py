"""ctypes bindings of the two native libraries.

``tables()`` loads libgame_tables.so (grid-table builder + run-time struct
layout; host code).  ``gpu()`` loads libgame_gb300.so, the CUDA library behind
include/game_gb300.h.  Neither falls back to anything: a missing library is an
error that names the build step.
"""
import ctypes
import os

from . import build as _build

_tables = None
_gpu = None

c_int, c_long, c_double, c_void_p, c_char_p, c_size_t = (
    ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t)


class GameMember(ctypes.Structure):
    _fields_ = [("name", c_char_p), ("is_int", c_int), ("count", c_long), ("offset", c_size_t)]


class GameDims(ctypes.Structure):
    _fields_ = [("res_id", c_int), ("n_layers", c_int), ("moisture_on", c_int),
                ("n_cells", c_long), ("n_edges", c_long), ("n_triangles", c_long),
                ("n_scalars", c_long), ("n_vectors", c_long), ("n_dual_vectors", c_long),
                ("n_curl", c_long), ("vpl", c_long), ("dpl", c_long),
                ("n_constituents", c_int), ("n_condensed", c_int), ("n_soil", c_int),
                ("n_latlon", c_long)]


def _declare_layout(lib):
    lib.game_dims_init.argtypes = [ctypes.POINTER(GameDims), c_int, c_int, c_int]
    lib.game_dims_init.restype = c_int
    lib.game_layout_count.argtypes = [c_int]
    lib.game_layout_count.restype = c_int
    lib.game_layout_member.argtypes = [ctypes.POINTER(GameDims), c_int, c_int, ctypes.POINTER(GameMember)]
    lib.game_layout_member.restype = c_int
    lib.game_layout_sizeof.argtypes = [ctypes.POINTER(GameDims), c_int]
    lib.game_layout_sizeof.restype = c_size_t


def tables():
    """libgame_tables.so, built on first use if absent (host C only)."""
    global _tables
    if _tables is None:
        if not os.path.exists(_build.TABLES_LIB):
            _build.build_tables()
        lib = ctypes.CDLL(_build.TABLES_LIB)
        lib.gt_build.restype = c_void_p
        lib.gt_build.argtypes = [c_int, c_int, c_int, c_double, c_double, c_double, c_int, c_int,
                                 c_void_p, c_int]
        lib.gt_last_error.restype = c_char_p
        lib.gt_count.argtypes = [c_void_p]
        lib.gt_count.restype = c_int
        lib.gt_info.argtypes = [c_void_p, c_int, ctypes.POINTER(c_char_p), ctypes.POINTER(c_int),
                                ctypes.POINTER(c_long), ctypes.POINTER(c_void_p)]
        lib.gt_info.restype = c_int
        lib.gt_free.argtypes = [c_void_p]
        lib.gt_free.restype = None
        _declare_layout(lib)
        _tables = lib
    return _tables


def gpu():
    """libgame_gb300.so; raises if it has not been built (no fallback)."""
    global _gpu
    if _gpu is None:
        if not os.path.exists(_build.GPU_LIB):
            raise RuntimeError(
                f"{_build.GPU_LIB} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA path has no CPU fallback)")
        lib = ctypes.CDLL(_build.GPU_LIB)
        from . import abi
        abi.declare(lib)
        _gpu = lib
    return _gpu
