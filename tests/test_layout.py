"""Run-time struct layout (csrc/common/layout.c) against the compiler's
offsetof/sizeof of the reference's own game_types.h (oracle/ref_harness.c),
for every member of every struct the C ABI takes."""
import ctypes

import pytest

from game_archived_gb300 import structs

refbind = pytest.importorskip("refbind")

STRUCT_IDS = structs.STRUCT_IDS


def test_layout_is_consistent():
    for res, moist in ((3, 0), (5, 1), (7, 1)):
        lay = structs.Layout(res, 26, moist)
        for kind, members in lay.members.items():
            end = 0
            for name, (is_int, count, off) in sorted(members.items(), key=lambda kv: kv[1][2]):
                assert off >= end, (kind, name)
                assert off % (4 if is_int else 8) == 0
                end = off + count * (4 if is_int else 8)
            assert lay.sizes[kind] >= end and lay.sizes[kind] % 8 == 0


@pytest.mark.skipif(not refbind.available(), reason="reference sources not present")
@pytest.mark.parametrize("res,moist", [(3, 0), (3, 1), (4, 0), (4, 1)])
def test_layout_matches_reference_compiler(res, moist):
    from oracle import build_ref
    lib = ctypes.CDLL(build_ref.build(res, moist))
    lib.ref_offsetof.restype = ctypes.c_long
    lib.ref_offsetof.argtypes = [ctypes.c_int, ctypes.c_char_p]
    lib.ref_sizeof.restype = ctypes.c_long
    lib.ref_sizeof.argtypes = [ctypes.c_int]
    lay = structs.Layout(res, 26, moist)
    for kind, sid in STRUCT_IDS.items():
        assert lay.sizes[kind] == lib.ref_sizeof(sid), kind
        for name, (_, _, off) in lay.members[kind].items():
            assert lib.ref_offsetof(sid, name.encode()) == off, (kind, name)


def test_config_io_layout_matches_reference():
    """structs.ConfigIo against the reference compiler's offsetof/sizeof"""
    import ctypes
    from oracle import build_ref
    from game_archived_gb300.structs import ConfigIo
    if not build_ref.available():
        import pytest
        pytest.skip("reference sources not present")
    lib = ctypes.CDLL(build_ref.build(3, 0))
    lib.ref_config_io_offsetof.restype = ctypes.c_long
    lib.ref_config_io_offsetof.argtypes = [ctypes.c_char_p]
    lib.ref_config_io_sizeof.restype = ctypes.c_long
    for name, _ in ConfigIo._fields_:
        assert getattr(ConfigIo, name).offset == lib.ref_config_io_offsetof(name.encode()), name
    assert ctypes.sizeof(ConfigIo) == lib.ref_config_io_sizeof()
