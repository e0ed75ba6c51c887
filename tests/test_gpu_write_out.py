"""write_out and write_out_integral (the reference's output entry points) on
the GPU: the files they write against the same files written from the
oracle's fields by the library's writers (whose files equal the reference's
byte for byte, tests/test_output_files.py): the same dimensions, variables,
units and order; the computed fields within 1e-11 of the oracle relative to
each field's largest magnitude, the copied State fields bit for bit.  A
device-resident run writes byte-identical files.  GRIB output is refused."""
import ctypes
import os

import numpy as np
import pytest

from game_archived_gb300 import abi
from game_archived_gb300.structs import ConfigIo
from helpers import clone, output_scenario
from ncfiles import read_file, write_files
from oracle import bind

pytestmark = pytest.mark.gpu
COPIED = {"densities", "wind", "t_soil", "tke", "pressure_levels"}


def config_io(grib=0):
    return ConfigIo(grib, 1, 1, 1, 1, 3600, 1, 2000, 1, 1, 0, b"gpu", b"01", b"01", b"00", 0)


def call_write_out(g, m, wl, nw, directory, cio):
    cwd = os.getcwd()
    os.chdir(directory)
    try:
        return g.lib.write_out(m.state_new.ptr, wl.ctypes.data if wl is not None else None, nw, 0.0, 3600.0,
                               m.diagnostics.ptr, m.forcings.ptr, m.grid.ptr, m.dualgrid.ptr, ctypes.byref(cio),
                               m.config.ptr, m.irrev.ptr)
    finally:
        os.chdir(cwd)


def close(a, b, tol=1e-11):
    miss_a, miss_b = a == 9999, b == 9999
    if not np.array_equal(miss_a, miss_b):
        return False
    a, b = a[~miss_b], b[~miss_b]
    s = np.max(np.abs(b)) if b.size else 0
    return b.size == 0 or (np.max(np.abs(a - b)) <= tol * s if s else np.array_equal(a, b))


@pytest.mark.parametrize("moist,case", [(1, "tracers"), (0, "std_wind_tpert")])
def test_write_out_files_match_oracle(moist, case, tmp_path):
    m, wl, nw = output_scenario(3, moist, case, True)
    m_orc = clone(m)
    orc = bind.Oracle(m_orc)
    o = bind.write_out_fields(orc, m_orc.state_new, wl, nw)
    d = m_orc.diagnostics
    fields = dict(o)
    fields.update(densities=m_orc.state_new["rho"], temperature=d["temperature"], wind=m_orc.state_new["wind"],
                  tke=m_orc.irrev["tke"], t_soil=m_orc.state_new["temperature_soil"])
    (tmp_path / "want").mkdir()
    (tmp_path / "got").mkdir()
    want = write_files(m.layout, fields, str(tmp_path / "want"), "gpu+3600s")
    g = abi.GpuModel(m, abi.FP64)
    try:
        assert call_write_out(g, m, wl, nw, str(tmp_path / "got"), config_io()) == 0, \
            g.lib.game_gpu_last_error().decode()
    finally:
        g.close()
    for kind, path in want.items():
        got_path = str(tmp_path / "got" / os.path.basename(path))
        defs_w, data_w = read_file(path)
        defs_g, data_g = read_file(got_path)
        assert defs_g == defs_w, kind
        for name in data_w:
            if name in COPIED:
                assert np.array_equal(data_g[name], data_w[name]), (kind, name)
            else:
                assert close(data_g[name], data_w[name]), (kind, name)
    assert np.array_equal(m.state_new["theta_v_pert"], m_orc.state_new["theta_v_pert"])


def test_write_out_resident_files_identical_and_grib_refused(tmp_path):
    m0, wl, nw = output_scenario(3, 1, "tracers", True)
    blobs = []
    for resident in (False, True):
        m = clone(m0)
        out = tmp_path / ("res" if resident else "host")
        out.mkdir()
        g = abi.GpuModel(m, abi.FP64, resident=resident)
        try:
            if resident:
                g.sync_to_device(m.state_new)
            assert call_write_out(g, m, wl, nw, str(out), config_io()) == 0, g.lib.game_gpu_last_error().decode()
            if not resident:
                assert call_write_out(g, m, wl, nw, str(out), config_io(grib=1)) != 0
                assert "GRIB" in g.lib.game_gpu_last_error().decode()
        finally:
            g.close()
        blobs.append({p: open(out / p, "rb").read() for p in sorted(os.listdir(out))})
    assert blobs[0].keys() == blobs[1].keys() and len(blobs[0]) == 3
    for name in blobs[0]:
        assert blobs[0][name] == blobs[1][name], name


def test_write_out_integral_files(tmp_path):
    m, _, _ = output_scenario(3, 1, "tracers", False)
    m_orc = clone(m)
    orc = bind.Oracle(m_orc)
    t = orc.temperature(m_orc.state_new)
    want = {i: orc.write_out_integral(m_orc.state_new, i, t) for i in range(3)}
    g = abi.GpuModel(m, abi.FP64)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        for i in range(3):
            for _ in range(2):
                assert g.lib.write_out_integral(m.state_new.ptr, 7200.0, m.grid.ptr, m.dualgrid.ptr,
                                                m.diagnostics.ptr, i) == 0
    finally:
        os.chdir(cwd)
        g.close()
    for i, name in enumerate(("masses", "potential_temperature_density", "energy")):
        lines = open(tmp_path / name).read().splitlines()
        assert len(lines) == 2 and lines[0] == lines[1]
        vals = [float(x) for x in lines[0].split("\t")]
        assert vals[0] == 7200.0
        assert np.allclose(vals[1:], want[i], rtol=1e-9, atol=1e-6), (name, vals, want[i])


def test_interpolation_t_is_the_weighted_blend():
    m, _, _ = output_scenario(3, 0, "std_wind_tpert", False)
    g = abi.GpuModel(m, abi.FP64)
    try:
        a = clone(m)
        g.linear_combine_two_states(m.state_old, m.state_new, a.state_tendency, 1.0 - 0.25, 0.25)
        assert g.lib.interpolation_t(m.state_old.ptr, m.state_new.ptr, m.state_tendency.ptr, 0.0, 400.0, 100.0,
                                     m.grid.ptr) == 0
    finally:
        g.close()
    for f in ("rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind"):
        assert np.array_equal(m.state_tendency[f], a.state_tendency[f]), f
