"""The library's writers of write_out's netCDF files against the reference's.

The reference's write_out runs through the recording netCDF stand-in (every
dimension and variable definition, units attribute and array recorded); the
library's writers (csrc/common/ncwrite.c) write the same fields, computed by
the oracle on a clone of the same model, to real files, which scipy reads
back.  The files must define the same dimensions and variables, in the same
order, with the same shapes and units, and hold the same bytes.
"""
import numpy as np
import pytest

import refbind
from helpers import clone, output_scenario
from ncfiles import read_file, write_files
from oracle import bind

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference sources not present")


@pytest.mark.parametrize("res,moist,case,mountain", [(3, 1, "tracers", True), (3, 0, "std_wind_tpert", False)])
def test_output_files_equal_reference(res, moist, case, mountain, tmp_path):
    m, wl, nw = output_scenario(res, moist, case, mountain)
    m_orc = clone(m)
    ref = refbind.write_out(refbind.Reference(m), m.state_new, wl, nw, str(tmp_path / "ref"))
    orc = bind.Oracle(m_orc)
    o = bind.write_out_fields(orc, m_orc.state_new, wl, nw)
    d = m_orc.diagnostics
    fields = dict(o)
    fields.update(densities=m_orc.state_new["rho"], temperature=d["temperature"], wind=m_orc.state_new["wind"],
                  tke=m_orc.irrev["tke"], t_soil=m_orc.state_new["temperature_soil"])
    out = tmp_path / "ours"
    out.mkdir()
    paths = write_files(m.layout, fields, str(out), "run+3600s")
    for kind, path in paths.items():
        defs, data = read_file(path)
        ref_defs = [dd[1:] for dd in ref["defs"] if dd[0] == kind]
        assert defs == ref_defs, kind
        ref_data = ref[kind if kind != "model_levels" else "model_levels"]
        assert sorted(data) == sorted(ref_data), kind
        for name, values in data.items():
            assert np.array_equal(values, ref_data[name], equal_nan=True), (kind, name)
