"""Builds the reference's own RKHEVI C code into oracle/_ref/ (test infrastructure).

The GAME reference (MHBalsmeier/GAME_archived) is plain C99 + OpenMP.  Its grid
size, layer count and moisture switch are compile-time enums in
src/game_types.h:12-60, and every source file includes that header with a
relative path ("../game_types.h"), so an -I flag cannot override it.  This
recipe therefore builds a tree of symbolic links to the unmodified reference
sources under oracle/_ref/build_R<res>_M<moist>/, where only game_types.h is a
generated file (the reference header with the three enum values replaced), and
compiles it with gcc:

* src/time_stepping, src/spatial_operators, src/constituents,
  src/subgrid_scale, src/radiation/{held_suar,manage_radiation_calls}.c;
* grid_generator/src/{geodesy,index_helpers}.c stand in for the un-vendored
  geos95 library (they define passive_turn, find_min_index and rad2deg);
* grid_generator/src/interpolate_ll.c (the lat-lon interpolation tables);
* src/io/{write_output,spatial_ops_for_output}.c, the output diagnostics,
  against stand-ins for the netCDF and ecCodes headers (oracle/ref_stubs/)
  whose definitions (oracle/ref_io_stubs.c) write no file but record the
  arrays handed to the writers;
* the Fortran radiation coupler is replaced by a stub that aborts if called
  (radiation is off in every configuration used here);
* oracle/ref_harness.c (ours) exports sizeof/offsetof of the reference structs
  so the run-time layout can be checked against the compiler's.

Output: oracle/_ref/libgame_ref_v<version>_R<res>_M<moist>.so.

build_gridgen compiles the reference's grid generator program
(grid_generator/src/*.c) the same way into
oracle/_ref/libgame_refgrid_v<version>_R<res>_L<layers>.so; its main runs
in-process and the tables it would write to its netCDF grid file are
recorded by the stand-in.  Nothing is copied into the
repository; oracle/_ref/ is git-ignored.  Runs only where the reference tree
exists (this build container), never on the GPU host.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $GAME_REFERENCE_ROOT, else a directory named
# "reference" beside the repository's root
REF_ROOT = os.environ.get("GAME_REFERENCE_ROOT",
                          os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))
OUT = os.path.join(HERE, "_ref")

SRC_DIRS = ["time_stepping", "spatial_operators", "constituents", "subgrid_scale"]
RAD_FILES = ["held_suar.c", "manage_radiation_calls.c"]
GEOS_FILES = ["geodesy.c", "index_helpers.c"]
# the grid generator's lat-lon interpolation table builder
GRIDGEN_FILES = ["interpolate_ll.c"]
# the output diagnostics (write_out) and the operators only output uses
IO_FILES = ["write_output.c", "spatial_ops_for_output.c"]
# bumped whenever the set of compiled sources changes, so that stale
# libraries are not reused
BUILD_VERSION = 5

GEOS95_H = """/* declarations of the geos95 functions the model uses; their definitions
   come from grid_generator/src/geodesy.c and index_helpers.c */
int passive_turn(double, double, double, double *, double *);
int find_min_index(double [], int);
double rad2deg(double);
"""

RAD_STUB_C = """#include <stdio.h>
#include <stdlib.h>
void calc_radiative_flux_convergence(double a[], double b[], double c[], double d[], double e[], double f[],
    double g[], double h[], double i[], double j[], double k[], int *l, int *m, int *n, int *o, double *p)
{
    (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k;
    (void)l; (void)m; (void)n; (void)o; (void)p;
    fprintf(stderr, "radiation is not available in this build\\n");
    abort();
}
void radiation_init(void) {}
"""


def available():
    return os.path.isfile(os.path.join(REF_ROOT, "src", "game_types.h"))


def lib_path(res_id, moisture_on):
    return os.path.join(OUT, f"libgame_ref_v{BUILD_VERSION}_R{res_id}_M{moisture_on}.so")


def _link(src, dst):
    if os.path.lexists(dst):
        os.remove(dst)
    os.symlink(src, dst)


def build(res_id, moisture_on, n_layers=26, force=False):
    """Builds (or reuses) the reference library for one enum configuration."""
    if not available():
        raise RuntimeError("reference sources not present")
    out = lib_path(res_id, moisture_on)
    if os.path.exists(out) and not force:
        return out
    bdir = os.path.join(OUT, f"build_R{res_id}_M{moisture_on}")
    src = os.path.join(bdir, "src")
    os.makedirs(src, exist_ok=True)
    # generated game_types.h: the reference header with the enum values replaced
    with open(os.path.join(REF_ROOT, "src", "game_types.h")) as f:
        hdr = f.read()
    hdr = re.sub(r"RES_ID = \d+", f"RES_ID = {res_id}", hdr)
    hdr = re.sub(r"NO_OF_LAYERS = \d+", f"NO_OF_LAYERS = {n_layers}", hdr)
    hdr = re.sub(r"MOISTURE_ON = \d+", f"MOISTURE_ON = {moisture_on}", hdr)
    gen = os.path.join(src, "game_types.h")
    if os.path.lexists(gen):
        os.remove(gen)
    with open(gen, "w") as f:
        f.write(hdr)
    _link(os.path.join(REF_ROOT, "src", "game_constants.h"), os.path.join(src, "game_constants.h"))
    sources = []
    for d in SRC_DIRS + ["radiation", "io"]:
        os.makedirs(os.path.join(src, d), exist_ok=True)
        for name in os.listdir(os.path.join(REF_ROOT, "src", d)):
            if name.endswith(".h") or (name.endswith(".c") and (d in SRC_DIRS or name in RAD_FILES or name in IO_FILES)):
                _link(os.path.join(REF_ROOT, "src", d, name), os.path.join(src, d, name))
                if name.endswith(".c"):
                    sources.append(os.path.join(src, d, name))
    gg = os.path.join(bdir, "grid_generator", "src")
    os.makedirs(gg, exist_ok=True)
    for name in os.listdir(os.path.join(REF_ROOT, "grid_generator", "src")):
        if name.endswith(".h") or name in GEOS_FILES + GRIDGEN_FILES:
            _link(os.path.join(REF_ROOT, "grid_generator", "src", name), os.path.join(gg, name))
            if name in GEOS_FILES + GRIDGEN_FILES:
                sources.append(os.path.join(gg, name))
    inc = os.path.join(bdir, "include")
    os.makedirs(inc, exist_ok=True)
    with open(os.path.join(inc, "geos95.h"), "w") as f:
        f.write(GEOS95_H)
    stub = os.path.join(bdir, "radiation_stub.c")
    with open(stub, "w") as f:
        f.write(RAD_STUB_C)
    harness = [os.path.join(HERE, "ref_harness.c"), os.path.join(HERE, "ref_io_stubs.c")]
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w",
           "-I", inc, "-I", os.path.join(HERE, "ref_stubs"), "-I", src, "-o", out] + sources + [stub] + harness + ["-lm"]
    subprocess.run(cmd, check=True)
    return out


def gridgen_path(res_id, n_layers=26):
    return os.path.join(OUT, f"libgame_refgrid_v{BUILD_VERSION}_R{res_id}_L{n_layers}.so")


def build_gridgen(res_id, n_layers=26, force=False):
    """Builds (or reuses) the reference's grid generator (every source of
    grid_generator/src, its main renamed ref_gridgen_main) with the netCDF
    stand-in, which records every table the generator writes to its grid
    file instead of writing it."""
    if not available():
        raise RuntimeError("reference sources not present")
    out = gridgen_path(res_id, n_layers)
    if os.path.exists(out) and not force:
        return out
    bdir = os.path.join(OUT, f"build_grid_R{res_id}_L{n_layers}")
    src = os.path.join(bdir, "src")
    os.makedirs(src, exist_ok=True)
    with open(os.path.join(REF_ROOT, "src", "game_types.h")) as f:
        hdr = f.read()
    hdr = re.sub(r"RES_ID = \d+", f"RES_ID = {res_id}", hdr)
    hdr = re.sub(r"NO_OF_LAYERS = \d+", f"NO_OF_LAYERS = {n_layers}", hdr)
    gen = os.path.join(src, "game_types.h")
    if os.path.lexists(gen):
        os.remove(gen)
    with open(gen, "w") as f:
        f.write(hdr)
    _link(os.path.join(REF_ROOT, "src", "game_constants.h"), os.path.join(src, "game_constants.h"))
    # vertical_grid.c includes the model's constituents header (declarations only)
    os.makedirs(os.path.join(src, "constituents"), exist_ok=True)
    for name in os.listdir(os.path.join(REF_ROOT, "src", "constituents")):
        if name.endswith(".h"):
            _link(os.path.join(REF_ROOT, "src", "constituents", name), os.path.join(src, "constituents", name))
    gg = os.path.join(bdir, "grid_generator", "src")
    os.makedirs(gg, exist_ok=True)
    sources = []
    for name in sorted(os.listdir(os.path.join(REF_ROOT, "grid_generator", "src"))):
        if name.endswith(".h") or name.endswith(".c"):
            _link(os.path.join(REF_ROOT, "grid_generator", "src", name), os.path.join(gg, name))
            if name.endswith(".c"):
                sources.append(os.path.join(gg, name))
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w", "-Dmain=ref_gridgen_main",
           "-I", os.path.join(HERE, "ref_stubs"), "-I", src, "-o", out] + sources + [
        os.path.join(HERE, "ref_io_stubs.c"), os.path.join(HERE, "ref_harness_grid.c"), "-lm"]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    args = [int(a) for a in sys.argv[1:]] or [4, 0]
    print(build(args[0], args[1], force=True))
