"""In-tree build of the native libraries.

* libgame_tables.so  -- host C: grid-table builder and the run-time struct layout
                        (gcc, -ffp-contract=off so x86_64 and aarch64 round alike)
* libgame_gb300.so   -- the CUDA library behind the C ABI in include/game_gb300.h
                        (nvcc, sm_103a only)

Both land next to this file.  Sources are compiled in parallel; a library is
rebuilt only when one of its sources is newer than it.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")

TABLES_LIB = os.path.join(HERE, "libgame_tables.so")
GPU_LIB = os.path.join(HERE, "libgame_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def tables_sources():
    return [os.path.join(CSRC, "tables", "gridgen.c"), os.path.join(CSRC, "common", "layout.c"),
            os.path.join(CSRC, "common", "ncwrite.c")]


def build_tables(force=False):
    srcs = tables_sources()
    deps = srcs + glob.glob(os.path.join(CSRC, "tables", "*.h")) + glob.glob(os.path.join(CSRC, "common", "*.h"))
    if not force and not _newer(TABLES_LIB, deps):
        return TABLES_LIB
    _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
          "-I", os.path.join(CSRC, "common"), "-o", TABLES_LIB] + srcs + ["-lm"])
    return TABLES_LIB


def gpu_sources():
    return sorted(glob.glob(os.path.join(CSRC, "gpu", "*.cu")))


def nvcc_flags(src):
    """Per-file flags: the FP64 translation unit is compiled without FMA
    contraction so that it rounds exactly like the reference C built with
    -ffp-contract=off; every other unit may contract."""
    base = ["nvcc", "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CSRC, "common"), "-I", os.path.join(CSRC, "gpu")] + ARCH
    if os.path.basename(src).endswith("_f64.cu"):
        base += ["--fmad=false"]
    else:
        base += ["--fmad=true"]
    return base


def build_gpu(force=False, jobs=None):
    if shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    srcs = gpu_sources()
    hdrs = glob.glob(os.path.join(CSRC, "gpu", "*.h")) + glob.glob(os.path.join(CSRC, "gpu", "*.cuh")) \
        + glob.glob(os.path.join(CSRC, "common", "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    common_c = [os.path.join(CSRC, "common", "layout.c"), os.path.join(CSRC, "common", "ncwrite.c")]
    if not force and not _newer(GPU_LIB, srcs + hdrs + common_c):
        return GPU_LIB
    os.makedirs(BUILD, exist_ok=True)
    objs = []
    jobs_list = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        jobs_list.append(nvcc_flags(s) + ["-c", s, "-o", o])
    for s in common_c:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        jobs_list.append(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-I", os.path.join(CSRC, "common"), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs_list))
    _run(["nvcc", "-shared", "-o", GPU_LIB] + ARCH + objs + ["-lcudart"])
    return GPU_LIB


def build_all(force=False):
    build_tables(force)
    build_gpu(force)


if __name__ == "__main__":
    build_all(force=True)
    print("built", TABLES_LIB, GPU_LIB)
