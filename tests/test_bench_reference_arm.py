"""The benchmark's CPU reference arm (bench.py --impl reference) on a small
configuration (RES_ID=4, config1): it reads the prepared grid tables and
struct layout with numpy, runs the oracle on all host threads and a one-thread
row in a child process, honours --steps and --warmup, and loads no library of
the package (only the oracle's)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUN_WITH_MAPS = r"""
import atexit, runpy, sys
def dump():
    libs = sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l})
    sys.stderr.write('LOADED ' + ' '.join(libs) + '\n')
atexit.register(dump)
sys.argv = ['bench.py'] + sys.argv[1:]
runpy.run_path(sys.argv[0], run_name='__main__')
"""


@pytest.mark.skipif(not os.path.exists("/proc/self/maps"), reason="needs /proc")
def test_reference_arm_loads_no_library_of_the_package(tmp_path):
    env = dict(os.environ, GAME_INPUT_DIR=str(tmp_path), OMP_NUM_THREADS="2")
    prep = subprocess.run([sys.executable, "-c", "from game_archived_gb300 import workloads; "
                                                 "workloads.prepare('config1', n_lloyd=20)"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert prep.returncode == 0, prep.stderr
    r = subprocess.run([sys.executable, "-c", RUN_WITH_MAPS, "--impl", "reference", "--config", "config1",
                        "--steps", "3", "--warmup", "4", "--n-lloyd", "20"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 4
    assert line["value"] > 0 and line["cpu_1thread"]["value"] > 0
    loaded = [l for l in r.stderr.splitlines() if l.startswith("LOADED")][-1].split()[1:]
    ours = [p for p in loaded if p.startswith(ROOT)]
    assert ours == [os.path.join(ROOT, "oracle", "liboracle.so")], ours


def test_reference_arm_without_inputs_reports_unavailable(tmp_path):
    env = dict(os.environ, GAME_INPUT_DIR=str(tmp_path / "empty"))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                        "config1", "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
