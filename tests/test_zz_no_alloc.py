"""game_gpu_weighted_sums_noalloc through the C ABI against the context-based
integrators (global_scalar_integrator, game_gpu_write_out_integral).

Both run the same compensated reduction, which returns the exact sum of the
exact products rounded once; they differ only in the order of the
accumulation, so they agree to within 2 ulp (tolerance below).  The file name
puts it last in a full run, so it passes both after every other test in the
same process and alone in a fresh one.  Device buffers come from torch (test
infrastructure only).
"""
import math

import numpy as np
import pytest

from game_archived_gb300 import abi, native
from helpers import clone, make_model

pytestmark = pytest.mark.gpu

ULPS = 2


def _close(got, ref):
    return abs(got - ref) <= ULPS * math.ulp(ref)


def test_noalloc_matches_context_integrators_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    _, m = make_model(3, 1, "jet_moist", mountain=True)
    lay = m.layout
    ns, n_const = lay.n_scalars, lay.n_const
    rng = np.random.default_rng(11)
    field = rng.normal(size=ns) * np.exp(rng.uniform(-10, 10, size=ns))
    gpu = abi.GpuModel(clone(m), abi.FP64)
    try:
        ref_one = gpu.global_scalar_integrator(field)
        ref_masses = gpu.write_out_integral(gpu.m.state_old, 0)
    finally:
        gpu.close()

    lib = native.gpu()
    dev = torch.device("cuda:0")
    w = torch.from_numpy(np.ascontiguousarray(m.grid["volume"])).to(dev)
    f_one = torch.from_numpy(field.copy()).to(dev)
    f_masses = torch.from_numpy(np.ascontiguousarray(m.state_old["rho"][:n_const * ns])).to(dev)
    out = torch.full((8,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        out.fill_(float("nan"))
        rc = lib.game_gpu_weighted_sums_noalloc(f_one.data_ptr(), 1, ns, w.data_ptr(), out.data_ptr(), stream)
        assert rc == 0, lib.game_gpu_last_error().decode()
        torch.cuda.synchronize(dev)
        got = out[0].item()
        assert _close(got, ref_one), (call, got, ref_one)

        out.fill_(float("nan"))
        rc = lib.game_gpu_weighted_sums_noalloc(f_masses.data_ptr(), n_const, ns, w.data_ptr(), out.data_ptr(),
                                                stream)
        assert rc == 0, lib.game_gpu_last_error().decode()
        torch.cuda.synchronize(dev)
        got = out[:n_const].cpu().numpy()
        for k in range(n_const):
            assert _close(got[k], ref_masses[k]), (call, k, got[k], ref_masses[k])
        assert math.isnan(out[n_const].item())  # nothing written beyond n_fields


def test_noalloc_rejects_field_counts_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = native.gpu()
    dev = torch.device("cuda:0")
    f = torch.ones(9 * 16, dtype=torch.float64, device=dev)
    w = torch.ones(16, dtype=torch.float64, device=dev)
    out = torch.zeros(9, dtype=torch.float64, device=dev)
    for bad in (0, 9):
        rc = lib.game_gpu_weighted_sums_noalloc(f.data_ptr(), bad, 16, w.data_ptr(), out.data_ptr(), None)
        assert rc != 0
        assert "n_fields" in lib.game_gpu_last_error().decode()
    # a valid call afterwards still works: 8 fields of sixteen ones
    rc = lib.game_gpu_weighted_sums_noalloc(f.data_ptr(), 8, 16, w.data_ptr(), out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize(dev)
    assert out[:8].cpu().tolist() == [16.0] * 8


_FRESH_PROCESS_FIRST_CALL = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
import torch
from game_archived_gb300 import native
lib = native.gpu()
dev = torch.device("cuda:0")
n = 1 << 16
rng = np.random.default_rng(5)
f = rng.normal(size=3 * n)
w = rng.uniform(0.5, 2.0, size=n)
ft = torch.from_numpy(f).to(dev)
wt = torch.from_numpy(w).to(dev)
out = torch.full((3,), float("nan"), dtype=torch.float64, device=dev)
torch.cuda.synchronize(dev)
side = torch.cuda.Stream(dev)  # a non-blocking stream
with torch.cuda.stream(side):
    # the very first call of this process runs on the side stream
    rc = lib.game_gpu_weighted_sums_noalloc(ft.data_ptr(), 3, n, wt.data_ptr(), out.data_ptr(), side.cuda_stream)
    assert rc == 0, lib.game_gpu_last_error().decode()
side.synchronize()
ref = [float(np.sum(f[k * n:(k + 1) * n] * w)) for k in range(3)]
got = out.cpu().tolist()
for g, r in zip(got, ref):
    assert abs(g - r) <= 1e-12 * abs(r), (got, ref)
print("ok")
"""


def test_noalloc_first_call_of_a_process_on_a_side_stream():
    """The first call of a fresh process, made on a non-blocking stream,
    returns the right sums (the scratch's counters are never cleared from the
    host, so nothing unordered can land between the kernel's atomics)."""
    import os
    import subprocess
    import sys
    pytest.importorskip("torch")
    tests = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(tests)
    code = _FRESH_PROCESS_FIRST_CALL.format(root=root, tests=tests)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


def test_noalloc_calls_leave_device_memory_untouched():
    """Repeated calls take no device memory: cudaMemGetInfo's free bytes are
    the same before and after, with torch's caching allocator idle."""
    torch = pytest.importorskip("torch")
    lib = native.gpu()
    dev = torch.device("cuda:0")
    n = 1 << 20
    f = torch.rand(4 * n, dtype=torch.float64, device=dev)
    w = torch.rand(n, dtype=torch.float64, device=dev)
    out = torch.zeros(4, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.game_gpu_weighted_sums_noalloc(f.data_ptr(), 4, n, w.data_ptr(), out.data_ptr(), stream)
    assert rc == 0, lib.game_gpu_last_error().decode()
    torch.cuda.synchronize(dev)
    free_before, _ = torch.cuda.mem_get_info(dev)
    for _ in range(10):
        rc = lib.game_gpu_weighted_sums_noalloc(f.data_ptr(), 4, n, w.data_ptr(), out.data_ptr(), stream)
        assert rc == 0, lib.game_gpu_last_error().decode()
    torch.cuda.synchronize(dev)
    free_after, _ = torch.cuda.mem_get_info(dev)
    assert free_after == free_before, (free_before, free_after)
    ref = (f.view(4, n) * w).sum(dim=1)
    assert torch.allclose(out, ref, rtol=1e-12, atol=0.0)
