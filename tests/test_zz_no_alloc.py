"""bp_grid_build_static: the grid build for callers that cannot allocate.

A plug-in that lives inside a host application owning all device memory, or
a real-time loop that may not allocate (or synchronise, as cudaMalloc and
cudaFree can) after start-up, cannot hand bp_grid_build a workspace of its
own.  bp_grid_build_static keeps the sort's scratch in a fixed array inside
the library instead.  These tests call it through the C ABI several times in
a row, with different sizes, and require outputs identical to bp_grid_build's
on the same inputs: the grid is integer work, so the tolerance is zero.

The file is named to be collected last, so that it also runs after every other
GPU test in one process; it passes alone as well."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 262144


def _outputs(torch, n, D):
    i32 = dict(dtype=torch.int32, device="cuda:0")
    return [torch.empty(n, **i32) for _ in range(3)] + [torch.full((D ** 3,), -1, **i32) for _ in range(2)]


def _with_workspace(bp, torch, lib, stream, p, cell, D):
    n = p.shape[0]
    out = _outputs(torch, n, D)
    ws_bytes = C.c_size_t()
    bp.abi.check(lib, lib.bp_grid_workspace_size(n, D, C.byref(ws_bytes)))
    ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device="cuda:0")
    bp.abi.check(lib, lib.bp_grid_build(stream, n, p.data_ptr(), C.c_float(cell), D,
                                        *[t.data_ptr() for t in out], ws.data_ptr(), ws_bytes.value))
    return out


def _static(bp, torch, lib, stream, p, cell, D):
    n = p.shape[0]
    out = _outputs(torch, n, D)
    bp.abi.check(lib, lib.bp_grid_build_static(stream, n, p.data_ptr(), C.c_float(cell), D,
                                               *[t.data_ptr() for t in out]))
    return out


@pytest.mark.parametrize("order", ["large_first", "small_first"])
def test_static_grid_matches_workspace_grid_on_consecutive_calls(bp, gpu, order):
    torch = gpu
    lib = bp.abi.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    # (particles, grid_dim, cell size, spread): two sort passes at D = 64,
    # three at D = 512; the largest case fills the fixed scratch exactly.
    cases = [(MAX_PARTICLES, 512, 0.05, 30.0), (200_000, 64, 0.2, 12.0), (1_000, 16, 0.5, 6.0)]
    if order == "small_first":
        cases = cases[::-1]
    for n, D, cell, spread in cases:
        pos = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
        p = torch.from_numpy(pos).to("cuda:0")
        got = _static(bp, torch, lib, stream, p, cell, D)
        want = _with_workspace(bp, torch, lib, stream, p, cell, D)
        torch.cuda.synchronize()
        names = ["cell_ids", "sorted_cell_ids", "sorted_particle_ids", "cell_start", "cell_end"]
        for name, g, w in zip(names, got, want):
            assert torch.equal(g, w), f"{name} differs for n={n}, D={D}"
        del got, want, p


def test_static_grid_rejects_more_than_its_capacity(bp, gpu):
    torch = gpu
    lib = bp.abi.load()
    n = MAX_PARTICLES + 1
    p = torch.zeros((n, 3), dtype=torch.float32, device="cuda:0")
    out = _outputs(torch, n, 8)
    st = lib.bp_grid_build_static(torch.cuda.current_stream().cuda_stream, n, p.data_ptr(), C.c_float(0.1), 8,
                                  *[t.data_ptr() for t in out])
    assert st == bp.abi.BP_ERR_CAPACITY
    assert b"262144" in lib.bp_last_error_string()
    torch.cuda.synchronize()
    assert bool((out[3] == -1).all())
