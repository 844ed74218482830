"""Hash grid on the GPU through the C ABI, bit-exact against the reference.

bp_grid_build (cell keys, stable radix sort, cellStart/cellEnd) and
bp_grid_neighbor_counts are compared with the golden fixtures produced by the
reference's own kernels, and with the oracle on fresh inputs up to 1M points."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def gpu_grid(bp, torch, pos, cell, D, h=None):
    lib = bp.abi.load()
    n = len(pos)
    dev = torch.device("cuda:0")
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).to(dev)
    i32 = dict(dtype=torch.int32, device=dev)
    cid = torch.empty(max(n, 1), **i32)
    scid = torch.empty(max(n, 1), **i32)
    spid = torch.empty(max(n, 1), **i32)
    cs = torch.full((D ** 3,), -1, **i32)
    ce = torch.full((D ** 3,), -1, **i32)
    ws_bytes = C.c_size_t()
    bp.abi.check(lib, lib.bp_grid_workspace_size(n, D, C.byref(ws_bytes)))
    ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    bp.abi.check(lib, lib.bp_grid_build(stream, n, p.data_ptr(), C.c_float(cell), D, cid.data_ptr(),
                                        scid.data_ptr(), spid.data_ptr(), cs.data_ptr(), ce.data_ptr(),
                                        ws.data_ptr(), ws_bytes.value))
    counts = None
    if h is not None and n:
        sp = p[spid.long()].contiguous()
        cnt = torch.empty(n, **i32)
        bp.abi.check(lib, lib.bp_grid_neighbor_counts(stream, n, sp.data_ptr(), C.c_float(cell), D, C.c_float(h),
                                                      cs.data_ptr(), ce.data_ptr(), cnt.data_ptr()))
        counts = cnt.cpu().numpy()
    torch.cuda.synchronize()
    out = [t.cpu().numpy()[:n] for t in (cid, scid, spid)]
    return out + [cs.cpu().numpy(), ce.cpu().numpy(), counts, (lib, stream, scid, cs, ce)]


@pytest.mark.parametrize("name", ["grid_d32.npz", "grid_d4_alias.npz", "grid_faces_d16.npz", "grid_d512.npz",
                                  "grid_single.npz"])
def test_grid_matches_reference_golden(bp, gpu, name):
    z = np.load(GOLDEN / name)
    cid, scid, spid, cs, ce, counts, _ = gpu_grid(bp, gpu, z["positions"], float(z["cell"]), int(z["D"]),
                                                  float(z["h"]))
    np.testing.assert_array_equal(cid, z["cell_ids"])
    np.testing.assert_array_equal(scid, z["sorted_cell_ids"])
    np.testing.assert_array_equal(spid, z["sorted_particle_ids"])
    occ = np.nonzero(cs >= 0)[0]
    np.testing.assert_array_equal(occ, z["occupied"])
    np.testing.assert_array_equal(cs[occ], z["cell_start"])
    np.testing.assert_array_equal(ce[occ], z["cell_end"])
    assert ((ce >= 0) == (cs >= 0)).all()
    np.testing.assert_array_equal(counts, z["neighbor_counts"])


@pytest.mark.parametrize("n,D,spread,seed", [
    (4095, 64, 5.0, 1),      # one key short of a sort tile
    (4097, 64, 5.0, 2),      # one key past it
    (100_000, 64, 12.8, 3),  # table aliased in every axis
    (1_048_576, 64, 12.0, 4),
    (50_000, 128, 3.0, 5),   # 21-bit keys: three radix passes
    (20_000, 8, 2.0, 6),     # tiny table, long runs of equal keys
])
def test_grid_matches_oracle(bp, gpu, oracle, n, D, spread, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    cell = 0.2
    cid, scid, spid, cs, ce, counts, _ = gpu_grid(bp, gpu, pos, cell, D, 0.2 if n <= 200_000 else None)
    ocid, oscid, ospid, ocs, oce = oracle.grid_build("oracle", pos, cell, D)
    np.testing.assert_array_equal(cid, ocid)
    np.testing.assert_array_equal(spid, ospid)
    np.testing.assert_array_equal(scid, oscid)
    np.testing.assert_array_equal(cs, ocs)
    np.testing.assert_array_equal(ce, oce)
    if counts is not None:
        np.testing.assert_array_equal(counts, oracle.neighbor_counts("oracle", pos[ospid], cell, D, 0.2, ocs, oce))


def test_grid_sort_stable_with_ties(bp, gpu):
    n = 10_000
    pos = np.zeros((n, 3), np.float32)
    pos[::2] = 0.31  # two cells, interleaved
    _, scid, spid, cs, ce, _, _ = gpu_grid(bp, gpu, pos, 0.2, 16)
    a = spid[scid == scid[0]]
    b = spid[scid != scid[0]]
    assert (np.diff(a) > 0).all() and (np.diff(b) > 0).all()


def test_grid_reset_restores_minus_one(bp, gpu):
    rng = np.random.default_rng(9)
    pos = rng.uniform(-1, 1, (5000, 3)).astype(np.float32)
    *_, (lib, stream, scid, cs, ce) = gpu_grid(bp, gpu, pos, 0.2, 32)
    bp.abi.check(lib, lib.bp_grid_reset(stream, len(pos), scid.data_ptr(), cs.data_ptr(), ce.data_ptr()))
    gpu.cuda.synchronize()
    assert int((cs != -1).sum()) == 0 and int((ce != -1).sum()) == 0


def test_grid_empty_input(bp, gpu):
    cid, scid, spid, cs, ce, counts, _ = gpu_grid(bp, gpu, np.zeros((0, 3), np.float32), 0.2, 8)
    assert len(cid) == 0 and (cs == -1).all()
