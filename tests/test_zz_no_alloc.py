"""The allocation-free time-of-impact entry point (abd_pt_min_toi_noalloc), called
through the C ABI with caller-owned device buffers, against the allocating batched
entry point (abd_pt_collision_time_batch): per-trajectory TOIs and their minimum must
match exactly (the same device function computes them), on two calls in a row with
different sizes so a stale scratch array from the first call would show. Kept in its
own file, collected last."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 8, 3))
    # half of them constructed to collide (Sample-Test1/test.cpp:9-31)
    toi = rng.random(n // 2)
    x[: n // 2, 4] = x[: n // 2, 2] / toi[:, None] - x[: n // 2, 0] * ((1 - toi) / toi)[:, None]
    x[: n // 2, 5:8] = x[: n // 2, 1:4]
    return np.ascontiguousarray(x.reshape(n, 24))


def test_noalloc_min_toi_matches_batched_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    from adb_gb300 import abdtk
    L = gpu_lib
    for n, seed in ((5000, 1), (777, 2)):
        x = _batch(n, seed)
        ref = abdtk.pt_collision_time_batch(x.reshape(n, 8, 3))
        dx = torch.from_numpy(x).cuda()
        dtoi = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
        dmin = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.abd_pt_min_toi_noalloc(n, C.c_void_p(dx.data_ptr()), C.c_void_p(dtoi.data_ptr()),
                                      C.c_void_p(dmin.data_ptr()), None)
        assert rc == 0, L.abd_noalloc_last_error()
        torch.cuda.synchronize()
        toi = dtoi.cpu().numpy()
        assert np.array_equal(toi, ref)
        assert dmin.cpu().item() == ref.min()


def test_noalloc_rejects_oversized_batches(gpu_lib):
    L = gpu_lib
    rc = L.abd_pt_min_toi_noalloc((1 << 22) + 1, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 8
    assert b"ABD_NOALLOC_MAX_N" in L.abd_noalloc_last_error()
