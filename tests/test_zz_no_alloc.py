"""The allocation-free selection entry point against the allocating one.

kmc_select_samples_far_from_centroid_noalloc_f32_i32 keeps its scratch in a
static device array (n_selected <= 4096) instead of allocating it per call.
Two consecutive calls with different inputs must both give exactly the
results of kmc_select_samples_far_from_centroid_f32_i32 on the same inputs,
so nothing left in the static scratch by the first call leaks into the
second.  The file sorts last so the check also runs after every other test
in the same process; it passes on its own as well.
"""
import ctypes

import numpy as np
import pytest

from kmeans_dpcpp_gb300 import capi

MAX_SELECTED = 4096


def test_noalloc_rejects_more_than_its_static_scratch_holds():
    L = capi.lib()
    rc = L.kmc_select_samples_far_from_centroid_noalloc_f32_i32(
        MAX_SELECTED + 1, None, None, None, None, None, 10 ** 6, 256, None)
    assert rc == 1
    msg = L.kmc_last_error().decode()
    assert "exceeds 4096" in msg and "allocation-free" in msg
    assert L.kmc_select_samples_far_from_centroid_noalloc_f32_i32(
        0, None, None, None, None, None, 10, 256, None) == 1
    assert "must be positive" in L.kmc_last_error().decode()
    assert L.kmc_select_samples_far_from_centroid_noalloc_f32_i32(
        11, None, None, None, None, None, 10, 256, None) == 1
    assert "too large" in L.kmc_last_error().decode()


def _distances(n, seed):
    rng = np.random.default_rng(seed)
    # few distinct values: many samples tie with the threshold
    return rng.integers(0, 2000, n).astype(np.float32) * np.float32(0.25)


def _select(fn, n_sel, dist, thr_value, gt0, eq0):
    import torch

    n = dist.shape[0]
    d = torch.from_numpy(dist).cuda()
    thr = torch.tensor([thr_value], dtype=torch.float32, device="cuda")
    sel = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    ngt = torch.tensor([gt0], dtype=torch.int32, device="cuda")
    neq = torch.tensor([eq0], dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    capi.check(fn(n_sel, d.data_ptr(), thr.data_ptr(), sel.data_ptr(), ngt.data_ptr(),
                  neq.data_ptr(), n, 256, stream.cuda_stream))
    stream.synchronize()
    return sel.cpu().numpy(), int(ngt.item()), int(neq.item())


@pytest.mark.gpu
def test_noalloc_select_matches_allocating_entry_on_consecutive_calls():
    L = capi.lib()
    cases = [  # (n, n_selected, seed, initial gt / eq counters)
        (300_000, MAX_SELECTED, 1, 0, 0),
        (50_001, 37, 2, 3, 5),
    ]
    for n, n_sel, seed, gt0, eq0 in cases:
        dist = _distances(n, seed)
        thr = np.sort(dist)[::-1][n_sel - 1]   # the n_sel-th largest distance
        ref = _select(L.kmc_select_samples_far_from_centroid_f32_i32, n_sel, dist, thr, gt0, eq0)
        got = _select(L.kmc_select_samples_far_from_centroid_noalloc_f32_i32, n_sel, dist, thr,
                      gt0, eq0)
        np.testing.assert_array_equal(got[0], ref[0])
        assert got[1:] == ref[1:]
        n_gt = int((dist > thr).sum())
        assert got[1] == gt0 + n_gt
        assert got[2] == eq0 + min(n_sel - n_gt, int((dist == thr).sum()))
        # the strictly-greater samples are ranked: selected[gt0 + n_gt - 1 - r]
        # is the r-th farthest, ties by lowest index
        front = got[0][gt0:gt0 + n_gt][::-1]
        order = np.lexsort((np.arange(n), -dist))[:n_gt]
        np.testing.assert_array_equal(front, order)
