"""Host-side pieces of the batched engine and the serving loop (no GPU)."""
import ctypes

import numpy as np
import pytest

from kmeans_dpcpp_gb300 import capi


def test_serve_structs_match_the_header():
    assert ctypes.sizeof(capi.ServeRequest) == 80
    assert ctypes.sizeof(capi.ServeResult) == 40


@pytest.mark.parametrize("n,k,seed", [(10, 10, 0), (1000, 37, 5), (2 ** 20, 1024, 123), (7, 1, 9)])
def test_seeded_rows_are_distinct_and_in_range(n, k, seed):
    out = (ctypes.c_int32 * k)()
    capi.check(capi.lib().kmc_seeded_rows(n, k, seed, out))
    rows = np.frombuffer(out, np.int32)
    assert len(set(rows.tolist())) == k
    assert rows.min() >= 0 and rows.max() < n


def test_request_bytes_grow_with_the_request():
    L = capi.lib()

    def need(kind, n, d, k, form):
        b = ctypes.c_int64()
        capi.check(L.kmc_serve_bytes_needed(kind, n, d, k, form, ctypes.byref(b)))
        return b.value

    base = need(0, 100000, 32, 64, 0)
    assert need(0, 200000, 32, 64, 0) > base and need(0, 100000, 64, 64, 0) > base
    assert need(1, 100000, 32, 64, 0) < base          # predictions hold no sums
    assert need(0, 100000, 32, 64, 2) > base          # tensor-core operands
    assert base >= 100000 * 32 * 4                    # at least the samples themselves


def _reqs(rows):
    arr = (capi.ServeRequest * len(rows))()
    for r, row in enumerate(rows):
        arr[r] = capi.ServeRequest(*row)
    return arr


@pytest.mark.parametrize("rows,msg", [
    ([(0.5, 0, 4, 100, 8, 2, 1, 0.0, 10, -1, 1.0, 1.0), (0.1, 0, 4, 100, 8, 2, 1, 0.0, 10, -1, 1.0, 1.0)],
     "sorted by arrival"),
    ([(0.0, 1, 4, 100, 8, 2, 1, 0.0, 0, 0, 1.0, 1.0)], "earlier fit"),
    ([(0.0, 0, 4, 10, 80, 2, 1, 0.0, 10, -1, 1.0, 1.0)], "invalid sizes"),
    ([(0.0, 3, 4, 100, 8, 2, 1, 0.0, 10, -1, 1.0, 1.0)], "kind must be"),
    ([(0.0, 2, 4, 100, 8, 2, 1, 0.0, 0, 0, 1.0, 1.0)], "earlier fit"),   # transform without a model
])
def test_serve_run_rejects_bad_request_streams(rows, msg):
    L = capi.lib()
    res = (capi.ServeResult * len(rows))()
    mk = ctypes.c_double()
    rc = L.kmc_serve_run(_reqs(rows), len(rows), 0, 1 << 30, 8, None, res, ctypes.byref(mk))
    assert rc == 1
    assert msg in L.kmc_last_error().decode()
