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


def test_work_items_cover_every_tile_once_under_concurrent_pulls():
    """A mocked work queue on CPU threads: the engine's own planner
    (kmc_debug_batch_items) splits uneven instances into items; eight threads
    take items from a shared counter, as the persistent assign CTAs do with
    their device counter, and every 128-sample tile of every instance must be
    handled exactly once, in the group of its kind and tile variant."""
    import itertools
    import threading

    L = capi.lib()
    rng = np.random.default_rng(3)
    count = 40
    n = rng.integers(0, 300_000, count).astype(np.int64)
    n[:3] = [0, 1, 128 * 8 + 1]           # empty, one sample, just past one item
    modes = rng.integers(0, 3, count).astype(np.int32)
    variants = rng.integers(0, 3, count).astype(np.int32)
    total = ctypes.c_int64()
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    capi.check(L.kmc_debug_batch_items(count, P(n, ctypes.c_int64), P(modes, ctypes.c_int),
                                       P(variants, ctypes.c_int), 0, None, None, None, None,
                                       ctypes.byref(total)))
    m = total.value
    inst = np.empty(m, np.int32)
    tiles = np.empty(m, np.int32)
    first = np.empty(m, np.int64)
    group = np.empty(m, np.int32)
    capi.check(L.kmc_debug_batch_items(count, P(n, ctypes.c_int64), P(modes, ctypes.c_int),
                                       P(variants, ctypes.c_int), m, P(inst, ctypes.c_int32),
                                       P(tiles, ctypes.c_int32), P(first, ctypes.c_int64),
                                       P(group, ctypes.c_int32), ctypes.byref(total)))
    assert np.all((tiles >= 1) & (tiles <= 8))
    assert np.all(group == (modes[inst] == 2) * 3 + variants[inst])
    assert np.all(np.diff(group) >= 0)     # listed group by group

    seen = [np.zeros(-(-int(v) // 128), np.int32) for v in n]
    lock = threading.Lock()
    for g in np.unique(group):
        idx = np.flatnonzero(group == g)
        counter = itertools.count()

        def worker():
            while True:
                with lock:
                    j = next(counter)
                if j >= len(idx):
                    return
                it = idx[j]
                s = seen[inst[it]]
                for t in range(first[it], first[it] + tiles[it]):
                    with lock:
                        s[t] += 1

        threads = [threading.Thread(target=worker) for _ in range(8)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    for q in range(count):
        assert np.all(seen[q] == 1), q
