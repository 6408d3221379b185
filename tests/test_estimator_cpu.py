"""KMeans estimator parameter checks and the oracle's k-means++ (no GPU)."""
import numpy as np
import pytest

from kmeans_dpcpp_gb300 import KMeans


@pytest.mark.parametrize("kwargs,n,d,msg", [
    (dict(n_clusters=0), 10, 2, "n_clusters"),
    (dict(n_clusters=11), 10, 2, "n_samples=10"),
    (dict(n_clusters=3, init="kmeans"), 10, 2, "init should be"),
    (dict(n_clusters=3, init=np.zeros((3, 3))), 10, 2, "init array should have shape"),
    (dict(n_clusters=3, n_init=0), 10, 2, "n_init"),
    (dict(n_clusters=3, max_iter=0), 10, 2, "max_iter"),
    (dict(n_clusters=3, tol=-1.0), 10, 2, "tol"),
    (dict(n_clusters=3, form="int8"), 10, 2, "form"),
])
def test_estimator_rejects_bad_parameters(kwargs, n, d, msg):
    with pytest.raises(ValueError, match=msg):
        KMeans(**kwargs)._check_params(n, d)


def test_oracle_kmeans_plusplus_draws_distinct_rows(oracle):
    X = np.random.default_rng(0).standard_normal((5, 3000)).astype(np.float32)
    rows, C = oracle.kmeans_plusplus(X, 50, 11)
    assert len(set(rows.tolist())) == 50
    np.testing.assert_array_equal(C, X[:, rows])
    rows2, _ = oracle.kmeans_plusplus(X, 50, 11)
    np.testing.assert_array_equal(rows, rows2)
    rows3, _ = oracle.kmeans_plusplus(X, 50, 12)
    assert not np.array_equal(rows, rows3)
