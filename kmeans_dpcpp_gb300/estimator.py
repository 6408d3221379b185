"""A scikit-learn-style ``KMeans`` estimator on top of the drop-in module.

The reference module is the offloading layer of an estimator it does not
contain (its README names the sklearn-numba-dpex style engine as the caller).
This is that caller for the GB300 engine: ``fit`` takes row-major samples
``X`` (n_samples, n_features), transposes them on the device into the
feature-major ``X_t`` the engine reads, seeds the centroids on the device
(``"k-means++"``, ``"random"`` rows, or given), scales ``tol`` by the mean
per-feature variance of ``X`` (as scikit-learn's Lloyd engine does) and runs
``kmeans_lloyd_driver``.  ``predict``, ``transform`` and ``score`` use the
``assignment``, ``compute_centroid_to_sample_distances`` and
``compute_inertia`` kernels.  Results are NumPy arrays on the host.

Every computation runs the engine's CUDA kernels; torch only provides device
memory and the stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi as _capi
from ._kmeans_dpcpp import (
    assignment as _assignment,
    compute_centroid_to_sample_distances as _distances,
    compute_inertia as _inertia,
    half_l2_norm_squared as _half_norm,
    kmeans_lloyd_driver as _driver,
    reduce_vector_blocking as _reduce,
)

_FORMS = ("plain", "mixed-fp16", "mixed-bf16")


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("KMeans needs a CUDA device")
    return torch


def _suffix(dtype):
    import torch

    if dtype == torch.float32:
        return "f32"
    if dtype == torch.float64:
        return "f64"
    raise ValueError("X must be float32 or float64")


class KMeans:
    """Lloyd k-means on one GB300.

    Parameters follow scikit-learn's ``KMeans`` where they apply:
    ``n_clusters``, ``init`` ("k-means++", "random" or an array of shape
    (n_clusters, n_features)), ``n_init`` (runs with different seeds; the
    lowest inertia wins), ``max_iter``, ``tol`` (relative: multiplied by the
    mean per-feature variance of X), ``verbose`` and ``random_state``.
    ``form`` selects the engine's arithmetic: "plain" (exact float32 /
    float64, the reference's) or a mixed tensor-core form ("mixed-fp16",
    "mixed-bf16"; float32 data, same labels, see the engine's notes).

    Attributes after ``fit``: ``cluster_centers_`` (n_clusters, n_features),
    ``labels_`` (n_samples,), ``inertia_``, ``n_iter_``, ``n_features_in_``.
    """

    def __init__(self, n_clusters=8, *, init="k-means++", n_init=1, max_iter=300, tol=1e-4,
                 verbose=False, random_state=None, form="plain"):
        self.n_clusters = n_clusters
        self.init = init
        self.n_init = n_init
        self.max_iter = max_iter
        self.tol = tol
        self.verbose = verbose
        self.random_state = random_state
        self.form = form

    # ------------------------------------------------------------------ checks
    def _check_params(self, n_samples, n_features):
        if not isinstance(self.n_clusters, (int, np.integer)) or self.n_clusters < 1:
            raise ValueError(f"n_clusters should be a positive integer, got {self.n_clusters!r}")
        if self.n_clusters > n_samples:
            raise ValueError(f"n_samples={n_samples} should be >= n_clusters={self.n_clusters}")
        if not isinstance(self.n_init, (int, np.integer)) or self.n_init < 1:
            raise ValueError(f"n_init should be a positive integer, got {self.n_init!r}")
        if not isinstance(self.max_iter, (int, np.integer)) or self.max_iter < 1:
            raise ValueError(f"max_iter should be a positive integer, got {self.max_iter!r}")
        if self.tol < 0:
            raise ValueError(f"tol should be non-negative, got {self.tol!r}")
        if self.form not in _FORMS:
            raise ValueError(f"form should be one of {_FORMS}, got {self.form!r}")
        if isinstance(self.init, str):
            if self.init not in ("k-means++", "random"):
                raise ValueError(f"init should be 'k-means++', 'random' or an array, got {self.init!r}")
        else:
            c = np.asarray(self.init)
            if c.shape != (self.n_clusters, n_features):
                raise ValueError(f"init array should have shape ({self.n_clusters}, {n_features}), "
                                 f"got {c.shape}")

    # ------------------------------------------------------------------ device
    def _to_device_t(self, X, dtype=None):
        """Row-major (n, d) samples -> feature-major (d, n) device tensor."""
        torch = _torch()
        if isinstance(X, torch.Tensor):
            Xd = X.detach()
            if dtype is not None:
                Xd = Xd.to(dtype)
            Xd = Xd.to("cuda").contiguous()
        else:
            a = np.asarray(X)
            if dtype is None:
                dtype = torch.float64 if a.dtype == np.float64 else torch.float32
            Xd = torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")
        if Xd.dim() != 2:
            raise ValueError(f"X should be a 2-D array, got shape {tuple(Xd.shape)}")
        if Xd.dtype not in (torch.float32, torch.float64):
            Xd = Xd.to(torch.float32)
        n, d = Xd.shape
        Xt = torch.empty((d, n), dtype=Xd.dtype, device="cuda")
        L = _capi.lib()
        s = torch.cuda.current_stream().cuda_stream
        _capi.check(getattr(L, f"kmc_transpose_{_suffix(Xd.dtype)}")(Xd.data_ptr(), Xt.data_ptr(), n, d, s))
        return Xt

    def _weights(self, sample_weight, n, dtype):
        torch = _torch()
        if sample_weight is None:
            return torch.ones(n, dtype=dtype, device="cuda")
        w = torch.as_tensor(np.asarray(sample_weight) if not isinstance(sample_weight, torch.Tensor)
                            else sample_weight, dtype=dtype, device="cuda").contiguous()
        if w.shape != (n,):
            raise ValueError(f"sample_weight should have shape ({n},), got {tuple(w.shape)}")
        return w

    def _seed_centroids(self, Xt, w, seed):
        torch = _torch()
        d, n = Xt.shape
        k = self.n_clusters
        L = _capi.lib()
        s = torch.cuda.current_stream().cuda_stream
        suf = _suffix(Xt.dtype)
        C = torch.empty((d, k), dtype=Xt.dtype, device="cuda")
        if isinstance(self.init, str) and self.init == "k-means++":
            rows = torch.empty(k, dtype=torch.int32, device="cuda")
            _capi.check(getattr(L, f"kmc_kmeans_plusplus_{suf}")(Xt.data_ptr(), w.data_ptr(), n, d, k,
                                                                 seed, C.data_ptr(), rows.data_ptr(), s))
        elif isinstance(self.init, str):  # "random": distinct rows drawn on the host
            idx = np.random.default_rng(seed).choice(n, size=k, replace=False).astype(np.int32)
            rows = torch.as_tensor(idx, device="cuda")
            _capi.check(getattr(L, f"kmc_gather_rows_{suf}")(Xt.data_ptr(), n, d, rows.data_ptr(), k,
                                                             C.data_ptr(), s))
        else:
            C.copy_(torch.as_tensor(np.asarray(self.init), dtype=Xt.dtype, device="cuda").t())
        return C

    # ------------------------------------------------------------------ API
    def fit(self, X, y=None, sample_weight=None):
        torch = _torch()
        Xt = self._to_device_t(X)
        d, n = Xt.shape
        self._check_params(n, d)
        if self.form != "plain" and Xt.dtype != torch.float32:
            raise ValueError("the mixed forms take float32 data")
        w = self._weights(sample_weight, n, Xt.dtype)
        # scikit-learn's Lloyd tolerance: tol times the mean per-feature variance
        mv = ctypes.c_double()
        _capi.check(getattr(_capi.lib(), f"kmc_mean_feature_variance_{_suffix(Xt.dtype)}")(
            Xt.data_ptr(), n, d, ctypes.byref(mv), torch.cuda.current_stream().cuda_stream))
        tol_abs = mv.value * self.tol
        rng = np.random.default_rng(self.random_state)
        best = None
        for _ in range(self.n_init):
            seed = int(rng.integers(0, 2 ** 63 - 1))
            C = self._seed_centroids(Xt, w, seed)
            labels = torch.empty(n, dtype=torch.int32, device="cuda")
            res = torch.empty_like(C)
            n_iter, inertia = _driver(Xt, w, C, labels, res, tol_abs, bool(self.verbose), int(self.max_iter),
                                      8, 128, 0.7, None, form=self.form)
            inertia = float(np.asarray(inertia).reshape(-1)[0])
            if best is None or inertia < best[0]:
                best = (inertia, n_iter, res, labels)
        inertia, n_iter, res, labels = best
        torch.cuda.current_stream().synchronize()
        self._centers_t = res
        self.cluster_centers_ = res.t().contiguous().cpu().numpy()
        self.labels_ = labels.cpu().numpy().astype(np.int64)
        self.inertia_ = inertia
        self.n_iter_ = int(n_iter)
        self.n_features_in_ = d
        return self

    def _check_fitted(self, Xt):
        if not hasattr(self, "_centers_t"):
            raise RuntimeError("this KMeans instance is not fitted yet; call fit first")
        if Xt.shape[0] != self.n_features_in_:
            raise ValueError(f"X has {Xt.shape[0]} features, but KMeans was fitted with "
                             f"{self.n_features_in_}")

    def predict(self, X, sample_weight=None):
        torch = _torch()
        Xt = self._to_device_t(X, self._centers_t.dtype)
        self._check_fitted(Xt)
        d, n = Xt.shape
        k = self._centers_t.shape[1]
        hn = torch.empty(k, dtype=Xt.dtype, device="cuda")
        labels = torch.empty(n, dtype=torch.int32, device="cuda")
        for ev in _half_norm(self._centers_t, hn, 128, None):
            ev.wait()
        for ev in _assignment(Xt, self._centers_t, hn, labels, 8, 128, None):
            ev.wait()
        torch.cuda.current_stream().synchronize()
        return labels.cpu().numpy().astype(np.int64)

    def transform(self, X):
        """Euclidean distances to the cluster centres, shape (n_samples, n_clusters)."""
        torch = _torch()
        Xt = self._to_device_t(X, self._centers_t.dtype if hasattr(self, "_centers_t") else None)
        self._check_fitted(Xt)
        d, n = Xt.shape
        k = self._centers_t.shape[1]
        D = torch.empty((k, n), dtype=Xt.dtype, device="cuda")
        for ev in _distances(Xt, self._centers_t, D, 128, 8, None):
            ev.wait()
        torch.cuda.current_stream().synchronize()
        return D.t().contiguous().cpu().numpy()

    def score(self, X, y=None, sample_weight=None):
        """Opposite of the (weighted) inertia of X against the cluster centres."""
        torch = _torch()
        Xt = self._to_device_t(X, self._centers_t.dtype if hasattr(self, "_centers_t") else None)
        self._check_fitted(Xt)
        d, n = Xt.shape
        labels = torch.as_tensor(self.predict(X).astype(np.int32), device="cuda")
        w = self._weights(sample_weight, n, Xt.dtype)
        per = torch.empty(n, dtype=Xt.dtype, device="cuda")
        for ev in _inertia(Xt, w, self._centers_t, labels, per, 128, None):
            ev.wait()
        torch.cuda.current_stream().synchronize()
        return -float(_reduce(per, None))

    def fit_predict(self, X, y=None, sample_weight=None):
        return self.fit(X, sample_weight=sample_weight).labels_

    def fit_transform(self, X, y=None, sample_weight=None):
        return self.fit(X, sample_weight=sample_weight).transform(X)
