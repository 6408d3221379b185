"""The mixed forms' certification bound, checked on the CPU.

A numpy emulation of the tensor-core arithmetic -- operands sigma x and
sigma c rounded to fp16 (or bf16), exact products accumulated in float32, the
half norms as three 16-bit parts against constant columns -- produces every
score; a sample is certified when exactly one column reaches
thr = M - 2 E_i, with E_i = ||x_i|| alpha + ||dX_i|| / sigma beta1 + beta0 built
from the measured operand rounding errors as the kernels build it.  Every
certified winner must be the reference's exact float32 label (the oracle's
assignment: sequential fused dot, hn - dot, strict < over ascending j), on
random blobs and on adversarial data full of near-ties.  This checks the bound
itself; the GPU tests check the kernels' labels.
"""
import numpy as np
import pytest


def _round16(a, bf16):
    a = np.asarray(a, np.float32)
    if not bf16:
        return a.astype(np.float16).astype(np.float64)
    # bf16: round to nearest even on the upper 16 bits of the float32 pattern
    b = a.view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _sigma(xmax, d, bf16):
    if bf16 or xmax == 0:
        return 1.0
    hx = 0.5 * d * xmax * xmax
    fits = lambda s: xmax * s <= 2.0 ** 14 and s * s * hx <= 2.0 ** 25  # noqa: E731
    s = 1.0
    while s < 2.0 ** 60 and fits(s * 2):
        s *= 2
    while s > 2.0 ** -60 and not fits(s):
        s *= 0.5
    return s


def _certified_labels(X, C, hn, bf16, order="sequential"):
    d, n = X.shape
    k = C.shape[1]
    xmax = float(np.abs(X).max())
    sigma = _sigma(xmax, d, bf16)
    s2 = sigma * sigma
    u = 2.0 ** -8 if bf16 else 2.0 ** -11
    xs = _round16(sigma * X.astype(np.float64), bf16)        # (d, n)
    cs = _round16(sigma * C.astype(np.float64), bf16)        # (d, k)
    up = 1 + 1e-6
    nx = np.sqrt((X.astype(np.float64) ** 2).sum(0)) * up
    ndx = np.sqrt(((xs - sigma * X.astype(np.float64)) ** 2).sum(0)) / sigma * up
    cmax = float(np.sqrt((C.astype(np.float64) ** 2).sum(0)).max()) * up
    dcmax = float(np.sqrt(((cs - sigma * C.astype(np.float64)) ** 2).sum(0)).max()) / sigma * up
    hmax = float(np.abs(hn).max())
    flush = 2.0 ** -126 * np.sqrt(d) * (1 + u) if bf16 else 0.0
    alpha = dcmax + 2.0 ** -16 * (cmax + dcmax) + (d + 4) * 2.0 ** -23 * cmax + flush
    beta1 = (cmax + dcmax) * (1 + 2.0 ** -16)
    hfloor = (2.0 ** -126 if bf16 else 2.0 ** -34) / s2
    beta0 = hmax * (u ** 3 + 2.0 ** -16 + 2.0 ** -23) + hfloor + flush * cmax
    E = (nx * alpha + ndx * beta1 + beta0) * up

    # sigma^2 hn in three 16-bit parts h_p against the constant column weights
    # c_p (fp16: 2^10, 1, 2^-10; bf16: 1, 1, 1), each part the rounded
    # remainder of the previous ones
    coef = (1.0, 1.0, 1.0) if bf16 else (2.0 ** 10, 1.0, 2.0 ** -10)
    H = hn.astype(np.float64) * s2
    h0 = _round16((H / coef[0]).astype(np.float32), bf16)
    r1 = H - coef[0] * h0
    h1 = _round16((r1 / coef[1]).astype(np.float32), bf16)
    r2 = r1 - coef[1] * h1
    h2 = _round16((r2 / coef[2]).astype(np.float32), bf16)
    # scores: exact 16-bit products accumulated in float32 over the features,
    # then the three norm terms -c_p h_p (exact products)
    acc = np.zeros((n, k), np.float32)
    if order == "sequential":
        for f in range(d):
            acc = (acc + np.outer(xs[f], cs[f]).astype(np.float32)).astype(np.float32)
    else:
        # K = 16 steps: each step's 16 products summed as a float32 tree, the
        # step then added to the accumulator (another order the hardware may use)
        for f0 in range(0, d, 16):
            terms = [np.outer(xs[f], cs[f]).astype(np.float32) for f in range(f0, min(d, f0 + 16))]
            while len(terms) > 1:
                terms = [(terms[i] + terms[i + 1]).astype(np.float32) if i + 1 < len(terms)
                         else terms[i] for i in range(0, len(terms), 2)]
            acc = (acc + terms[0]).astype(np.float32)
    for c_p, part in zip(coef, (h0, h1, h2)):
        acc = (acc - (c_p * part).astype(np.float32)[None, :]).astype(np.float32)
    score = acc.astype(np.float64) / s2                       # x.c - hn, unscaled
    M = score.max(axis=1)
    thr = M - 2 * E
    hot = score >= thr[:, None]
    cert = hot.sum(axis=1) == 1
    return cert, np.argmax(score, axis=1)


def _near_ties(rng, n, d, k):
    # samples on segments between two random centroids, at offsets from the
    # bisector spread over six decades, so that the gaps between the best two
    # scores run from far below the bound to far above it
    C = rng.uniform(-4, 4, (d, k)).astype(np.float32)
    a = rng.integers(0, k, n)
    b = (a + rng.integers(1, k, n)) % k
    delta = np.exp(rng.uniform(np.log(1e-6), np.log(0.5), n)) * rng.choice([-1.0, 1.0], n)
    t = 0.5 + delta
    X = (C[:, a] * t + C[:, b] * (1 - t)).astype(np.float32)
    return np.ascontiguousarray(X), np.ascontiguousarray(C)


@pytest.mark.parametrize("order", ["sequential", "blocks16"])
@pytest.mark.parametrize("bf16", [False, True])
@pytest.mark.parametrize("kind", ["blobs", "near_ties"])
@pytest.mark.parametrize("d,k", [(8, 16), (33, 40), (64, 64)])
def test_certified_winners_are_the_exact_labels(oracle, bf16, kind, d, k, order):
    import bench

    rng = np.random.default_rng(d * 100 + k + (7 if bf16 else 0))
    n = 3000
    if kind == "blobs":
        X, _, _ = bench.make_blobs(n, d, k, (-5, 5), 1.0, d + k)
        C = np.ascontiguousarray(bench.random_row_init(X, k, d + k))
    else:
        X, C = _near_ties(rng, n, d, k)
    hn = oracle.half_l2_norm_squared(C)
    ref = oracle.assignment(X, C)
    cert, win = _certified_labels(X, C, hn, bf16, order)
    assert cert.mean() > (0.5 if kind == "blobs" else 0.2)
    bad = np.flatnonzero(cert & (win != ref))
    assert bad.size == 0, f"{bad.size} certified samples disagree with the exact labels"
