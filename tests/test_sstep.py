"""Host-side pieces of s-step CG: tridiagonal eigenvalues, Leja ordering,
and the numpy MLP oracle's own gradient (finite differences)."""
import numpy as np

import mpk_gb300 as M
from oracle import mlp_ref


def test_tridiag_eigs_match_numpy():
    rng = np.random.default_rng(0)
    for m in (1, 2, 5, 17):
        al, be = rng.normal(size=m), rng.normal(size=max(m - 1, 0))
        T = np.diag(al) + (np.diag(be, 1) + np.diag(be, -1) if m > 1 else 0)
        got = M.tridiag_eigs(al, be)
        assert np.allclose(got, np.linalg.eigvalsh(T), rtol=0, atol=1e-12)


def test_leja_order():
    pts = np.array([0.3, 2.5, 1.1, 0.05, 1.9, 0.7])
    o = M.leja(pts)
    assert sorted(o) == sorted(pts)
    assert o[0] == 2.5
    for k in range(2, len(o)):  # each next point maximises the product of distances
        cand = [p for p in pts if p not in o[:k - 1]]
        prod = lambda p: np.prod(np.abs(p - o[:k - 1]))
        assert prod(o[k - 1]) >= max(prod(c) for c in cand) - 1e-15


def test_mlp_oracle_gradient_finite_differences():
    rng = np.random.default_rng(1)
    nin, w, nout, B = 5, 7, 3, 4
    n = w * nin + w + w * w + w + nout * w + nout
    p = rng.normal(size=n) * 0.5
    X, T = rng.normal(size=(B, nin)), rng.normal(size=(B, nout))
    g, _ = mlp_ref.gradient(p, X, T, nin, w, nout)
    eps = 1e-6
    for k in rng.choice(n, 20, replace=False):
        e = np.zeros(n)
        e[k] = eps
        lp = mlp_ref.gradient(p + e, X, T, nin, w, nout)[1]
        lm = mlp_ref.gradient(p - e, X, T, nin, w, nout)[1]
        assert abs((lp - lm) / (2 * eps) - g[k]) < 1e-6


def test_sstep_gram_mode_is_checked():
    """The Gram mode is a host setting: known modes are accepted, others
    are refused with EINVAL before any GPU work."""
    lib = M.lib()
    assert lib.mpkg_sstep_gram(M.GRAM_DF64) == 0
    assert lib.mpkg_sstep_gram(M.GRAM_FP64) == 0
    assert lib.mpkg_sstep_gram(7) == M.EINVAL


def test_sstep_loop_mode_is_checked():
    lib = M.lib()
    assert lib.mpkg_sstep_loop(M.SSTEP_HOST_LOOP) == 0
    assert lib.mpkg_sstep_loop(M.SSTEP_DEVICE_LOOP) == 0
    assert lib.mpkg_sstep_loop(2) == M.EINVAL
