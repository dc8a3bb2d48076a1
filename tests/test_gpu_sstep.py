"""s-step CG on the GPU and the pieces that choose its basis: features,
Lanczos (against the numpy oracle), the MLP's forward pass and gradient
(against the numpy oracle), its training, and what the learned shifts gain
over the monomial basis."""
import numpy as np
import pytest

import mpk_gb300 as M
from mpk_gb300 import shifts as S
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradient_match_oracle(gpu):
    m = M.Mlp(M.NFEAT, 64, 8, seed=3)
    rng = np.random.default_rng(0)
    X = rng.normal(size=(48, M.NFEAT)).astype(np.float32)
    T = rng.uniform(size=(48, 8)).astype(np.float32)
    p = m.params()
    Y = m.forward(X)
    Yo = mlp_ref.forward(p, X, M.NFEAT, 64, 8)[0]
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 1e-5
    g, loss = m.gradient(X, T)
    go, lo = mlp_ref.gradient(p, X, T, M.NFEAT, 64, 8)
    assert np.linalg.norm(g - go) / np.linalg.norm(go) < 1e-4
    assert abs(loss - lo) / lo < 1e-5


def test_mlp_training_reduces_loss(gpu):
    X, T = S.training_set(200, seed=5)
    mlp, curve = S.train(X, T, epochs=150)
    assert curve[-1] < curve[0] / 10


def test_features_match_numpy(gpu):
    a = M.Csr.diffusion(30, 20, 1, sigma=0.8, seed=2)
    f, glo, ghi = M.features(a)
    d = np.array([a.val[a.ptr[i]:a.ptr[i + 1]][a.col[a.ptr[i]:a.ptr[i + 1]] == i].sum() for i in range(a.n)])
    o = np.array([np.abs(a.val[a.ptr[i]:a.ptr[i + 1]][a.col[a.ptr[i]:a.ptr[i + 1]] != i]).sum() for i in range(a.n)])
    assert np.isclose(glo, (d - o).min()) and np.isclose(ghi, (d + o).max())
    assert np.isclose(f[1], d.mean() / ghi, rtol=1e-6) and np.isclose(f[5], o.max() / ghi, rtol=1e-6)


def test_lanczos_matches_oracle(gpu):
    a = M.Csr.diffusion(40, 40, 1, sigma=1.0, seed=5)
    r, al, be = M.lanczos(a, 8, seed=2)
    alo, beo = mlp_ref.lanczos(a.ptr, a.col, a.val, 8, M.uniform(2, a.n))
    assert np.allclose(al, alo, rtol=1e-12, atol=1e-12) and np.allclose(be, beo, rtol=1e-12)
    T = np.diag(alo) + np.diag(beo, 1) + np.diag(beo, -1)
    assert np.allclose(r, np.linalg.eigvalsh(T), rtol=1e-12)


@pytest.fixture(scope="module")
def trained_mlp():
    X, T = S.training_set(400, seed=11)
    return S.train(X, T, epochs=200)[0]


@pytest.mark.parametrize("dims", [(96, 96, 1), (36, 36, 36)])
def test_sstep_cg_bases(dims, trained_mlp, gpu):
    """All bases reach 1e-8 (true residual); the learned shifts (no Lanczos
    run) need no more outer iterations than the monomial basis and stay
    within 20 % of the Lanczos-shift basis; standard CG agrees."""
    a = M.Csr.diffusion(*dims, sigma=1.0, seed=77)
    b = M.uniform(3, a.n)
    x_cg, cg = M.cg(a, b)
    assert cg["converged"]
    _, mono = M.sstep_cg(a, b, 8)
    x_l, lan = M.sstep_cg(a, b, 8, shifts=S.from_lanczos(a, 8))
    _, lrn = M.sstep_cg(a, b, 8, shifts=S.predict(trained_mlp, a))
    for inf in (mono, lan, lrn):
        assert inf["converged"] and inf["relres"] <= 1e-8
    assert lrn["iterations"] <= mono["iterations"]
    assert lrn["iterations"] <= 1.2 * lan["iterations"]
    assert np.linalg.norm(x_l - x_cg) / np.linalg.norm(x_cg) < 1e-6


@pytest.mark.parametrize("dims,seed", [((96, 96, 96), 5), ((64, 64, 64), 6)])
def test_learned_shifts_need_no_more_iterations_than_lanczos(dims, seed, gpu):
    """The criterion of the learned part on config-5-like problems (3-D
    7-point variable-coefficient diffusion, log-normal sigma = 1): with the
    shipped MLP (trained on the Ritz values of 2000 synthetic matrices),
    s-step CG (s = 8) reaches 1e-8 in no more outer iterations than with
    the Lanczos shifts, and in fewer than with the monomial basis."""
    import os
    from mpk_gb300.train_shifts import load
    path = os.path.join(os.path.dirname(M.__file__), "shift_mlp.npz")
    mlp = load(path)
    a = M.Csr.diffusion(*dims, sigma=1.0, dominance=0.01, seed=seed)
    b = M.uniform(7, a.n)
    _, mono = M.sstep_cg(a, b, 8)
    _, lan = M.sstep_cg(a, b, 8, shifts=S.from_lanczos(a, 8))
    _, lrn = M.sstep_cg(a, b, 8, shifts=S.predict(mlp, a))
    for inf in (mono, lan, lrn):
        assert inf["converged"] and inf["relres"] <= 1e-8
    assert lrn["iterations"] <= lan["iterations"]
    assert lrn["iterations"] < mono["iterations"]


def test_sstep_gram_modes_agree(gpu):
    """The FP64 Gram (default) and the double-float Gram take the same
    outer iterations on a diffusion problem and give solutions that agree
    far below the solve's tolerance.  The basis condition number is the
    largest over all outer iterations; the last ones depend on rounding
    along the way, so only its magnitude is compared."""
    a = M.Csr.diffusion(64, 64, 8, sigma=1.0, seed=5)
    b = M.uniform(9, a.n)
    sh = S.from_lanczos(a, 8)
    x64, i64 = M.sstep_cg(a, b, 8, shifts=sh, gram=M.GRAM_FP64)
    xdf, idf = M.sstep_cg(a, b, 8, shifts=sh, gram=M.GRAM_DF64)
    for inf in (i64, idf):
        assert inf["converged"] and inf["relres"] <= 1e-8
    assert abs(i64["iterations"] - idf["iterations"]) <= 1
    assert np.linalg.norm(x64 - xdf) / np.linalg.norm(x64) < 1e-7
    assert 0.5 < i64["basis_cond"] / idf["basis_cond"] < 2.0


@pytest.mark.parametrize("gram", [M.GRAM_FP64, M.GRAM_DF64])
def test_sstep_device_loop_equals_host_loop(gram, gpu):
    """The solve as one graph with a device-side WHILE node gives the
    bits, iteration counts and basis condition number of the host-driven
    loop (the same kernels in the same order), including a run cut short
    by max_outer."""
    a = M.Csr.diffusion(48, 48, 16, sigma=1.0, seed=8)
    b = M.uniform(4, a.n)
    sh = S.from_lanczos(a, 8)
    for max_outer in (2000, 3):
        xd, idev = M.sstep_cg(a, b, 8, shifts=sh, gram=gram, max_outer=max_outer, loop=M.SSTEP_DEVICE_LOOP)
        xh, ihost = M.sstep_cg(a, b, 8, shifts=sh, gram=gram, max_outer=max_outer, loop=M.SSTEP_HOST_LOOP)
        assert xd.tobytes() == xh.tobytes()
        for key in ("iterations", "mpk_steps", "breakdowns", "converged", "relres", "basis_cond"):
            assert idev[key] == ihost[key], key
        assert idev["loop_launches"] == 1  # the device-side loop ran
        assert ihost["loop_launches"] == ihost["iterations"]
    assert idev["iterations"] == 3 and not idev["converged"]


@pytest.mark.parametrize("loop", [M.SSTEP_DEVICE_LOOP, M.SSTEP_HOST_LOOP])
def test_sstep_mpk_basis_equals_step_launches(loop, gpu):
    """The basis built as one matrix powers launch (wavefront form, the
    default) gives the bits of the basis built by one SpMV launch per step:
    same solution, iterations and basis condition number."""
    a = M.Csr.diffusion(40, 40, 24, sigma=1.0, seed=12)
    b = M.uniform(6, a.n)
    sh = S.from_lanczos(a, 8)
    xm, im = M.sstep_cg(a, b, 8, shifts=sh, loop=loop, basis=M.SSTEP_BASIS_MPK)
    xs, ist = M.sstep_cg(a, b, 8, shifts=sh, loop=loop, basis=M.SSTEP_BASIS_STEPS)
    assert xm.tobytes() == xs.tobytes()
    for key in ("iterations", "mpk_steps", "breakdowns", "converged", "relres", "basis_cond"):
        assert im[key] == ist[key], key
    assert im["converged"]


def test_sstep_mpk_basis_wait_times_out_and_recovers(gpu):
    """The basis launch's bounded waits give up on levels that are never
    published (MPKG_ETIMEOUT, context usable); the next solve is right."""
    a = M.Csr.diffusion(32, 32, 16, sigma=1.0, seed=13)
    b = M.uniform(2, a.n)
    _check = M._check
    _check(M.lib().mpkg_sstep_debug_stall(50))
    try:
        with pytest.raises(M.MpkError) as e:
            M.sstep_cg(a, b, 4, max_outer=2, basis=M.SSTEP_BASIS_MPK)
        assert e.value.code == M.ETIMEOUT
    finally:
        _check(M.lib().mpkg_sstep_debug_stall(0))
    x1, i1 = M.sstep_cg(a, b, 4, basis=M.SSTEP_BASIS_MPK)
    x2, i2 = M.sstep_cg(a, b, 4, basis=M.SSTEP_BASIS_STEPS)
    assert i1["converged"] and x1.tobytes() == x2.tobytes()
