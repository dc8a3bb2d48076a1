"""Newton-basis shifts for s-step CG: from Lanczos Ritz values, or predicted
from cheap matrix features by the library's MLP.

The MLP is trained on the Ritz values that the library's own GPU Lanczos
produces for seeded synthetic diffusion matrices (variable coefficients,
2-D 9-point and 3-D 7-point, random anisotropy and diagonal dominance).
Targets are the s Ritz values of an s-step Lanczos run, ascending, mapped
to [0, 1] across the Gershgorin interval; predictions are mapped back,
sorted and Leja-ordered.
"""
import numpy as np

from . import Csr, Mlp, NFEAT, features, lanczos, leja


def training_matrix(seed):
    """One seeded SPD diffusion matrix of the training distribution."""
    rng = np.random.default_rng(seed)
    sigma = float(rng.uniform(0.2, 1.5))
    dom = float(np.exp(rng.uniform(np.log(1e-4), np.log(0.3))))
    s = int(rng.integers(1 << 62))
    if rng.random() < 0.5:
        nx, ny = (int(v) for v in rng.integers(16, 65, size=2))
        return Csr.diffusion(nx, ny, 1, sigma=sigma, wx=float(rng.uniform(0.05, 1.0)), wy=float(rng.uniform(0.05, 1.0)),
                             wdiag=float(rng.uniform(0.0, 0.5)), dominance=dom, seed=s)
    nx, ny, nz = (int(v) for v in rng.integers(8, 25, size=3))
    return Csr.diffusion(nx, ny, nz, sigma=sigma, dominance=dom, seed=s)


def targets(a, s=8, seed=0):
    """(features, normalised ascending Ritz values of s Lanczos steps)."""
    f, glo, ghi = features(a)
    ritz, _, _ = lanczos(a, s, seed=seed)
    t = (np.sort(ritz) - glo) / (ghi - glo)
    return f, np.clip(t, 0.0, 1.0).astype(np.float32)


def training_set(count=2000, s=8, seed=0):
    X = np.zeros((count, NFEAT), dtype=np.float32)
    T = np.zeros((count, s), dtype=np.float32)
    for k in range(count):
        X[k], T[k] = targets(training_matrix(seed * 1_000_003 + k), s, seed=k)
    return X, T


def train(X, T, width=64, epochs=400, batch=64, lr=2e-3, seed=0):
    """A fresh MLP (NFEAT -> width -> width -> s) trained on (X, T); returns
    (mlp, loss per epoch)."""
    m = Mlp(X.shape[1], width, T.shape[1], seed=seed)
    curve = m.train(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return m, curve


def predict(mlp, a):
    """Leja-ordered shifts for matrix `a` from the MLP."""
    f, glo, ghi = features(a)
    y = mlp.forward(f[None, :])[0].astype(np.float64)
    return leja(glo + (ghi - glo) * np.sort(np.clip(y, 0.0, 1.0)))


def from_lanczos(a, s=8, seed=0):
    """Leja-ordered Ritz values of s Lanczos steps."""
    ritz, _, _ = lanczos(a, s, seed=seed)
    return leja(ritz)
