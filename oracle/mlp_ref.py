"""Test oracle for the shift-predicting MLP (mpk_gb300/csrc/mlp.cu): a numpy
FP64 restatement of its forward pass and mean-squared-error gradient, and a
numpy Lanczos.  These forms have no counterpart in the reference (its only
s-step material is a notebook with a monomial basis, jupyter/s-step-cg.ipynb);
tests use this file only as the checker, never as the thing measured."""
import numpy as np


def unpack(p, nin, w, nout):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + w * nin].reshape(w, nin); o += w * nin
    b1 = p[o:o + w]; o += w
    W2 = p[o:o + w * w].reshape(w, w); o += w * w
    b2 = p[o:o + w]; o += w
    W3 = p[o:o + nout * w].reshape(nout, w); o += nout * w
    b3 = p[o:o + nout]; o += nout
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(p, X, nin, w, nout):
    W1, b1, W2, b2, W3, b3 = unpack(p, nin, w, nout)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3.T + b3, h1, h2


def gradient(p, X, T, nin, w, nout):
    """(flat gradient of mean((Y - T)^2), loss)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, nin, w, nout)
    X = np.asarray(X, dtype=np.float64)
    Y, h1, h2 = forward(p, X, nin, w, nout)
    B = X.shape[0]
    dy = 2.0 * (Y - np.asarray(T, dtype=np.float64)) / (B * nout)
    dh2 = (dy @ W3) * (h2 > 0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g = np.concatenate([(dh1.T @ X).ravel(), dh1.sum(0), (dh2.T @ h1).ravel(), dh2.sum(0),
                        (dy.T @ h2).ravel(), dy.sum(0)])
    return g, float(np.mean((Y - T) ** 2))


def lanczos(ptr, col, val, m, x0):
    """m Lanczos steps (no reorthogonalisation) from x0: (alpha, beta)."""
    import scipy.sparse as sp
    n = len(ptr) - 1
    A = sp.csr_matrix((val, col, ptr), shape=(n, n))
    v = np.asarray(x0, dtype=np.float64) / np.linalg.norm(x0)
    vp = np.zeros(n)
    al, be = [], []
    b = 0.0
    for j in range(m):
        w_ = A @ v - b * vp
        a = w_ @ v
        al.append(a)
        if j + 1 == m:
            break
        w_ = w_ - a * v
        b = np.linalg.norm(w_)
        be.append(b)
        vp, v = v, w_ / b
    return np.array(al), np.array(be)
