"""CPU restatement (numpy, FP64) of the learned reference proposal's network.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's checks, never by
the product path.  The reference has no learned component (its alignment is
exhaustive, cuda/gpu_aln_noref.cu:multi_ref_align), so there is nothing of the
reference to pin this against; it is pinned instead by central finite
differences of its own loss (tests/test_nn_oracle.py), and the GPU kernels are
checked against it.

The network, as the CUDA kernels run it (gpu-isac_gb300/csrc/nn.cu):

    x      = features(spectra)            ring magnitudes log(1+|F|), unit norm
    h      = relu(x W1^T + b1)            W1 [hidden][n_in]
    z      = h W2^T + b2                  W2 [emb][hidden]
    e      = z / |z|                      one embedding per image
    s[i,j] = scale * e_p[i] . e_r[j]      particle i vs reference j
    loss   = mean_i  -log softmax(s[i])[label_i]

Particles and references go through the same weights; the gradient of a
shared weight is the sum over both batches.
"""
from __future__ import annotations

import numpy as np


def features(spectra: np.ndarray, nk: int) -> np.ndarray:
    """spectra [n][ring][128][2] in the subject basis (Re+Im, Re-Im), slot 0
    holding (F[0], F[128]) -> [n][ring*nk]: log(1 + |F_r[k]|), k < nk
    (k = 0 is |F[0]|), each row scaled to unit L2 norm."""
    sp = np.asarray(spectra, np.float64)
    n, nr = sp.shape[0], sp.shape[1]
    a, b = sp[:, :, :nk, 0], sp[:, :, :nk, 1]
    re, im = 0.5 * (a + b), 0.5 * (a - b)
    im[:, :, 0] = 0.0
    f = np.log1p(np.hypot(re, im)).reshape(n, nr * nk)
    return f / np.sqrt(np.maximum((f * f).sum(1, keepdims=True), 1e-30))


def init_params(n_in: int, hidden: int, emb: int, seed: int) -> dict:
    """He-uniform weights, zero biases (the initialisation the GPU net uses)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    l1 = np.sqrt(6.0 / n_in)
    l2 = np.sqrt(6.0 / hidden)
    return {"W1": rng.uniform(-l1, l1, (hidden, n_in)).astype(np.float32),
            "b1": np.zeros(hidden, np.float32),
            "W2": rng.uniform(-l2, l2, (emb, hidden)).astype(np.float32),
            "b2": np.zeros(emb, np.float32)}


def embed(params: dict, X: np.ndarray):
    """forward of one batch: returns (E, cache)"""
    W1, b1 = np.asarray(params["W1"], np.float64), np.asarray(params["b1"], np.float64)
    W2, b2 = np.asarray(params["W2"], np.float64), np.asarray(params["b2"], np.float64)
    X = np.asarray(X, np.float64)
    H = np.maximum(X @ W1.T + b1, 0.0)
    Z = H @ W2.T + b2
    nrm = np.sqrt((Z * Z).sum(1, keepdims=True))
    E = Z / nrm
    return E, (X, H, Z, nrm, E)


def scores(params: dict, Xp: np.ndarray, Xr: np.ndarray, scale: float) -> np.ndarray:
    Ep, _ = embed(params, Xp)
    Er, _ = embed(params, Xr)
    return scale * Ep @ Er.T


def _xent(S: np.ndarray, labels: np.ndarray):
    m = S.max(1, keepdims=True)
    ex = np.exp(S - m)
    se = ex.sum(1, keepdims=True)
    loss = (np.log(se) + m)[:, 0] - S[np.arange(S.shape[0]), labels]
    sm = ex / se
    return loss, sm


def loss_and_grads(params: dict, Xp: np.ndarray, Xr: np.ndarray, labels: np.ndarray, scale: float):
    """mean cross-entropy of the particles' reference scores and its gradient
    with respect to every parameter (both batches through shared weights)."""
    W2 = np.asarray(params["W2"], np.float64)
    W1 = np.asarray(params["W1"], np.float64)
    Ep, cp = embed(params, Xp)
    Er, cr = embed(params, Xr)
    S = scale * Ep @ Er.T
    labels = np.asarray(labels, np.int64)
    loss, sm = _xent(S, labels)
    B = S.shape[0]
    dS = sm.copy()
    dS[np.arange(B), labels] -= 1.0
    dS /= B
    dEp = scale * dS @ Er
    dEr = scale * dS.T @ Ep
    g = {k: np.zeros(np.shape(v), np.float64) for k, v in params.items()}
    for dE, (X, H, Z, nrm, E) in ((dEp, cp), (dEr, cr)):
        dZ = (dE - E * (E * dE).sum(1, keepdims=True)) / nrm
        g["W2"] += dZ.T @ H
        g["b2"] += dZ.sum(0)
        dH = dZ @ W2
        dH[H <= 0.0] = 0.0
        g["W1"] += dH.T @ X
        g["b1"] += dH.sum(0)
    return float(loss.mean()), g, {"S": S, "loss": loss, "dS": dS}


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
    """AdamW, bias-corrected (step counts from 1); returns new (p, m, v)"""
    p, g, m, v = (np.asarray(x, np.float64) for x in (p, g, m, v))
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * (mh / (np.sqrt(vh) + eps) + wd * p), m, v


def topk(S: np.ndarray, k: int) -> np.ndarray:
    """indices of the k largest scores per row, best first, ties to the
    smaller index"""
    S = np.asarray(S)
    order = np.lexsort((np.broadcast_to(np.arange(S.shape[1]), S.shape), -S), axis=1)
    return order[:, :k]
