"""The proposal network's CPU oracle on its own: its analytic gradient against
central finite differences (FP64), its feature map's invariances, and the
host-side rules of the proposal search (best-of-candidates, margin
calibration).  No GPU."""
import numpy as np
import pytest

import nn_oracle as nno
from gpuisac import learned


def _problem(seed=3, B=6, R=5, n_in=12, hidden=7, emb=4):
    rng = np.random.Generator(np.random.PCG64(seed))
    params = nno.init_params(n_in, hidden, emb, seed)
    params = {k: v.astype(np.float64) + 0.05 * rng.standard_normal(v.shape) for k, v in params.items()}
    Xp = rng.standard_normal((B, n_in))
    Xr = rng.standard_normal((R, n_in))
    labels = rng.integers(0, R, B)
    return params, Xp, Xr, labels


@pytest.mark.parametrize("name", ["W1", "b1", "W2", "b2"])
def test_gradient_matches_finite_differences(name):
    params, Xp, Xr, labels = _problem()
    scale = 5.0
    _, g, _ = nno.loss_and_grads(params, Xp, Xr, labels, scale)
    h = 1e-6
    flat = params[name].reshape(-1)
    num = np.zeros_like(flat)
    for i in range(flat.size):
        old = flat[i]
        flat[i] = old + h
        lp, _, _ = nno.loss_and_grads(params, Xp, Xr, labels, scale)
        flat[i] = old - h
        lm, _, _ = nno.loss_and_grads(params, Xp, Xr, labels, scale)
        flat[i] = old
        num[i] = (lp - lm) / (2 * h)
    ana = g[name].reshape(-1)
    assert np.allclose(ana, num, rtol=1e-5, atol=1e-8), np.abs(ana - num).max()


def test_loss_is_mean_cross_entropy():
    params, Xp, Xr, labels = _problem(seed=5)
    loss, _, aux = nno.loss_and_grads(params, Xp, Xr, labels, 3.0)
    S = nno.scores(params, Xp, Xr, 3.0)
    p = np.exp(S - S.max(1, keepdims=True))
    p /= p.sum(1, keepdims=True)
    assert np.isclose(loss, -np.log(p[np.arange(len(labels)), labels]).mean())
    assert np.allclose(aux["S"], S)


def test_features_rotation_and_mirror_invariant():
    """|F| of a ring does not change under a circular shift (rotation) or
    reversal (mirror) of the ring samples."""
    rng = np.random.Generator(np.random.PCG64(9))
    rings = rng.standard_normal((2, 7, 256))

    def spectra(x):
        F = np.fft.rfft(x, axis=-1)  # [.., 129]
        out = np.zeros(x.shape[:-1] + (128, 2))
        out[..., 1:, 0] = F[..., 1:128].real + F[..., 1:128].imag
        out[..., 1:, 1] = F[..., 1:128].real - F[..., 1:128].imag
        # slot 0: the pair (F[0], F[128]) in the same (Re+Im, Re-Im) basis
        out[..., 0, 0] = F[..., 0].real + F[..., 128].real
        out[..., 0, 1] = F[..., 0].real - F[..., 128].real
        return out

    f0 = nno.features(spectra(rings), 64)
    f1 = nno.features(spectra(np.roll(rings, 37, axis=-1)), 64)
    f2 = nno.features(spectra(np.roll(rings[..., ::-1], 5, axis=-1)), 64)
    assert f0.shape == (2, 7 * 64)
    assert np.allclose(np.linalg.norm(f0, axis=1), 1.0)
    assert np.allclose(f0, f1) and np.allclose(f0, f2)


def test_adam_matches_closed_form_first_step():
    p, g = np.array([1.0, -2.0]), np.array([0.5, -0.25])
    p1, m, v = nno.adam_step(p, g, np.zeros(2), np.zeros(2), 1, lr=0.1)
    # first bias-corrected step moves each weight by lr * sign(g)
    assert np.allclose(p1, p - 0.1 * np.sign(g), atol=1e-6)


def test_topk_ties_take_smaller_index():
    S = np.array([[1.0, 3.0, 3.0, 0.0, 2.0]])
    assert nno.topk(S, 3).tolist() == [[1, 2, 4]]


def test_init_params_shared_with_product():
    a = nno.init_params(20, 8, 4, 11)
    b = learned.init_params(20, 8, 4, 11)
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_best_of_and_margin_calibration():
    # full-search peaks of 6 particles against 4 references (column = particle)
    d = np.array([[0.9, 0.1, 0.5, 0.2, 0.3, 0.8],
                  [0.2, 0.7, 0.5, 0.1, 0.6, 0.1],
                  [0.1, 0.2, 0.1, 0.9, 0.59, 0.2],
                  [0.0, 0.0, 0.0, 0.0, 0.0, 0.79]])
    prop = np.array([[0, 1], [1, 2], [1, 0], [2, 3], [2, 3], [3, 1]])
    pd = np.take_along_axis(d.T, prop, axis=1)
    pos, ref, best, second = learned.best_of(pd, prop)
    # particle 2: tie 0.5 / 0.5 -> the smaller reference (0)
    assert ref.tolist() == [0, 1, 0, 2, 2, 3]
    assert np.allclose(best - second, [0.7, 0.5, 0.0, 0.9, 0.59, 0.69])
    # wrong: particle 4 (true 1, gap 0.59) and particle 5 (true 0, gap 0.69)
    truth = d.argmax(0)
    gaps, correct = best - second, ref == truth
    g0 = learned.calibrate_margin(gaps, correct, max_wrong=0.0)
    assert g0 > 0.69
    assert (gaps >= g0).tolist() == [True, False, False, True, False, False]
    g1 = learned.calibrate_margin(gaps, correct, max_wrong=1.0 / 6)
    assert 0.59 < g1 <= np.nextafter(0.59, 1)
    assert learned.calibrate_margin(gaps, np.ones(6, bool)) == 0.0
