"""The CPU oracle on its own: reference semantics, known answers, edge cases.

The reference repository has no tests and no golden vectors for this path, so
the oracle is pinned by (a) known-answer cases whose result follows from the
geometry alone, (b) FP32 vs FP64 agreement, and (c) -m gpu tests that compare
its texture emulation with the texture unit the reference samples through
(tests/test_gpu_texture.py) and with golden fixtures (tests/golden/).
"""
import math

import numpy as np
import pytest

from gpuisac import synth


def circ_diff(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def test_polar_template_geometry(oracle_mod):
    t = oracle_mod.polar_template(35, 256)
    r = np.hypot(t[..., 0], t[..., 1])
    assert np.allclose(r, np.arange(1, 36)[:, None], atol=1e-5)
    # ring i, angle 0 is (i+1, 0); angle 64 is (~0, i+1)
    assert np.all(t[:, 0, 0] == np.arange(1, 36)) and np.all(t[:, 0, 1] == 0)
    assert np.allclose(t[:, 64, 1], np.arange(1, 36))


def test_shift_grid_order(oracle_mod):
    s = oracle_mod.shift_array(3.0, 3.0, 1.0)
    assert len(s) == 49
    # x outer, y inner (cuda/gpu_aln_common.cu:75-82)
    assert tuple(s[0]) == (-3, -3) and tuple(s[1]) == (-3, -2) and tuple(s[7]) == (-2, -3)
    s2 = oracle_mod.shift_array(1.0, 2.0, 0.5)
    assert len(s2) == 5 * 9


@pytest.mark.parametrize("t,expect", [(10.5, (10, 0.0)), (10.75, (10, 0.25)), (0.5, (0, 0.0)),
                                      (0.0, (-1, 0.5)), (10.5 + 1.0 / 512, (10, 1.0 / 256)),
                                      (10.5 + 3.0 / 512, (10, 2.0 / 256)), (11.49999, (11, 0.0)),
                                      (10.5 + 511.0 / 512, (11, 0.0))])
def test_texture_weight_rounding(oracle_mod, t, expect):
    i, a = oracle_mod.tex_split(t)
    assert (i, a) == expect


@pytest.mark.parametrize("fx,fy", [(0.0, 0.0), (221.0, 128.0), (196.0, 32.0), (128.0, 128.0), (255.0, 255.0)])
def test_texture_tap_weights(oracle_mod, fx, fy):
    ix, iy, w = oracle_mod.tex_weights(10.5 + fx / 256.0, 20.5 + fy / 256.0)
    A, B = int(fx), int(fy)
    w11 = (A * B + 128) >> 8
    assert (ix, iy) == (10, 20) and sum(w) == 256
    assert w == [256 - A - B + w11, A - w11, B - w11, w11]


def test_reference_layout_mref_workload(oracle_mod):
    cfg = oracle_mod.make_cfg(50000, 200, 76, 35, 256, 1.0, 3.0, 3.0)
    lay = oracle_mod.reference_layout(cfg)
    # cuFFT int32 guard: P_b * 100 * 98 * 258 <= 2^31 - 1  ->  849
    assert (lay.sbj_batch, lay.tex_limit, lay.ref_batch) == (849, 855, 100)


@pytest.mark.parametrize("k", [0, 1, 2, 3])
@pytest.mark.parametrize("mirror", [False, True])
def test_known_answer_quarter_turns(oracle_mod, k, mirror):
    """An odd-sized reference turned by k quarter turns (exact in pixel space)
    must come back as that reference, angle -90k (mod 360), no shift, and the
    mirror flag of the input."""
    st = synth.make_stack(1, 65, 3, 0, 0.0, 28.0, 11)
    img = st.refs[2][:, ::-1] if mirror else st.refs[2]
    img = np.rot90(img, k).copy()
    sbj = np.stack([img, img])
    cfg = oracle_mod.make_cfg(2, 3, 65, 29, 256, 1.0, 1.0, 1.0)
    lay = oracle_mod.reference_layout(cfg)
    peak, d = oracle_mod.multi_ref_align(cfg, lay, sbj, st.refs)
    q = int(np.argmax(d[:, 0]))
    assert q == 2
    ang, sx, sy, m = peak[q, 0]
    assert circ_diff(ang, -90.0 * k) < 1e-3
    assert (sx, sy, m) == (0.0, 0.0, 1.0 if mirror else 0.0)


@pytest.mark.parametrize("dx,dy", [(1, -2), (-2, 0), (2, 2)])
def test_known_answer_integer_shift(oracle_mod, dx, dy):
    st = synth.make_stack(1, 64, 2, 0, 0.0, 20.0, 5)
    ref = st.refs[1]
    img = np.zeros_like(ref)
    # particle = reference moved by (dx, dy) pixels (x = column, y = row)
    ys, xs = slice(max(dy, 0), 64 + min(dy, 0)), slice(max(dx, 0), 64 + min(dx, 0))
    yr, xr = slice(max(-dy, 0), 64 + min(-dy, 0)), slice(max(-dx, 0), 64 + min(-dx, 0))
    img[ys, xs] = ref[yr, xr]
    cfg = oracle_mod.make_cfg(1, 2, 64, 25, 256, 1.0, 2.0, 2.0)
    lay = oracle_mod.reference_layout(cfg)
    peak, d = oracle_mod.multi_ref_align(cfg, lay, img[None], st.refs)
    q = int(np.argmax(d[:, 0]))
    assert q == 1
    ang, sx, sy, m = peak[q, 0]
    assert (sx, sy, m) == (float(dx), float(dy), 0.0)
    assert circ_diff(ang, 0.0) < 1e-3


def test_peak_search_parabola_and_ties(oracle_mod):
    S, L = 3, 256
    ccf = np.full((2 * S, L), -1e6)
    tau0 = 10.3
    t = np.arange(L)
    ccf[4] = 100.0 - (t - tau0) ** 2  # mirror half, shift 1
    out, pk, tau = oracle_mod.peak_search(ccf)
    assert tau == 10 and out[1] == 1 and out[3] == 1
    # the 7-point least-squares parabola is exact on quadratic data
    expect = (360.0 - 360.0 / L * tau0 + 180.0) % 360.0
    assert abs(out[0] - expect) < 1e-4
    # ties: the first maximum in scan order (normal before mirror) wins
    ccf2 = np.zeros((2 * S, L))
    ccf2[5, 7] = 5.0
    ccf2[2, 9] = 5.0
    out2, _, tau2 = oracle_mod.peak_search(ccf2)
    assert (out2[1], out2[3], tau2) == (2, 0, 9)


def test_stacked_texture_reads_neighbour(oracle_mod):
    """Bilinear taps below an image read the next image of the same texture;
    the last image of a texture clamps (cuda/gpu_aln_noref.cu:1283-1287)."""
    D = 16
    stack = np.zeros((3, D, D), np.float32)
    stack[1] = 1.0
    stack[2] = 2.0
    cfg = oracle_mod.make_cfg(3, 1, D, 9, 256, 1.0, 0.0, 0.0)
    lay = oracle_mod.OrcLayout(3, 1000, 1)
    raw0 = _raw_polar(oracle_mod, cfg, lay, stack, 0)
    # ring 9 around centre 8: y reaches row 17 = row 1 of image 1 (value 1)
    assert raw0.max() > 0.5
    lay_clamp = oracle_mod.OrcLayout(1, 1000, 1)  # every image its own batch: clamps
    assert _raw_polar(oracle_mod, cfg, lay_clamp, stack, 0).max() == 0.0


def _raw_polar(oracle_mod, cfg, lay, stack, img):
    # undo the normalisation by comparing against a constant-offset copy
    a = oracle_mod.polar(cfg, lay, stack, img)
    return np.abs(a) if np.ptp(a) > 0 else np.zeros_like(a)


def test_f32_mode_agrees_with_f64(oracle_mod):
    st = synth.make_stack(24, 64, 4, 2, 0.1, 28.0, 3)
    cfg = oracle_mod.make_cfg(24, 4, 64, 29, 256, 1.0, 2.0, 2.0)
    lay = oracle_mod.reference_layout(cfg)
    p64, d64 = oracle_mod.multi_ref_align(cfg, lay, st.particles, st.refs, precision="f64")
    p32, d32 = oracle_mod.multi_ref_align(cfg, lay, st.particles, st.refs, precision="f32")
    rel = np.abs(d32 - d64) / np.abs(d64).max()
    assert rel.max() < 1e-5
    assert (np.argmax(d32, 0) == np.argmax(d64, 0)).all()
    same = (p32[..., 1:] == p64[..., 1:]).all(-1) & (circ_diff(p32[..., 0], p64[..., 0]) < 0.05)
    assert same.mean() >= 0.995


def test_recovers_synthetic_truth(oracle_mod):
    st = synth.make_stack(40, 64, 4, 2, 0.0, 28.0, 1)
    cfg = oracle_mod.make_cfg(40, 4, 64, 29, 256, 1.0, 2.0, 2.0)
    lay = oracle_mod.reference_layout(cfg)
    peak, d = oracle_mod.multi_ref_align(cfg, lay, st.particles, st.refs)
    q = np.argmax(d, 0)
    assert (q == st.cls).all()
    best = peak[q, np.arange(40)]
    assert (best[:, 3] == st.mirror).all()
    assert (best[:, 1:3] == st.shift).all()
    assert circ_diff(best[:, 0], st.angle).max() < 0.5


def test_pre_align_rule_known_answers(oracle_mod):
    """The pre-alignment's index rule: first strict maximum from 0, so a table
    with no positive value keeps (normal, shift 0, angle 0); the shift update
    adds in float and clamps to +-(img_dim - ring_num - 2)."""
    shifts = oracle_mod.shift_array(1.0, 1.0, 1.0)
    c = -np.ones((2, 9, 256))
    sx, sy, ang, mir = oracle_mod.pre_align_param(c, shifts, (0.25, -0.5), 64, 29)
    assert (sx, sy, mir) == (np.float32(0.25 + shifts[0][0]), np.float32(-0.5 + shifts[0][1]), False)
    assert ang == np.float32(360.0)          # flat neighbourhood: c3 = 0
    c = np.zeros((2, 9, 256))
    c[1, 4, 10] = 5.0
    c[1, 4, 9] = c[1, 4, 11] = 4.0           # symmetric peak: no sub-step offset
    c[0, 7, 3] = 5.0                         # a later-found equal value loses? no: normal comes first
    sx, sy, ang, mir = oracle_mod.pre_align_param(c, shifts, (0.0, 0.0), 64, 29)
    assert mir is False and (sx, sy) == (np.float32(shifts[7][0]), np.float32(shifts[7][1]))
    c[0, 7, 3] = 0.0
    sx, sy, ang, mir = oracle_mod.pre_align_param(c, shifts, (0.0, 0.0), 64, 29)
    assert mir is True and (sx, sy) == (np.float32(shifts[4][0]), np.float32(shifts[4][1]))
    assert abs(float(ang) - ((360.0 - 10 * 360.0 / 256) + 180.0 - 360.0)) < 1e-4
    # clamp: limit 64 - 29 - 2 = 33
    sx, _, _, _ = oracle_mod.pre_align_param(-np.ones((2, 9, 256)), shifts, (40.0, 0.0), 64, 29)
    assert sx == np.float32(33.0)
