"""The averaging step's restatement (oracle.class_averages and its parts) on
its own properties, CPU only.  EMAN2 (rot_shift2D, filt_tanl, fshift) is not
part of the reference tree, so parity with it is unpinned; these tests pin the
restatement's published definitions (quadratic interpolation exact on
quadratics, identity and mirror transforms, the filter's response, the Fourier
shift) and its agreement with the alignment it follows: particles made from
references by known turns, shifts and mirrors, aligned by the oracle's
multi-reference search and averaged with the parameters it found, give back
their references."""
import numpy as np
import pytest

from gpuisac import synth


def test_quadri_exact_on_quadratics(oracle_mod):
    D = 40
    yy, xx = np.meshgrid(np.arange(D, dtype=float), np.arange(D, dtype=float), indexing="ij")
    f = 0.7 + 0.3 * xx - 0.02 * xx ** 2 + 0.5 * yy + 0.011 * yy ** 2 - 0.03 * xx * yy
    rng = np.random.default_rng(3)
    xo, yo = rng.uniform(1.0, D - 2.0, 4000), rng.uniform(1.0, D - 2.0, 4000)
    t = 0.7 + 0.3 * xo - 0.02 * xo ** 2 + 0.5 * yo + 0.011 * yo ** 2 - 0.03 * xo * yo
    assert np.abs(oracle_mod.quadri(f, xo, yo) - t).max() < 1e-11
    # integer points return the pixel itself
    ix, iy = rng.integers(0, D, 200), rng.integers(0, D, 200)
    assert np.array_equal(oracle_mod.quadri(f, ix.astype(float), iy.astype(float)), f[iy, ix])


def test_rot_shift2d_identity_mirror_and_integer_shift(oracle_mod):
    rng = np.random.default_rng(5)
    for D in (64, 65):
        img = rng.standard_normal((D, D)).astype(np.float32)
        assert np.array_equal(oracle_mod.rot_shift2d(img, 0.0, 0.0, 0.0, 0), img.astype(np.float64))
        mir = oracle_mod.rot_shift2d(img, 0.0, 0.0, 0.0, 1)
        cols = (D - np.arange(D)) % D
        assert np.array_equal(mir, img[:, cols].astype(np.float64))
        # an integer shift moves the content by (+sx, +sy); pixels whose source
        # leaves the image keep their own value
        sh = oracle_mod.rot_shift2d(img, 0.0, 3.0, -2.0, 0)
        assert np.array_equal(sh[2:D - 3, 3:], img[4:D - 1, :D - 3].astype(np.float64))
        assert np.array_equal(sh[:, :3], img[:, :3].astype(np.float64))


def test_rot_shift2d_quarter_turn(oracle_mod):
    """90 degrees about (D/2, D/2): output (ix, iy) samples (D/2 - (iy - D/2),
    D/2 + (ix - D/2)) up to cos(90) rounding."""
    D = 48
    img = np.random.default_rng(7).standard_normal((D, D)).astype(np.float32)
    out = oracle_mod.rot_shift2d(img, 90.0, 0.0, 0.0, 0)
    h = D // 2
    for iy in range(4, D - 4):
        for ix in range(4, D - 4):
            assert abs(out[iy, ix] - img[h + (ix - h), h - (iy - h)]) < 1e-5


def test_tanl_fshift(oracle_mod):
    D = 64
    rng = np.random.default_rng(11)
    img = rng.standard_normal((D, D))
    assert np.abs(oracle_mod.tanl_fshift(img, 0.0, 0.2, 0.0, 0.0) - img).max() < 1e-12
    assert np.abs(oracle_mod.tanl_fshift(img, 0.0, 0.2, 5.0, -3.0) - np.roll(img, (-3, 5), (0, 1))).max() < 1e-12
    # a plane wave at (kx, ky) = (6, 4) is scaled by the filter's response there
    yy, xx = np.meshgrid(np.arange(D), np.arange(D), indexing="ij")
    wave = np.cos(2 * np.pi * (6 * xx + 4 * yy) / D)
    fl, ff = 0.1, 0.2
    r = np.hypot(6, 4) / D
    k = np.pi / (2 * ff * fl)
    h = 0.5 * (np.tanh(k * (r + fl)) - np.tanh(k * (r - fl)))
    assert np.abs(oracle_mod.tanl_fshift(wave, fl, ff, 0.0, 0.0) - h * wave).max() < 1e-12
    # ff = 0: the step
    assert np.abs(oracle_mod.tanl_fshift(wave, 0.2, 0.0, 0.0, 0.0) - wave).max() < 1e-12
    assert np.abs(oracle_mod.tanl_fshift(wave, 0.1, 0.0, 0.0, 0.0)).max() < 1e-12


def test_class_averages_invert_the_alignment(oracle_mod):
    """Particles = references turned, shifted and mirrored (no noise); the
    oracle's multi-reference search finds their parameters and the averaging
    step with them reproduces each reference inside the mask (no filter, no
    centring); the re-centred parameters have zero mean shift per group."""
    P, R, D = 24, 3, 64
    st = synth.make_stack(P, D, R, 2, None, 24.0, 7)
    cfg = oracle_mod.make_cfg(P, R, D, 25, 256, 1.0, 2.0, 2.0)
    lay = oracle_mod.reference_layout(cfg)
    peak, d = oracle_mod.multi_ref_align(cfg, lay, st.particles, st.refs)
    bel = np.argmax(d, axis=0)
    assert np.array_equal(bel, st.cls)
    avg, params, members, shifts = oracle_mod.class_averages(st.particles, peak, bel, 0.0, 0.2, center=False)
    assert members.tolist() == np.bincount(bel, minlength=R).tolist()
    mask = synth._mask(D, 24)
    for r in range(R):
        if members[r]:
            assert np.corrcoef(avg[r][mask], st.refs[r][mask])[0, 1] > 0.995
    mirrored = params[:, 3] != 0
    for r in range(R):
        sel = bel == r
        sx = np.where(mirrored[sel], -params[sel, 1], params[sel, 1])
        assert abs(sx.mean()) < 1e-5 and abs(params[sel, 2].mean()) < 1e-5
    # the parameters before centring are the caller's conversion of the peaks
    ang, sxc, syc, mir = oracle_mod.ormq_post(peak[bel, np.arange(P)])
    assert np.allclose(params[:, 0], ang)
    assert np.allclose(params[:, 1], np.where(mir == 0, sxc - shifts[bel, 0], sxc + shifts[bel, 0]), atol=1e-5)


def test_class_averages_centre_moves_average(oracle_mod):
    """Centring moves a group's average by minus its mean shift: with every
    member carrying the same extra shift the centred average equals the
    uncentred one moved back."""
    D, P = 32, 6
    rng = np.random.default_rng(2)
    imgs = rng.standard_normal((P, D, D)).astype(np.float32)
    peaks = np.zeros((1, P, 4), np.float32)
    peaks[0, :, 1] = -2.0  # converted sx = +2 at angle 0
    bel = np.zeros(P, np.int64)
    a0, _, _, sh = oracle_mod.class_averages(imgs, peaks, bel, 0.0, 0.2, center=False)
    a1, prm, _, _ = oracle_mod.class_averages(imgs, peaks, bel, 0.0, 0.2, center=True)
    assert np.allclose(sh[0], [2.0, 0.0])
    assert np.abs(a1[0] - np.roll(a0[0], -2, axis=1)).max() < 1e-9
    assert np.allclose(prm[:, 1], 0.0)


def test_base_shifts_invert_the_caller_conversion(oracle_mod):
    """gpuisac.isac.base_shifts_of gives back the alignment's shift from the
    parameters the caller's conversion made of it, at any angle."""
    from gpuisac.isac import base_shifts_of
    rng = np.random.default_rng(12)
    n = 1000
    peak = np.zeros((n, 4))
    peak[:, 0] = rng.uniform(0.0, 360.0, n)
    peak[:, 1:3] = rng.uniform(-6.0, 6.0, (n, 2))
    peak[:, 3] = rng.integers(0, 2, n)
    ang, sxs, sys_, mir = oracle_mod.ormq_post(peak)
    back = base_shifts_of(np.stack([ang, sxs, sys_, mir], 1))
    assert np.abs(back - peak[:, 1:3]).max() < 1e-5
