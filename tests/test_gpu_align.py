"""The whole multi-reference alignment on the GPU, through the C-ABI, against
the FP64 oracle.

Parity bar (floating point): peak values within 1e-4 relative of the FP64
oracle; the same best (ref, angle, sx, sy, mirror) for >= 99.5% of particles
(angle compared circularly within ANGLE_TOL degrees).
"""
import numpy as np
import pytest

from gpuisac import synth

pytestmark = pytest.mark.gpu

PEAK_RTOL = 1e-4
ANGLE_TOL = 0.05
SAME_BEST = 0.995
SAME_PAIR = 0.99


def circ_diff(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def cs_bound(ring_num, ring_len=256):
    """Cauchy-Schwarz bound of a peak value: both polar images are normalised
    to weighted mean 0 and weighted variance 1 (weights r+1), and the
    unnormalised inverse FFT of the unnormalised ring spectra multiplies the
    weighted dot product by L, so |d| <= L * L * sum_r (r+1)."""
    return float(ring_len) * ring_len * ring_num * (ring_num + 1) / 2.0


# Peaks below this fraction of the bound (|normalised correlation| < 1%) are
# near-total cancellations: their rounding error is set by the magnitudes
# summed, not by the peak, so they are held to 1e-4 of 1% of the bound.
NEAR_ZERO = 0.01


def compare(peak_g, d_g, peak_o, d_o, ring_num=None, ring_len=256):
    """peak_* [R][P][4], d_* [R][P]; with ring_num, peak values are compared
    relative to max(|d|, NEAR_ZERO x the Cauchy-Schwarz bound)"""
    floor = NEAR_ZERO * cs_bound(ring_num, ring_len) if ring_num else 1e-30
    rel = np.abs(d_g.astype(np.float64) - d_o) / np.maximum(np.abs(d_o), floor)
    assert rel.max() <= PEAK_RTOL, rel.max()
    same_tuple = (peak_g[..., 1:] == peak_o[..., 1:]).all(-1) & (circ_diff(peak_g[..., 0], peak_o[..., 0]) < ANGLE_TOL)
    qg, qo = np.argmax(d_g, 0), np.argmax(d_o, 0)
    P = d_o.shape[1]
    best_same = (qg == qo) & same_tuple[qo, np.arange(P)]
    assert best_same.mean() >= SAME_BEST, best_same.mean()
    assert same_tuple.mean() >= SAME_PAIR, same_tuple.mean()
    return rel.max(), best_same.mean(), same_tuple.mean()


def oracle_run(oracle_mod, parts, refs, NR, rng, base=None, tex=None):
    import oracle
    P, D = parts.shape[0], parts.shape[1]
    cfg = oracle.make_cfg(P, refs.shape[0], D, NR, 256, 1.0, rng, rng)
    lay = oracle.reference_layout(cfg)
    if tex is not None:
        lay = oracle.OrcLayout(lay.sbj_batch, tex, lay.ref_batch)
    return oracle_mod.multi_ref_align(cfg, lay, parts, refs, base_shifts=base)


@pytest.fixture(scope="module")
def small_case():
    return synth.make_stack(120, 64, 12, 2, 0.1, 28.0, 31)


def test_host_abi_matches_oracle(gpulib, cuda, oracle_mod, small_case):
    from gpuisac import multi_ref_align
    st = small_case
    pl, d = multi_ref_align(st.particles, st.refs, 29, 2.0, 2.0)
    peak_g = pl.reshape(12, 120, 4)
    peak_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, 29, 2.0, tex=gpulib.get_texture_limit(64))
    compare(peak_g, d, peak_o, d_o)
    # the synthetic ground truth comes back too
    q = np.argmax(d, 0)
    assert (q == st.cls).mean() > 0.95


def test_d_pitch_leaves_other_columns(gpulib, cuda, small_case):
    """isac_d points into a wider node-wide array (bin/sp_isac2_gpu.py:995):
    only this call's columns are written."""
    import ctypes

    from gpuisac import _lib, make_config
    from gpuisac.align import ptr_array
    st = small_case
    P, R, pitch = 120, 12, 173
    cfg = make_config(P, R, 64, 29, 256, 1.0, 2.0, 2.0)
    params = gpulib.multi_ref_align_init(ctypes.byref(cfg), 0)
    assert params
    d = np.full((R, pitch), -7.0, np.float32)
    pl = np.zeros((R, 4 * P), np.float32)
    gpulib.multi_ref_align(ptr_array(st.particles), ptr_array(st.refs), pl.ctypes.data_as(_lib.float_ptr),
                           d.ctypes.data_as(_lib.float_ptr), pitch, ctypes.c_float(0.9))
    _lib.check(gpulib)
    gpulib.gpu_clear()
    assert (d[:, P:] == -7.0).all() and (d[:, :P] != -7.0).all()


def test_device_path_matches_host_path(gpulib, cuda, small_case):
    import torch

    from gpuisac import multi_ref_align, multi_ref_align_device
    st = small_case
    pl, d = multi_ref_align(st.particles, st.refs, 29, 2.0, 2.0)
    dg, pg = multi_ref_align_device(torch.from_numpy(st.particles).to(cuda), torch.from_numpy(st.refs).to(cuda),
                                    29, 2.0, 2.0)
    assert np.array_equal(dg.cpu().numpy(), d)
    assert np.array_equal(pg.cpu().numpy(), pl.reshape(12, 120, 4))


def test_two_refs_per_cta_path_and_partial_tile(gpulib, cuda, oracle_mod):
    """61 rings (more than one ring chunk, 2 references per CTA), 5 references
    (a partial tile), large box, fractional base shifts."""
    from gpuisac import multi_ref_align
    st = synth.make_stack(16, 128, 5, 1, 0.05, 60.0, 32)
    base = np.random.default_rng(1).uniform(-1.2, 1.2, (16, 2)).astype(np.float32)
    pl, d = multi_ref_align(st.particles, st.refs, 61, 1.0, 1.0, base_shifts=base)
    peak_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, 61, 1.0, base=base,
                             tex=gpulib.get_texture_limit(128))
    compare(pl.reshape(5, 16, 4), d, peak_o, d_o)


@pytest.mark.parametrize("P,R,D,NR,rng", [(1, 1, 64, 29, 2.0), (9, 3, 65, 30, 0.0), (7, 6, 48, 1, 1.0),
                                          (33, 9, 76, 35, 3.0)])
def test_edge_shapes(gpulib, cuda, oracle_mod, P, R, D, NR, rng):
    from gpuisac import multi_ref_align
    st = synth.make_stack(P, D, R, int(rng), 0.1, D * 0.4, 33 + P)
    pl, d = multi_ref_align(st.particles, st.refs, NR, rng, rng)
    peak_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, NR, rng, tex=gpulib.get_texture_limit(D))
    rel = np.abs(d.astype(np.float64) - d_o) / np.maximum(np.abs(d_o), 1e-30)
    assert rel.max() <= PEAK_RTOL
    same = (pl.reshape(R, P, 4)[..., 1:] == peak_o[..., 1:]).all(-1)
    assert same.mean() >= (1.0 if P * R < 50 else SAME_PAIR)


def test_repeated_calls_are_identical(gpulib, cuda, small_case):
    from gpuisac import multi_ref_align
    st = small_case
    a = multi_ref_align(st.particles[:40], st.refs, 29, 2.0, 2.0)
    b = multi_ref_align(st.particles[:40], st.refs, 29, 2.0, 2.0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("D,NR", [(76, 29), (76, 35), (76, 36), (76, 3), (96, 45), (128, 61)])
def test_ccf_kernel_variants_agree(gpulib, cuda, oracle_mod, D, NR, monkeypatch):
    """The warp-specialised kernel with 8 and 4 contraction warps (4 shifts
    per group up to 36 rings, 2 beyond), the single-phase tensor-memory kernel
    (up to 36 rings) and the general kernel: all but the last run the same
    arithmetic in the same order (bit-identical), the general one sums the
    rings in another order (tolerance)."""
    from gpuisac import multi_ref_align
    st = synth.make_stack(70, D, 9, 3, 0.05, D * 0.45, 41)
    runs = {}
    for sel, warps in (("", "8"), ("ws", "4"), ("tmem", "8"), ("general", "8")):
        monkeypatch.setenv("GPUISAC_CCF_KERNEL", sel)
        monkeypatch.setenv("GPUISAC_CCF_WS_WARPS", warps)
        runs[sel] = multi_ref_align(st.particles, st.refs, NR, 3.0, 3.0)
    monkeypatch.delenv("GPUISAC_CCF_KERNEL")
    monkeypatch.delenv("GPUISAC_CCF_WS_WARPS")
    for sel in ("ws", "tmem"):
        assert np.array_equal(runs[""][0], runs[sel][0]) and np.array_equal(runs[""][1], runs[sel][1]), sel
    d0, dg = runs[""][1].astype(np.float64), runs["general"][1].astype(np.float64)
    assert (np.abs(d0 - dg) / np.maximum(np.abs(dg), 1e-30)).max() <= PEAK_RTOL


@pytest.mark.parametrize("P,D,NR,base", [(300, 64, 29, False), (160, 76, 35, True)])
def test_texture_unit_matches_emulation(gpulib, cuda, monkeypatch, P, D, NR, base):
    """The whole alignment sampled through the texture unit (the default) and
    through its emulation (GPUISAC_TEXTURE=0): the same tap weights, so peak
    values agree to 1e-5 relative and the (angle, shift, mirror) tuples on
    >= 99.5 % of pairs."""
    import torch
    from gpuisac.align import multi_ref_align_device
    st = synth.make_stack(P, D, 10, 2, 0.1, 0.37 * D, 77)
    parts = torch.from_numpy(st.particles).to(cuda)
    refs = torch.from_numpy(st.refs).to(cuda)
    b = None
    if base:
        b = torch.from_numpy((np.round(np.random.default_rng(5).uniform(-1.5, 1.5, (P, 2)) * 64) / 64)
                             .astype(np.float32)).to(cuda)
    out = []
    for flag in ("0", "1"):
        monkeypatch.setenv("GPUISAC_TEXTURE", flag)
        d, pk = multi_ref_align_device(parts, refs, NR, 2.0, 2.0, base_shifts=b)
        out.append((d.cpu().numpy().astype(np.float64), pk.cpu().numpy()))
    (d0, p0), (d1, p1) = out
    assert (np.abs(d1 - d0) / np.maximum(np.abs(d0), 1e-30)).max() <= 1e-5
    same = (p1[..., 1:] == p0[..., 1:]).all(-1) & (circ_diff(p1[..., 0], p0[..., 0]) < ANGLE_TOL)
    assert same.mean() >= 0.995, same.mean()


def test_host_abi_scattered_image_pointers(gpulib, cuda, small_case):
    """multi_ref_align with image pointers that do not form runs in host
    memory (the particles of a stack reached in a shuffled order, each copy
    a separate array) goes through the pinned staging path; the result is
    bit-identical to the contiguous call."""
    import ctypes
    from gpuisac import _lib, make_config, multi_ref_align
    st = small_case
    P, D, R = st.particles.shape[0], st.particles.shape[1], st.refs.shape[0]
    pl0, d0 = multi_ref_align(st.particles, st.refs, 29, 2.0, 2.0)
    # every particle its own allocation, allocated in a shuffled order
    by_index = [None] * P
    for i in np.random.default_rng(3).permutation(P):
        by_index[i] = np.array(st.particles[i], copy=True)
    fp = _lib.float_ptr
    sp = (fp * P)(*[by_index[i].ctypes.data_as(fp) for i in range(P)])
    keep = [np.array(st.refs[i], copy=True) for i in range(R)]
    rp = (fp * R)(*[k.ctypes.data_as(fp) for k in keep])
    L = _lib.load()
    cfg = make_config(P, R, D, 29, 256, 1.0, 2.0, 2.0)
    assert L.multi_ref_align_init(ctypes.byref(cfg), 0)
    pl = np.zeros((R, 4 * P), np.float32)
    d = np.zeros((R, P), np.float32)
    try:
        L.multi_ref_align(sp, rp, pl.ctypes.data_as(fp), d.ctypes.data_as(fp), P, ctypes.c_float(0.9))
        _lib.check(L)
    finally:
        L.gpu_clear()
    assert np.array_equal(d, d0) and np.array_equal(pl, pl0.reshape(R, 4 * P))


@pytest.mark.parametrize("rx,ry", [(1.0, 0.0), (0.0, 1.0), (2.0, 1.0)])
def test_shift_grids_across_ccf_kernels(gpulib, cuda, oracle_mod, monkeypatch, rx, ry):
    """Asymmetric shift grids (3 and 15 shifts): below 4 shifts every
    particle is padded to whole shift groups of the warp-specialised kernel,
    above it groups hold the end of one particle and the start of the next;
    the single-phase kernel runs each particle's shifts on their own.  Same
    arithmetic, so bit-identical; 45 rings (2 shifts per group) against the
    oracle."""
    from gpuisac import multi_ref_align
    st = synth.make_stack(23, 76, 6, 2, 0.1, 30.0, 77)
    runs = {}
    for sel, warps in (("", "8"), ("ws", "4"), ("tmem", "8")):
        monkeypatch.setenv("GPUISAC_CCF_KERNEL", sel)
        monkeypatch.setenv("GPUISAC_CCF_WS_WARPS", warps)
        runs[sel] = multi_ref_align(st.particles, st.refs, 35, rx, ry)
    monkeypatch.delenv("GPUISAC_CCF_KERNEL")
    monkeypatch.delenv("GPUISAC_CCF_WS_WARPS")
    for sel in ("ws", "tmem"):
        assert np.array_equal(runs[""][0], runs[sel][0]) and np.array_equal(runs[""][1], runs[sel][1]), sel
    import oracle
    big = synth.make_stack(23, 96, 6, 2, 0.1, 38.0, 78)
    pl, d = multi_ref_align(big.particles, big.refs, 45, rx, ry)
    cfg = oracle.make_cfg(23, 6, 96, 45, 256, 1.0, rx, ry)
    lay = oracle.reference_layout(cfg)
    lay = oracle.OrcLayout(lay.sbj_batch, gpulib.get_texture_limit(96), lay.ref_batch)
    peak_o, d_o = oracle_mod.multi_ref_align(cfg, lay, big.particles, big.refs)
    compare(pl.reshape(6, 23, 4), d, peak_o, d_o)


def test_pinned_host_stack_matches_pageable(gpulib, cuda, small_case):
    """A contiguous stack in pinned host memory is copied straight to the
    device; pageable stacks go through the pinned staging: same results."""
    import torch
    from gpuisac import multi_ref_align
    st = small_case
    pin = torch.empty(st.particles[:48].shape, dtype=torch.float32, pin_memory=True).numpy()
    pin[...] = st.particles[:48]
    a = multi_ref_align(st.particles[:48].copy(), st.refs, 29, 2.0, 2.0)
    b = multi_ref_align(pin, st.refs, 29, 2.0, 2.0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
