"""Polar resampling + normalisation + ring FFT on the GPU against the oracle
(FP64), through the C-ABI (gpuisac_spectra_device*)."""
import ctypes

import numpy as np
import pytest

from gpuisac import synth

pytestmark = pytest.mark.gpu

TOL = 2e-5  # |GPU - FP64 oracle| / max |F| of the ring, FP32 sampling + FFT


def decode(gpu, is_ref):
    """[n][S][NR][128][2] (a, b) basis -> complex [n][S][NR][129]"""
    a, b = gpu[..., 0].astype(np.float64), gpu[..., 1].astype(np.float64)
    re, im = 0.5 * (a + b), 0.5 * (a - b)
    n, S, NR, _ = re.shape
    out = np.zeros((n, S, NR, 129), np.complex128)
    out[..., 1:128] = re[..., 1:] + 1j * im[..., 1:]
    out[..., 0] = re[..., 0]
    out[..., 128] = im[..., 0]
    if is_ref:
        out /= np.arange(1, NR + 1)[None, None, :, None]
    return out


def run_gpu(gpulib, cuda, imgs, cfg, is_ref, base=None, layout=None):
    import torch
    from gpuisac import _lib
    t = torch.from_numpy(np.ascontiguousarray(imgs)).to(cuda)
    n = imgs.shape[0]
    S = 1 if is_ref else gpulib.gpuisac_shift_count(ctypes.byref(cfg))
    out = torch.empty((n, S, cfg.ring_num, 128, 2), dtype=torch.float32, device=cuda)
    bt = None if base is None else torch.from_numpy(np.ascontiguousarray(base, np.float32)).to(cuda)
    st = torch.cuda.current_stream(cuda).cuda_stream
    if layout is None:
        rc = gpulib.gpuisac_spectra_device(ctypes.byref(cfg), t.data_ptr(), n, int(is_ref),
                                           None if bt is None else bt.data_ptr(), out.data_ptr(), st)
    else:
        rc = gpulib.gpuisac_spectra_device_layout(ctypes.byref(cfg), t.data_ptr(), n, int(is_ref),
                                                  None if bt is None else bt.data_ptr(), layout[0], layout[1],
                                                  out.data_ptr(), st)
    if rc:
        _lib.check(gpulib)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def oracle_spectra(oracle_mod, imgs, ocfg, lay, is_ref, base=None):
    shifts = [(0.0, 0.0)] if is_ref else oracle_mod.shift_array(ocfg.shift_rng_x, ocfg.shift_rng_y, ocfg.shift_step)
    res = []
    for i in range(imgs.shape[0]):
        b = None if base is None else base[i]
        res.append([oracle_mod.spectra(ocfg, lay, imgs, i, is_ref, tuple(map(float, s)), b) for s in shifts])
    return np.array(res)


def check(gpu_c, orc_c):
    scale = np.abs(orc_c).max(axis=-1, keepdims=True)
    err = np.abs(gpu_c - orc_c) / scale
    assert err.max() < TOL, err.max()


def cfgs(n_sbj, n_ref, D, NR, rng_xy, step=1.0):
    from gpuisac import make_config
    import oracle
    return (make_config(n_sbj, n_ref, D, NR, 256, step, rng_xy, rng_xy),
            oracle.make_cfg(n_sbj, n_ref, D, NR, 256, step, rng_xy, rng_xy))


def test_texture_limit_is_reported(gpulib):
    assert gpulib.get_texture_limit(76) > 0


@pytest.mark.parametrize("D,NR,rng", [(64, 29, 2.0), (76, 35, 3.0), (65, 30, 1.0)])
def test_subject_spectra_match_oracle(gpulib, cuda, oracle_mod, D, NR, rng):
    st = synth.make_stack(5, D, 2, 2, 0.1, D * 0.4, 21)
    gcfg, ocfg = cfgs(5, 2, D, NR, rng)
    tex = gpulib.get_texture_limit(D)
    lay = oracle_mod.OrcLayout(oracle_mod.reference_layout(ocfg).sbj_batch, tex, 2)
    gpu = decode(run_gpu(gpulib, cuda, st.particles, gcfg, False), False)
    check(gpu, oracle_spectra(oracle_mod, st.particles, ocfg, lay, False))


def test_reference_spectra_match_oracle(gpulib, cuda, oracle_mod):
    st = synth.make_stack(1, 76, 7, 0, 0.0, 34.0, 22)
    gcfg, ocfg = cfgs(1, 7, 76, 35, 3.0)
    lay = oracle_mod.OrcLayout(1, gpulib.get_texture_limit(76), 7)
    gpu = decode(run_gpu(gpulib, cuda, st.refs, gcfg, True), True)
    check(gpu, oracle_spectra(oracle_mod, st.refs, ocfg, lay, True))


def test_fractional_base_shifts(gpulib, cuda, oracle_mod):
    st = synth.make_stack(6, 64, 2, 2, 0.1, 26.0, 23)
    base = np.random.default_rng(3).uniform(-1.7, 1.7, (6, 2)).astype(np.float32)
    gcfg, ocfg = cfgs(6, 2, 64, 29, 1.0)
    lay = oracle_mod.OrcLayout(oracle_mod.reference_layout(ocfg).sbj_batch, gpulib.get_texture_limit(64), 2)
    gpu = decode(run_gpu(gpulib, cuda, st.particles, gcfg, False, base=base), False)
    check(gpu, oracle_spectra(oracle_mod, st.particles, ocfg, lay, False, base=base))


@pytest.mark.parametrize("batch,tex", [(7, 7), (3, 2), (4, 3), (2, 5)])
def test_stacked_reads_batches_and_textures(gpulib, cuda, oracle_mod, batch, tex):
    """Rings larger than the image: taps read neighbouring images of the same
    texture, clamp at texture ends, and read stale slots in a short final batch."""
    rng = np.random.default_rng(batch * 10 + tex)
    imgs = rng.standard_normal((7, 32, 32)).astype(np.float32) + np.arange(7, dtype=np.float32)[:, None, None]
    gcfg, ocfg = cfgs(7, 1, 32, 20, 2.0)
    lay = oracle_mod.OrcLayout(batch, tex, 1)
    gpu = decode(run_gpu(gpulib, cuda, imgs, gcfg, False, layout=(batch, tex)), False)
    check(gpu, oracle_spectra(oracle_mod, imgs, ocfg, lay, False))


def test_single_ring_and_no_shift(gpulib, cuda, oracle_mod):
    st = synth.make_stack(3, 48, 1, 0, 0.2, 20.0, 24)
    gcfg, ocfg = cfgs(3, 1, 48, 1, 0.0)
    lay = oracle_mod.OrcLayout(3, gpulib.get_texture_limit(48), 1)
    gpu = decode(run_gpu(gpulib, cuda, st.particles, gcfg, False), False)
    check(gpu, oracle_spectra(oracle_mod, st.particles, ocfg, lay, False))


@pytest.mark.parametrize("n,batch,tex", [(20, 7, 3), (33, 10, 10), (9, 9, 4)])
def test_texture_unit_equals_emulation_on_stacked_layouts(gpulib, cuda, monkeypatch, n, batch, tex):
    """The spectra sampled through the texture unit (TexStack: batches,
    textures, stale slots of a short final batch) and through its emulation
    (GPUISAC_TEXTURE=0) on layouts where edge taps read neighbouring and
    stale images: the tap weights are the texture unit's own, so the spectra
    agree to the blend's rounding (1e-5 of the row's largest value)."""
    from gpuisac import make_config
    D, NR = 32, 15      # rings reach the image edge: taps cross into neighbours
    rng = np.random.default_rng(n * 100 + batch)
    imgs = rng.standard_normal((n, D, D)).astype(np.float32)
    base = (np.round(rng.uniform(-1.5, 1.5, (n, 2)) * 64) / 64).astype(np.float32)
    cfg = make_config(n, 1, D, NR, 256, 1.0, 2.0, 2.0)
    monkeypatch.setenv("GPUISAC_TEXTURE", "0")
    emu = run_gpu(gpulib, cuda, imgs, cfg, False, base=base, layout=(batch, tex))
    monkeypatch.setenv("GPUISAC_TEXTURE", "1")
    hw = run_gpu(gpulib, cuda, imgs, cfg, False, base=base, layout=(batch, tex))
    scale = np.abs(emu).reshape(n, -1).max(1)
    err = np.abs(hw - emu).reshape(n, -1).max(1) / scale
    assert err.max() <= 1e-5, err.max()
