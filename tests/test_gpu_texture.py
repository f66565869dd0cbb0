"""Pins the oracle's emulation of the texture unit's bilinear filter (8-bit
fixed-point weights, clamp, unnormalised coordinates) against the hardware
texture path the reference samples images through
(cuda/gpu_aln_noref.cu:1283-1287, 2314-2339)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def probe(cuda):
    src = os.path.join(ROOT, "tests", "gpu_probe", "tex_probe.cu")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libtex_probe.so")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler",
                        "-fPIC", "-o", so, src], check=True)
    lib = ctypes.CDLL(so)
    fp = ctypes.POINTER(ctypes.c_float)
    lib.tex_probe.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int, fp]
    lib.tex_probe.restype = ctypes.c_int

    def run(img, xy):
        img = np.ascontiguousarray(img, np.float32)
        xy = np.ascontiguousarray(xy, np.float32)
        out = np.zeros(len(xy), np.float32)
        rc = lib.tex_probe(img.ctypes.data_as(fp), img.shape[1], img.shape[0], xy.ctypes.data_as(fp), len(xy),
                           out.ctypes.data_as(fp))
        assert rc == 0
        return out
    return run


def emulate(oracle_mod, img, xy):
    H, W = img.shape
    out = np.zeros(len(xy))
    for n, (x, y) in enumerate(xy):
        ix, iy, w = oracle_mod.tex_weights(float(x), float(y))
        x0, x1 = np.clip([ix, ix + 1], 0, W - 1)
        y0, y1 = np.clip([iy, iy + 1], 0, H - 1)
        out[n] = (w[0] * float(img[y0, x0]) + w[1] * float(img[y0, x1]) + w[2] * float(img[y1, x0]) +
                  w[3] * float(img[y1, x1])) / 256.0
    return out


def test_weight_quantisation_and_rounding(probe, oracle_mod):
    # a 2x1 ramp 0 -> 256: the filtered value is 256 * weight
    img = np.array([[0.0, 256.0]], np.float32)
    fr = np.concatenate([np.arange(0, 1, 1.0 / 1024), np.arange(0.5 / 256, 1, 1.0 / 256)])  # incl. exact ties
    xy = np.stack([0.5 + fr, np.full_like(fr, 0.5)], 1).astype(np.float32)
    hw = probe(img, xy)
    em = emulate(oracle_mod, img, xy)
    assert np.array_equal(hw, em.astype(np.float32)), np.c_[fr, hw, em][hw != em][:10]


def test_tap_weights_single_texel(probe, oracle_mod):
    """One texel of 256 on a zero image: each filtered value is one tap weight."""
    rng = np.random.default_rng(7)
    img = np.zeros((16, 16), np.float32)
    img[7, 7] = 256.0
    xy = np.stack([rng.uniform(6.5, 8.5, 6000), rng.uniform(6.5, 8.5, 6000)], 1).astype(np.float32)
    hw = probe(img, xy)
    em = emulate(oracle_mod, img, xy)
    assert np.array_equal(hw, em.astype(np.float32))


def test_random_coordinates_match(probe, oracle_mod):
    rng = np.random.default_rng(0)
    img = rng.standard_normal((48, 40)).astype(np.float32)
    xy = np.stack([rng.uniform(-3, 43, 4000), rng.uniform(-3, 51, 4000)], 1).astype(np.float32)
    hw = probe(img, xy)
    em = emulate(oracle_mod, img, xy)
    assert np.abs(hw - em).max() <= 2e-6 * np.abs(img).max()
