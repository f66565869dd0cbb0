"""The pre-alignment path through the reference's entry points
(pre_align_size_check / init / fetch / run, reset_shifts, gpu_clear) against
the oracle's restatement of the pre-alignment rule on the FP64 correlation
tables: single batch, batches with a short last one (its free slots keep the
previous fetch's images, as the reference's textures do), fractional
accumulated shifts, and a second round on a narrower grid."""
import ctypes

import numpy as np
import pytest

from gpuisac import synth
from gpuisac.prealign import pre_align

pytestmark = pytest.mark.gpu

SAME = 0.95        # (shift, mirror) identical on >= 95% of particles (near-ties may flip)
ANGLE_TOL = 0.05   # degrees, where (shift, mirror) agree


def circ(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def oracle_round(oracle_mod, parts, ref, NR, rng, step, base, batch, tex):
    P, D = parts.shape[0], parts.shape[1]
    cfg = oracle_mod.make_cfg(P, 1, D, NR, 256, step, rng, rng)
    lay = oracle_mod.OrcLayout(batch, tex, 1)
    shifts = oracle_mod.shift_array(rng, rng, step)
    out = []
    for p in range(P):
        c = oracle_mod.pair_ccf(cfg, lay, parts, ref[None], p, 0, base_shifts=base)
        out.append(oracle_mod.pre_align_param(c, shifts, base[p], D, NR))
    return np.array([[o[0], o[1], o[2], float(o[3])] for o in out], np.float32)


def compare(gpu, orc):
    same = (gpu[:, 0] == orc[:, 0]) & (gpu[:, 1] == orc[:, 1]) & (gpu[:, 3] == orc[:, 3])
    assert same.mean() >= SAME, (same.mean(), np.nonzero(~same)[0])
    assert circ(gpu[same, 2], orc[same, 2]).max() < ANGLE_TOL


@pytest.mark.parametrize("batch,base", [(None, False), (16, False), (16, True)])
def test_pre_align_matches_oracle(gpulib, cuda, oracle_mod, batch, base):
    P, D, NR, rng = 40, 64, 29, 2.0
    st = synth.make_stack(P, D, 1, 2, 0.3, 28.0, seed=71)
    ref = st.refs[0]
    b = np.zeros((P, 2), np.float32)
    if base:
        b = (np.round(np.random.default_rng(4).uniform(-1.5, 1.5, (P, 2)) * 64) / 64).astype(np.float32)
    gpu = pre_align(st.particles, ref, NR, rng, 1.0, batch=batch, base_shifts=b)
    tex = gpulib.get_texture_limit(D)
    orc = oracle_round(oracle_mod, st.particles, ref, NR, rng, 1.0, b, batch or P, tex)
    compare(gpu, orc)


def test_second_round_narrower_grid(gpulib, cuda, oracle_mod):
    """One session, two rounds: reset_shifts between them (same grid length:
    range 2 step 1, then range 1 step 0.5); the second round starts from the
    shifts the first one accumulated in the AlignParam array."""
    from gpuisac import _lib, make_config
    from gpuisac.align import ptr_array
    from gpuisac._lib import AlignParam
    P, D, NR = 24, 64, 29
    st = synth.make_stack(P, D, 1, 2, 0.3, 28.0, seed=72)
    ref = np.ascontiguousarray(st.refs[:1])
    L = _lib.load()
    cfg = make_config(P, 1, D, NR, 256, 1.0, 2.0, 2.0, b"pre_aln")
    addr = L.pre_align_init(P, ctypes.byref(cfg), 0)
    assert addr, _lib.last_error(L)
    prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))

    def params():
        return np.array([[prm[i].shift_x, prm[i].shift_y, prm[i].angle, float(prm[i].mirror)] for i in range(P)],
                        np.float32)
    try:
        L.pre_align_fetch(ptr_array(ref), 1, b"ref_batch")
        L.pre_align_fetch(ptr_array(st.particles), P, b"sbj_batch")
        L.pre_align_run(0, P)
        _lib.check(L)
        first = params()
        L.reset_shifts(ctypes.c_float(1.0), ctypes.c_float(0.5))
        L.pre_align_run(0, P)
        _lib.check(L)
        second = params()
    finally:
        L.gpu_clear()
    tex = gpulib.get_texture_limit(D)
    compare(first, oracle_round(oracle_mod, st.particles, ref[0], NR, 2.0, 1.0, np.zeros((P, 2), np.float32), P,
                                tex))
    compare(second, oracle_round(oracle_mod, st.particles, ref[0], NR, 1.0, 0.5, first[:, :2].copy(), P, tex))


def test_size_check_and_errors(gpulib, cuda):
    from gpuisac import _lib, make_config
    L = _lib.load()
    cfg = make_config(64, 1, 64, 29, 256, 1.0, 2.0, 2.0, b"pre_aln")
    assert L.pre_align_size_check(64, ctypes.byref(cfg), 0, ctypes.c_float(0.9), False)
    huge = make_config(4_000_000, 1, 256, 29, 256, 1.0, 2.0, 2.0, b"pre_aln")
    assert not L.pre_align_size_check(4_000_000, ctypes.byref(huge), 0, ctypes.c_float(0.9), False)
    L.gpuisac_clear_error()
    assert L.pre_align_init(8, ctypes.byref(cfg), 0)
    L.pre_align_fetch(None, 1, b"ref_batch")
    assert _lib.last_error(L)[0] == 2
    L.gpuisac_clear_error()
    L.pre_align_run(0, 8)      # no reference fetched yet
    code, msg = _lib.last_error(L)
    assert code == 3 and "reference" in msg
    L.gpuisac_clear_error()
    L.gpu_clear()
