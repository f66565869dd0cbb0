"""The stability test's multigroup alignment (ref_free_alignment_2D_init /
_filter_references / ref_free_alignment_2D / gpu_clear,
cuda/gpu_aln_noref.cu:782-1005) against the oracle, iteration by iteration
on the GPU's own previous state (so that tolerances do not compound):

* filter: the averages after _filter_references against the oracle's FP64
  restatement of the tangent filter on the averages before it (per image,
  within 2e-5 of its largest value);
* alignment: every particle's new (shift, mirror) against the oracle's
  pre-alignment rule on the FP64 correlation with its class average at its
  accumulated shift (identical on >= 95 % of particles, angles within 0.05
  degrees where they agree -- near-ties may flip);
* averages: the new class averages against the oracle's transform + average
  of the particles with the GPU's new parameters (within 1e-5 of the image's
  largest value: the same texels and weights, only the bilinear blend's
  rounding may differ)."""
import ctypes

import numpy as np
import pytest

from gpuisac import synth
from gpuisac.multigroup import multigroup_refinement

pytestmark = pytest.mark.gpu

SAME, ANGLE_TOL, AVG_RTOL, FILTER_RTOL = 0.95, 0.05, 1e-5, 2e-5


def circ(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def class_stack(P, D, R, seed, snr=0.3):
    st = synth.make_stack(P, D, R, 2, snr, 0.37 * D, seed)
    order = np.argsort(st.cls, kind="stable")
    cls = st.cls[order]
    parts = np.ascontiguousarray(st.particles[order])
    # renumber so that the classes present are 0..R'-1
    _, cid = np.unique(cls, return_inverse=True)
    return parts, cid.astype(np.int64)


class Session:
    def __init__(self, parts, cid, NR, rng, avgs=None, shifts=None):
        from gpuisac import _lib
        from gpuisac._lib import AlignParam
        from gpuisac.align import make_config, ptr_array
        self.L = L = _lib.load()
        self.parts, self.cid = parts, cid
        self.P, self.D = parts.shape[0], parts.shape[1]
        self.R = int(cid[-1]) + 1
        if avgs is None:
            avgs = np.stack([parts[cid == k].mean(0) for k in range(self.R)]).astype(np.float32)
        self.avgs0 = np.ascontiguousarray(avgs, np.float32)
        cfg = make_config(self.P, self.R, self.D, NR, 256, 1.0, rng, rng, b"multigroup_aln")
        self.cfg = cfg
        addr = L.ref_free_alignment_2D_init(ctypes.byref(cfg), ptr_array(parts), ptr_array(self.avgs0),
                                            (ctypes.c_int * self.P)(*[int(c) for c in cid]), 0)
        assert addr, _lib.last_error(L)
        self.prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))
        if shifts is not None:
            for i in range(self.P):
                self.prm[i].shift_x, self.prm[i].shift_y = float(shifts[i, 0]), float(shifts[i, 1])
        self._lib = _lib

    def params(self):
        p = self.prm
        return np.array([[p[i].shift_x, p[i].shift_y, p[i].angle, float(p[i].mirror)] for i in range(self.P)],
                        np.float32)

    def averages(self):
        out = np.zeros((self.R, self.D, self.D), np.float32)
        assert self.L.gpuisac_ref_free_averages(out.ctypes.data) == 0
        return out

    def step(self):
        self.L.ref_free_alignment_2D()
        self._lib.check(self.L)

    def filter(self, freq, falloff):
        self.L.ref_free_alignment_2D_filter_references(ctypes.c_float(freq), ctypes.c_float(falloff))
        self._lib.check(self.L)

    def close(self):
        self.L.gpu_clear()


def oracle_params(oracle_mod, parts, avgs, cid, NR, rng, step, base, tex):
    P, D = parts.shape[0], parts.shape[1]
    R = avgs.shape[0]
    cfg = oracle_mod.make_cfg(P, R, D, NR, 256, step, rng, rng)
    lay = oracle_mod.OrcLayout(P, tex, R)
    shifts = oracle_mod.shift_array(rng, rng, step)
    out = []
    for p in range(P):
        c = oracle_mod.pair_ccf(cfg, lay, parts, avgs, p, int(cid[p]), base_shifts=base)
        out.append(oracle_mod.pre_align_param(c, shifts, base[p], D, NR))
    return np.array([[o[0], o[1], o[2], float(o[3])] for o in out], np.float32)


def compare_params(gpu, orc):
    same = (gpu[:, 0] == orc[:, 0]) & (gpu[:, 1] == orc[:, 1]) & (gpu[:, 3] == orc[:, 3])
    assert same.mean() >= SAME, (same.mean(), np.nonzero(~same)[0])
    assert (circ(gpu[same, 2], orc[same, 2]) < ANGLE_TOL).all()


def close_images(got, want, rtol):
    for k in range(want.shape[0]):
        scale = max(np.abs(want[k]).max(), 1e-30)
        err = np.abs(got[k].astype(np.float64) - want[k]).max() / scale
        assert err <= rtol, (k, err)


def check_iteration(oracle_mod, s, NR, rng, tex, freq=None, falloff=0.2):
    if freq is not None:
        before = s.averages()
        s.filter(freq, falloff)
        close_images(s.averages(), oracle_mod.tanl_filter_averages(before, freq, falloff), FILTER_RTOL)
    avgs, base = s.averages(), s.params()[:, :2].copy()
    s.step()
    gpu = s.params()
    compare_params(gpu, oracle_params(oracle_mod, s.parts, avgs, s.cid, NR, rng, 1.0, base, tex))
    want = oracle_mod.multigroup_averages(s.parts, gpu[:, [2, 0, 1]], gpu[:, 3] != 0, s.cid, tex)
    close_images(s.averages(), want, AVG_RTOL)
    return gpu


@pytest.mark.parametrize("D,NR,P,R,filt", [(64, 29, 48, 4, False), (76, 35, 40, 3, True), (33, 14, 36, 3, True)])
def test_iterations_match_oracle(gpulib, cuda, oracle_mod, D, NR, P, R, filt):
    parts, cid = class_stack(P, D, R, seed=90 + D)
    tex = gpulib.get_texture_limit(D)
    s = Session(parts, cid, NR, 2.0)
    try:
        for it in range(3):
            check_iteration(oracle_mod, s, NR, 2.0, tex, freq=(0.1 + 0.15 * it) if filt else None)
    finally:
        s.close()


def test_start_shifts_clamp_and_reset_shifts(gpulib, cuda, oracle_mod):
    """Fractional starting shifts written into the AlignParam array after
    init, some beyond the clamp limit img_dim - ring_num - 2 = 33; then
    reset_shifts to a grid of the same length between iterations."""
    D, NR, P = 64, 29, 30
    parts, cid = class_stack(P, D, 3, seed=7)
    rs = np.random.default_rng(3)
    start = (np.round(rs.uniform(-2.5, 2.5, (P, 2)) * 64) / 64).astype(np.float32)
    start[:3] = [[40.0, -35.5], [-34.25, 0.5], [33.0, 33.0]]
    tex = gpulib.get_texture_limit(D)
    s = Session(parts, cid, NR, 2.0, shifts=start)
    try:
        first = check_iteration(oracle_mod, s, NR, 2.0, tex)
        assert (np.abs(first[:, :2]) <= 33.0).all()
        s.L.reset_shifts(ctypes.c_float(1.0), ctypes.c_float(0.5))
        s._lib.check(s.L)
        avgs, base = s.averages(), s.params()[:, :2].copy()
        s.step()
        gpu = s.params()
        # grid after reset_shifts: range 1, step 0.5 (25 entries, as before)
        orc = []
        cfg = oracle_mod.make_cfg(P, s.R, D, NR, 256, 0.5, 1.0, 1.0)
        lay = oracle_mod.OrcLayout(P, tex, s.R)
        shifts = oracle_mod.shift_array(1.0, 1.0, 0.5)
        for p in range(P):
            c = oracle_mod.pair_ccf(cfg, lay, parts, avgs, p, int(cid[p]), base_shifts=base)
            orc.append(oracle_mod.pre_align_param(c, shifts, base[p], D, NR))
        compare_params(gpu, np.array([[o[0], o[1], o[2], float(o[3])] for o in orc], np.float32))
    finally:
        s.close()


def test_one_particle_classes(gpulib, cuda, oracle_mod):
    """Every class a single particle: its average is the particle itself,
    transformed."""
    D, NR, P = 48, 20, 6
    parts, _ = class_stack(P, D, 2, seed=11)
    cid = np.arange(P)
    tex = gpulib.get_texture_limit(D)
    s = Session(parts, cid, NR, 1.0)
    try:
        check_iteration(oracle_mod, s, NR, 1.0, tex, freq=0.3)
    finally:
        s.close()


def test_python_driver_equals_session(gpulib, cuda):
    D, NR, P = 64, 29, 40
    parts, cid = class_stack(P, D, 4, seed=5)
    got, avg = multigroup_refinement(parts, cid, NR, 2.0, 2.0, num_iter=3, cutoff_freq=0.4, falloff=0.2,
                                     return_averages=True)
    s = Session(parts, cid, NR, 2.0)
    try:
        for i in range(3):
            s.filter(0.1 + (0.4 - 0.1) * i / 2.0, 0.2)
            s.step()
        want = s.params()
        np.testing.assert_array_equal(got[:, [1, 2, 0, 3]], want)
        np.testing.assert_array_equal(avg, s.averages())
    finally:
        s.close()


def test_size_check_and_session_end(gpulib, cuda):
    from gpuisac import _lib, make_config
    L = _lib.load()
    cfg = make_config(2000, 10, 76, 35, 256, 1.0, 2.0, 2.0, b"multigroup_aln")
    assert L.ref_free_alignment_2D_size_check(ctypes.byref(cfg), 0, ctypes.c_float(0.9), False)
    huge = make_config(40_000_000, 1000, 256, 35, 256, 1.0, 2.0, 2.0, b"multigroup_aln")
    assert not L.ref_free_alignment_2D_size_check(ctypes.byref(huge), 0, ctypes.c_float(0.9), False)
    parts, cid = class_stack(12, 32, 2, seed=1)
    s = Session(parts, cid, 12, 1.0)
    s.step()
    s.close()
    L.gpuisac_clear_error()
    L.ref_free_alignment_2D()
    assert _lib.last_error(L)[0] == 3
    L.gpuisac_clear_error()
