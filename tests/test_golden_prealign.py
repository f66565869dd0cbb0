"""Parity of the pre-alignment path with the reference's own GPU library.

tests/golden/ref_pre_*.npz hold the AlignParam arrays the reference's
gpu_aln_pack.so returned after each pre-alignment run
(tests/golden/make_ref_golden_prealign.py: built from its sources, driven as
ali2d_base_gpu_isac_CLEAN drives it -- reset_shifts per shift step, the
average fetched per iteration, one batch or several with a short last one;
inputs regenerated bit for bit).  The oracle's chained restatement (CPU:
per-particle FP64 correlation + pre_align_param) and this library (GPU) must
both reproduce every run: (shift, mirror) identical for >= 95 % of particles,
angles within 0.05 degrees where they are."""
import ctypes
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
_spec = importlib.util.spec_from_file_location("make_ref_golden_prealign",
                                               os.path.join(GOLDEN, "make_ref_golden_prealign.py"))
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)

SAME, ANGLE_TOL = 0.95, 0.05
NAMES = [c[0] for c in gen.CASES]
TEX_ROWS = 65000


def circ(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def load(name):
    path = os.path.join(GOLDEN, f"ref_{name}.npz")
    assert os.path.exists(path), f"missing golden fixture {path}"
    z = np.load(path)
    case = gen.CASES[NAMES.index(name)]
    _, P, D, NR, batch, schedule, iters, seed = case
    parts, avg = gen.case_inputs(P, D, seed)
    assert float(z["input_sum"]) == parts.astype(np.float64).sum() + avg.astype(np.float64).sum()
    return z["params"], parts, avg, case


def compare(got, want):
    same = (got[:, 0] == want[:, 0]) & (got[:, 1] == want[:, 1]) & (got[:, 3] == want[:, 3])
    assert same.mean() >= SAME, (same.mean(), np.nonzero(~same)[0])
    assert (circ(got[same, 2], want[same, 2]) < ANGLE_TOL).all()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_reference(oracle_mod, name):
    want, parts, avg, case = load(name)
    _, P, D, NR, batch, schedule, iters, _ = case
    tex = TEX_ROWS // D
    base = np.zeros((P, 2), np.float32)
    k = 0
    for rng, step in schedule:
        cfg = oracle_mod.make_cfg(P, 1, D, NR, 256, step, rng, rng)
        lay = oracle_mod.OrcLayout(batch, tex, 1)
        grid = oracle_mod.shift_array(rng, rng, step)
        for _ in range(iters):
            got = []
            for p in range(P):
                c = oracle_mod.pair_ccf(cfg, lay, parts, avg, p, 0, base_shifts=base)
                got.append(oracle_mod.pre_align_param(c, grid, base[p], D, NR))
            got = np.array([[g[0], g[1], g[2], float(g[3])] for g in got], np.float32)
            compare(got, want[k])
            base = got[:, :2].copy()
            k += 1


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_library_reproduces_reference(gpulib, cuda, name):
    from gpuisac import _lib
    from gpuisac._lib import AlignParam
    from gpuisac.align import make_config, ptr_array
    want, parts, avg, case = load(name)
    _, P, D, NR, batch, schedule, iters, _ = case
    L = _lib.load()
    rng0, step0 = schedule[0]
    cfg = make_config(batch, 1, D, NR, 256, step0, rng0, rng0, b"pre_aln")
    addr = L.pre_align_init(P, ctypes.byref(cfg), 0)
    assert addr, _lib.last_error(L)
    prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))
    n_batches = (P + batch - 1) // batch
    k = 0
    try:
        if n_batches == 1:
            L.pre_align_fetch(ptr_array(parts), P, b"sbj_batch")
        for rng, step in schedule:
            L.reset_shifts(ctypes.c_float(rng), ctypes.c_float(step))
            for _ in range(iters):
                L.pre_align_fetch(ptr_array(avg), 1, b"ref_batch")
                for b in range(n_batches):
                    s, e = b * batch, min(P, (b + 1) * batch)
                    if n_batches > 1:
                        L.pre_align_fetch(ptr_array(np.ascontiguousarray(parts[s:e])), e - s, b"sbj_batch")
                    L.pre_align_run(s, e)
                    _lib.check(L)
                got = np.array([[prm[i].shift_x, prm[i].shift_y, prm[i].angle, float(prm[i].mirror)]
                                for i in range(P)], np.float32)
                compare(got, want[k])
                k += 1
    finally:
        L.gpu_clear()
