"""Python host side of the stability test's multigroup alignment, mirroring
multigroup_refinement_gpu (bin/sp_isac_applications.py:4552-4650) on numpy
stacks instead of EMData lists: init with the particles, their classes and the
initial class averages, write the particles' starting shifts, run num_iter
iterations (the tangent filter's cut-off ramping from 0.1 to cutoff_freq
before each when cutoff_freq > 0), read the AlignParam array, gpu_clear.

The reference builds the initial averages with EMAN2's ave_series and the
starting shifts from the images' headers; here the caller passes them
(default: the plain class means and zero shifts)."""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import AlignParam, GpuIsacError
from .align import make_config, ptr_array


def multigroup_refinement(particles: np.ndarray, cid_list, ring_num: int, shift_rng_x: float, shift_rng_y: float,
                          num_iter: int, cutoff_freq: float = 0.0, falloff: float = 0.0,
                          init_averages: np.ndarray | None = None, init_shifts: np.ndarray | None = None,
                          device: int = 0, return_averages: bool = False):
    """Returns a float32 array [P][4] (angle, shift_x, shift_y, mirror) as the
    AlignParam array holds them after the last iteration, and with
    return_averages the class averages [R][D][D] the session ended with."""
    L = _lib.load()
    particles = np.ascontiguousarray(particles, np.float32)
    P, D = particles.shape[0], particles.shape[1]
    cid = np.asarray(cid_list, np.int64)
    if cid.shape != (P,):
        raise GpuIsacError("one class id per particle")
    R = int(cid[-1]) + 1
    if init_averages is None:
        init_averages = np.stack([particles[cid == k].mean(0) for k in range(R)]).astype(np.float32)
    avgs = np.ascontiguousarray(init_averages, np.float32).reshape(R, D, D)
    cfg = make_config(P, R, D, ring_num, 256, 1.0, shift_rng_x, shift_rng_y, b"multigroup_aln")
    cids = (ctypes.c_int * P)(*[int(c) for c in cid])
    addr = L.ref_free_alignment_2D_init(ctypes.byref(cfg), ptr_array(particles), ptr_array(avgs), cids, device)
    if not addr:
        _lib.check(L)
        raise GpuIsacError("ref_free_alignment_2D_init returned NULL")
    prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))
    try:
        if init_shifts is not None:
            sh = np.asarray(init_shifts, np.float32).reshape(P, 2)
            for i in range(P):
                prm[i].shift_x, prm[i].shift_y = float(sh[i, 0]), float(sh[i, 1])
        for i in range(num_iter):
            if cutoff_freq > 0.0:
                freq = 0.1 + (cutoff_freq - 0.1) * i / float(num_iter - 1)
                L.ref_free_alignment_2D_filter_references(ctypes.c_float(freq), ctypes.c_float(falloff))
                _lib.check(L)
            L.ref_free_alignment_2D()
            _lib.check(L)
        out = np.array([(prm[i].angle, prm[i].shift_x, prm[i].shift_y, float(prm[i].mirror)) for i in range(P)],
                       np.float32)
        final = None
        if return_averages:
            final = np.zeros((R, D, D), np.float32)
            if L.gpuisac_ref_free_averages(final.ctypes.data):
                _lib.check(L)
    finally:
        L.gpu_clear()
    return (out, final) if return_averages else out


def header_params(params: np.ndarray) -> np.ndarray:
    """The parameters in the form the caller writes to the images' headers
    (bin/sp_isac_applications.py:4636-4645): angle, the negated shift rotated
    by -angle, mirror."""
    out = np.zeros((params.shape[0], 4), np.float32)
    for k, (angle, sx, sy, mir) in enumerate(np.asarray(params, np.float64)):
        c, s = math.cos(math.radians(angle)), -math.sin(math.radians(angle))
        out[k] = (angle, -sx * c + sy * s, -sx * s - sy * c, mir)
    return out
