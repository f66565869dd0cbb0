"""Python host side of the pre-alignment path, mirroring the calls
bin/sp_isac_applications.py:1455-1660 makes (size check, init, fetch the
particles and the average, reset_shifts, run per GPU batch, read the
AlignParam array, gpu_clear), on numpy stacks instead of EMData lists."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import AlignParam, GpuIsacError
from .align import make_config, ptr_array


def pre_align(particles: np.ndarray, ref: np.ndarray, ring_num: int, shift_range: float, shift_step: float = 1.0,
              rounds: int = 1, batch: int | None = None, base_shifts: np.ndarray | None = None, device: int = 0,
              keep_session: bool = False):
    """Align every particle against the one reference image `rounds` times
    (each round starts from the shifts the previous one left), the particles
    fed to the GPU in batches of `batch` (default: all).  Returns a float32
    array [P][4]: shift_x, shift_y, angle, mirror."""
    L = _lib.load()
    particles = np.ascontiguousarray(particles, np.float32)
    ref = np.ascontiguousarray(ref, np.float32).reshape(1, particles.shape[1], particles.shape[2])
    P, D = particles.shape[0], particles.shape[1]
    B = min(batch or P, P)
    cfg = make_config(B, 1, D, ring_num, 256, shift_step, shift_range, shift_range, b"pre_aln")
    L.pre_align_init.restype = ctypes.c_ulonglong
    addr = L.pre_align_init(P, ctypes.byref(cfg), device)
    if not addr:
        _lib.check(L)
        raise GpuIsacError("pre_align_init returned NULL")
    prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))
    try:
        if base_shifts is not None:
            bs = np.asarray(base_shifts, np.float32).reshape(P, 2)
            for i in range(P):
                prm[i].shift_x, prm[i].shift_y = float(bs[i, 0]), float(bs[i, 1])
        rp = ptr_array(ref)
        L.pre_align_fetch(rp, 1, b"ref_batch")
        _lib.check(L)
        n_batches = (P + B - 1) // B
        if n_batches == 1:
            L.pre_align_fetch(ptr_array(particles), P, b"sbj_batch")
            _lib.check(L)
        for _ in range(rounds):
            for b in range(n_batches):
                s0, s1 = b * B, min(P, (b + 1) * B)
                if n_batches > 1:
                    L.pre_align_fetch(ptr_array(particles[s0:s1]), s1 - s0, b"sbj_batch")
                    _lib.check(L)
                L.pre_align_run(s0, s1)
                _lib.check(L)
        out = np.array([[prm[i].shift_x, prm[i].shift_y, prm[i].angle, float(prm[i].mirror)] for i in range(P)],
                       np.float32)
    finally:
        if not keep_session:
            L.gpu_clear()
    return out
