"""The CPU alignment's entry shapes on the GPU path, batched: ``ormq``
(bin/sp_isac_alignment.py:400-447) and the masked normalisation ISAC applies
before every alignment call (``normalize.mask``, bin/sp_isac2_gpu.py:925-931).

``ormq`` keeps the reference's argument meaning -- shift ranges ``xrng`` /
``yrng`` with ``step``, ring layout ``numr`` from ``Numrinit``, centre
``cnx`` / ``cny`` in FORTRAN (1-based) convention, ``mode``, ``delta`` -- and
its return values (ang, sxs, sys, mirror, peak), for a stack of images
against one reference or against a stack of references.  It runs the
multi-reference alignment of this library (the reference GPU path's
semantics: every ring sampled at the last ring's length, ring weights r+1)
and the caller's conversion of the shifts (bin/sp_isac2_gpu.py:1015-1022).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GpuIsacError
from .align import multi_ref_align, multi_ref_align_device


def numr_rings(numr) -> tuple[int, int]:
    """(ring count, ring length) of a Numrinit layout: triples (radius, start,
    length).  The GPU path samples rings 1, 2, .., N at one length; the
    layout must start at radius 1 with step 1."""
    a = [int(round(float(v))) for v in numr]
    if len(a) % 3 or not a:
        raise ValueError("numr must hold (radius, start, length) triples")
    radii = a[0::3]
    if radii != list(range(1, len(radii) + 1)):
        raise ValueError(f"rings must be 1..N step 1 on this path (got radii {radii[:4]}...)")
    return len(radii), a[-1]


def _shift_range(rng, step: float) -> float:
    lo, hi = float(rng[0]), float(rng[-1])
    if abs(lo - hi) > 1e-6:
        raise ValueError(f"the shift grid is symmetric on this path: {rng} is not")
    return hi


def ormq(images, refs, xrng, yrng, step, mode, numr, cnx, cny, delta: float = 0.0,
         contraction_mode: str | None = None):
    """Best (angle, shift, mirror) of every image against every reference.

    images: [P][D][D] (numpy, or a CUDA torch tensor for the device path);
    refs: one reference [D][D] or a stack [R][D][D].  Returns (ang, sxs, sys,
    mirror, peak) as arrays [P] for one reference or [R][P], the values
    ormq() returns per image: ang in degrees, (sxs, sys) the negated search
    shift rotated by -ang, mirror 0/1, peak the correlation maximum.
    """
    if str(mode).upper() != "F":
        raise ValueError("only full-circle mode 'F' is on this path (the reference's GPU path is full-circle)")
    if float(delta) != 0.0:
        raise ValueError("delta != 0 (restricted angular search) is not on this path")
    ring_num, ring_len = numr_rings(numr)
    if ring_len not in (256, 512):
        raise ValueError(f"the last ring's length is {ring_len}; this path samples every ring at 256 "
                         "(the reference GPU path's ring length) or 512")
    sx_r, sy_r = _shift_range(xrng, step), _shift_range(yrng, step)
    device = hasattr(images, "is_cuda") and images.is_cuda
    single = refs.ndim == 2
    if single:
        refs = refs[None]
    P, D = images.shape[0], images.shape[1]
    # the search centre cnx, cny (1-based) as a base shift of the sampling
    # centre D/2 (0-based) of every image
    bx, by = float(cnx) - 1.0 - D // 2, float(cny) - 1.0 - D // 2
    if device:
        import torch
        base = torch.tensor([bx, by], dtype=torch.float32, device=images.device).repeat(P, 1)
        d, pk = multi_ref_align_device(images, refs, ring_num, sx_r, sy_r, float(step), base_shifts=base,
                                       contraction_mode=contraction_mode, ring_len=ring_len)
        d, pk = d.cpu().numpy(), pk.cpu().numpy()
    else:
        base = np.tile(np.array([bx, by], np.float32), (P, 1))
        pl, d = multi_ref_align(np.asarray(images, np.float32), np.asarray(refs, np.float32), ring_num, sx_r, sy_r,
                                float(step), base_shifts=base, contraction_mode=contraction_mode, ring_len=ring_len)
        pk = pl.reshape(refs.shape[0], P, 4)
    pk = pk.astype(np.float64)
    ang = pk[..., 0]
    sx, sy = -(pk[..., 1] - bx), -(pk[..., 2] - by)  # ormq's sx = -ix: the search shift alone
    c, s = np.cos(np.radians(ang)), -np.sin(np.radians(ang))
    out = (ang, sx * c - sy * s, sx * s + sy * c, pk[..., 3].astype(np.int32), d.astype(np.float64))
    return tuple(o[0] for o in out) if single else out


def normalize_mask(imgs, mask, no_sigma: bool, stream=None):
    """In place on a CUDA torch stack [n][D][D]: per image, subtract the mean
    of the pixels under mask (> 0.5) and, unless no_sigma, divide by their
    population standard deviation (gpuisac_normalize_mask).  References take
    no_sigma=True, particles no_sigma=False, as bin/sp_isac2_gpu.py:925-931."""
    import torch

    if not (imgs.is_cuda and imgs.dtype == torch.float32 and imgs.is_contiguous()):
        raise GpuIsacError("normalize_mask needs a contiguous float32 CUDA tensor")
    mask = torch.as_tensor(mask, dtype=torch.float32, device=imgs.device).contiguous()
    if mask.shape != imgs.shape[1:]:
        raise ValueError("mask must be [D][D] like one image")
    L = _lib.load()
    st = stream if stream is not None else torch.cuda.current_stream(imgs.device)
    if L.gpuisac_normalize_mask(imgs.data_ptr(), imgs.shape[0], imgs.shape[1], mask.data_ptr(), int(bool(no_sigma)),
                                st.cuda_stream):
        _lib.check(L)
    return imgs
