"""Seeded synthetic particle stacks with the shapes of the alignment workloads.

The reference's example stack ships without its pixel data, so workloads are
generated: each class phantom is a sum of 6-12 Gaussian blobs (sigma 2-8 px,
amplitude U(0.5, 1)) with centres uniform in a disk; a particle is its class
phantom mirrored (x -> -x about the centre, p = 0.5), rotated by U(0, 360)
degrees and shifted by an integer U{-s..s} per axis, plus white noise at the
requested SNR, then normalised to zero mean / unit sigma inside the mask.
References are the noise-free phantoms, normalised the same way.

Blobs are rendered analytically (a Gaussian stays a Gaussian under rotation,
mirror and shift), so the ground-truth parameters are exact.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED_BASE = 20261203


@dataclass
class Workload:
    name: str
    n_particles: int
    img_dim: int
    n_classes: int
    ring_num: int
    shift_rng: int
    snr: float
    blob_radius: float
    ring_len: int = 256
    shift_step: float = 1.0


# the five alignment workloads (index = seed offset)
WORKLOADS = {
    0: Workload("cpu_2000x64_16ref", 2000, 64, 16, 29, 2, 0.1, 28.0),
    1: Workload("mref_50000x76_200ref", 50000, 76, 200, 35, 3, 0.05, 34.0),
    3: Workload("learned_100000x76_500ref", 100000, 76, 500, 35, 3, 0.05, 34.0),
    4: Workload("largebox_200000x128_500ref", 200000, 128, 500, 61, 4, 0.03, 60.0),
}


@dataclass
class Stack:
    particles: np.ndarray   # [P, D, D] float32
    refs: np.ndarray        # [R, D, D] float32
    cls: np.ndarray         # [P] int32 true class
    angle: np.ndarray       # [P] float32 rotation in degrees
    shift: np.ndarray       # [P, 2] int32 (dx, dy)
    mirror: np.ndarray      # [P] bool
    seed: int


def _blobs(rng, n_classes, radius):
    nb = rng.integers(6, 13, size=n_classes)
    maxb = 12
    amp = rng.uniform(0.5, 1.0, size=(n_classes, maxb))
    sig = rng.uniform(2.0, 8.0, size=(n_classes, maxb))
    r = radius * np.sqrt(rng.uniform(0.0, 1.0, size=(n_classes, maxb)))
    th = rng.uniform(0.0, 2 * np.pi, size=(n_classes, maxb))
    cx, cy = r * np.cos(th), r * np.sin(th)
    amp[np.arange(maxb)[None, :] >= nb[:, None]] = 0.0
    return amp, sig, cx, cy


def _render(amp, sig, cx, cy, dim, chunk=4096):
    """images [N, D, D] of blob sums; centres relative to pixel dim//2."""
    coords = np.arange(dim, dtype=np.float64) - dim // 2
    out = np.empty((amp.shape[0], dim, dim), np.float32)
    for s in range(0, amp.shape[0], chunk):
        e = min(s + chunk, amp.shape[0])
        inv = 1.0 / (2.0 * sig[s:e] ** 2)
        gx = np.exp(-(coords[None, None, :] - cx[s:e, :, None]) ** 2 * inv[:, :, None])
        gy = np.exp(-(coords[None, None, :] - cy[s:e, :, None]) ** 2 * inv[:, :, None])
        gy *= amp[s:e, :, None]
        out[s:e] = np.einsum("nby,nbx->nyx", gy, gx, optimize=True).astype(np.float32)
    return out


def _mask(dim, radius):
    c = np.arange(dim) - dim // 2
    return (c[None, :] ** 2 + c[:, None] ** 2) <= radius ** 2


def _normalise(imgs, mask):
    m = mask[None]
    n = mask.sum()
    mean = (imgs * m).sum(axis=(1, 2)) / n
    var = ((imgs - mean[:, None, None]) ** 2 * m).sum(axis=(1, 2)) / n
    return ((imgs - mean[:, None, None]) / np.sqrt(var + 1e-12)[:, None, None]).astype(np.float32)


def make_stack(n_particles, img_dim, n_classes, shift_rng, snr, blob_radius, seed,
               mask_radius=None, mirror_p=0.5, particle_seed=None) -> Stack:
    """particle_seed: draw the particles from their own stream (same class
    phantoms as `seed`, independent particles: training / held-out splits)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    amp, sig, cx, cy = _blobs(rng, n_classes, blob_radius)
    mask = _mask(img_dim, mask_radius if mask_radius is not None else blob_radius)
    refs = _normalise(_render(amp, sig, cx, cy, img_dim), mask)
    if particle_seed is not None:
        rng = np.random.Generator(np.random.PCG64(particle_seed))

    cls = rng.integers(0, n_classes, size=n_particles).astype(np.int32)
    ang = rng.uniform(0.0, 360.0, size=n_particles).astype(np.float32)
    sh = rng.integers(-shift_rng, shift_rng + 1, size=(n_particles, 2)).astype(np.int32)
    mir = rng.uniform(size=n_particles) < mirror_p

    pcx, pcy = cx[cls].copy(), cy[cls].copy()
    pcx[mir] = -pcx[mir]
    t = np.deg2rad(ang.astype(np.float64))[:, None]
    rx = np.cos(t) * pcx - np.sin(t) * pcy + sh[:, 0:1]
    ry = np.sin(t) * pcx + np.cos(t) * pcy + sh[:, 1:2]
    parts = _render(amp[cls], sig[cls], rx, ry, img_dim)
    if snr is not None and snr > 0:
        m = mask[None]
        n = mask.sum()
        mean = (parts * m).sum(axis=(1, 2)) / n
        var = ((parts - mean[:, None, None]) ** 2 * m).sum(axis=(1, 2)) / n
        sigma_n = np.sqrt(var / snr).astype(np.float32)
        noise = rng.standard_normal(size=parts.shape, dtype=np.float32)
        parts += noise * sigma_n[:, None, None]
    parts = _normalise(parts, mask)
    return Stack(parts, refs, cls, ang, sh, mir, seed)


def workload_stack(idx: int, n_particles: int | None = None, n_refs: int | None = None,
                   split: int | None = None) -> Stack:
    """split: None for the workload's own particles; k >= 1 for an independent
    particle set over the same references (k = 1: the training set of the
    learned proposal)."""
    w = WORKLOADS[idx]
    ps = None if split is None else SEED_BASE + 1000 * split + idx
    return make_stack(n_particles or w.n_particles, w.img_dim, n_refs or w.n_classes,
                      w.shift_rng, w.snr, w.blob_radius, SEED_BASE + idx, particle_seed=ps)


def stability_classes(cls, class_size: int = 100):
    """Particle order and class ids for a stability-test run: particles sorted
    by class (stable), each class split into runs of at most class_size
    (ISAC's classes hold at most img_per_grp members).  Returns (order, cid)
    with cid the sorted runs 0..R-1."""
    order = np.argsort(np.asarray(cls), kind="stable")
    c = np.asarray(cls)[order]
    cid = np.zeros(c.size, np.int64)
    k, run, prev = -1, 0, None
    for i, v in enumerate(c):
        if v != prev or run == class_size:
            k, run, prev = k + 1, 0, v
        cid[i] = k
        run += 1
    return order, cid
