"""ctypes front-end of the CPU oracle (oracle/_build/libisac_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product path.  The C
sources restate the reference's GPU path; see isac_oracle.h for the
file:line map.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libisac_oracle.so")
_lib = None


class OrcCfg(ctypes.Structure):
    _fields_ = [("sbj_num", ctypes.c_uint), ("ref_num", ctypes.c_uint),
                ("img_dim", ctypes.c_uint), ("ring_num", ctypes.c_uint),
                ("ring_len", ctypes.c_uint), ("shift_step", ctypes.c_float),
                ("shift_rng_x", ctypes.c_float), ("shift_rng_y", ctypes.c_float)]


class OrcLayout(ctypes.Structure):
    _fields_ = [("sbj_batch", ctypes.c_uint), ("tex_limit", ctypes.c_uint),
                ("ref_batch", ctypes.c_uint)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    return any(os.path.getmtime(os.path.join(_HERE, f)) > t
               for f in ("isac_oracle.c", "isac_oracle.h", "isac_oracle_core.h", "assign_oracle.cpp"))


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        cfgp = ctypes.POINTER(OrcCfg)
        layp = ctypes.POINTER(OrcLayout)
        L.orc_polar_template.argtypes = [ctypes.c_uint, ctypes.c_uint, fp]
        L.orc_shift_array.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, fp, ctypes.c_int]
        L.orc_shift_array.restype = ctypes.c_int
        L.orc_tex_split.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_int), fp]
        L.orc_tex_weights.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.orc_reference_sbj_batch.argtypes = [cfgp]
        L.orc_reference_sbj_batch.restype = ctypes.c_uint
        for pfx, rp in (("f64", dp), ("f32", fp)):
            f = getattr(L, f"orc_{pfx}_polar")
            f.argtypes = [cfgp, layp, fp, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
                          ctypes.c_float, ctypes.c_float, fp, rp]
            f = getattr(L, f"orc_{pfx}_spectra")
            f.argtypes = [cfgp, layp, fp, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
                          ctypes.c_float, ctypes.c_float, fp, rp]
            f = getattr(L, f"orc_{pfx}_pair_ccf")
            f.argtypes = [cfgp, layp, fp, fp, ctypes.c_uint, ctypes.c_uint, fp, rp]
            f = getattr(L, f"orc_{pfx}_multi_ref_align")
            f.argtypes = [cfgp, layp, fp, fp, fp, fp, rp, ctypes.c_uint, ctypes.c_int]
        L.orc_f64_peak_search.argtypes = [dp, ctypes.c_uint, ctypes.c_uint, fp, dp,
                                          ctypes.POINTER(ctypes.c_uint)]
        L.orc_multigroup_averages.argtypes = [fp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, fp,
                                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint),
                                              ctypes.c_uint, fp]
        L.orc_multigroup_averages.restype = ctypes.c_int
        L.orc_assign_groups.argtypes = [fp, ctypes.c_uint, ctypes.c_uint, ctypes.POINTER(ctypes.c_int)]
        L.orc_assign_groups.restype = ctypes.c_int
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_cfg(sbj_num, ref_num, img_dim, ring_num, ring_len=256, shift_step=1.0,
             shift_rng_x=1.0, shift_rng_y=1.0) -> OrcCfg:
    return OrcCfg(sbj_num, ref_num, img_dim, ring_num, ring_len, shift_step, shift_rng_x, shift_rng_y)


def reference_layout(cfg: OrcCfg, tex_height: int = 65000) -> OrcLayout:
    """Image grouping the reference uses on a device whose
    maxTexture2DLinear height is tex_height (65000 on current GPUs)."""
    sb = lib().orc_reference_sbj_batch(ctypes.byref(cfg))
    return OrcLayout(max(sb, 1), max(tex_height // cfg.img_dim, 1), max(min(cfg.ref_num, 100), 1))


def polar_template(ring_num: int, ring_len: int) -> np.ndarray:
    out = np.zeros((ring_num, ring_len, 2), np.float32)
    lib().orc_polar_template(ring_num, ring_len, _fp(out))
    return out


def shift_array(rx: float, ry: float, step: float) -> np.ndarray:
    cap = 1 << 16
    out = np.zeros((cap, 2), np.float32)
    n = lib().orc_shift_array(rx, ry, step, _fp(out), cap)
    if n < 0:
        raise ValueError("bad shift grid")
    return out[:n].copy()


def tex_split(t: float):
    i = ctypes.c_int()
    a = ctypes.c_float()
    lib().orc_tex_split(t, ctypes.byref(i), ctypes.byref(a))
    return i.value, a.value


def tex_weights(x: float, y: float):
    """(ix, iy, [w00, w10, w01, w11]) in units of 1/256"""
    ix, iy = ctypes.c_int(), ctypes.c_int()
    w = (ctypes.c_int * 4)()
    lib().orc_tex_weights(x, y, ctypes.byref(ix), ctypes.byref(iy), w)
    return ix.value, iy.value, list(w)


def _real(precision):
    return (np.float64, _dp) if precision == "f64" else (np.float32, _fp)


def polar(cfg, lay, stack, img, is_ref=False, shift=(0.0, 0.0), base=None, precision="f64"):
    dt, cast = _real(precision)
    stack = np.ascontiguousarray(stack, np.float32)
    out = np.zeros((cfg.ring_num, cfg.ring_len), dt)
    b = None if base is None else np.ascontiguousarray(base, np.float32)
    rc = getattr(lib(), f"orc_{precision}_polar")(
        ctypes.byref(cfg), ctypes.byref(lay), _fp(stack), stack.shape[0], img, int(is_ref),
        shift[0], shift[1], None if b is None else _fp(b), cast(out))
    if rc:
        raise RuntimeError("oracle polar failed")
    return out


def spectra(cfg, lay, stack, img, is_ref=False, shift=(0.0, 0.0), base=None, precision="f64"):
    dt, cast = _real(precision)
    stack = np.ascontiguousarray(stack, np.float32)
    out = np.zeros((cfg.ring_num, cfg.ring_len // 2 + 1, 2), dt)
    b = None if base is None else np.ascontiguousarray(base, np.float32)
    rc = getattr(lib(), f"orc_{precision}_spectra")(
        ctypes.byref(cfg), ctypes.byref(lay), _fp(stack), stack.shape[0], img, int(is_ref),
        shift[0], shift[1], None if b is None else _fp(b), cast(out))
    if rc:
        raise RuntimeError("oracle spectra failed")
    return out[..., 0] + 1j * out[..., 1]


def pair_ccf(cfg, lay, sbj, ref, p, q, base_shifts=None, precision="f64"):
    """c[mirror][shift][tau] of one particle/reference pair."""
    dt, cast = _real(precision)
    n_shift = len(shift_array(cfg.shift_rng_x, cfg.shift_rng_y, cfg.shift_step))
    out = np.zeros((2, n_shift, cfg.ring_len), dt)
    sbj = np.ascontiguousarray(sbj, np.float32)
    ref = np.ascontiguousarray(ref, np.float32)
    b = None if base_shifts is None else np.ascontiguousarray(base_shifts, np.float32)
    rc = getattr(lib(), f"orc_{precision}_pair_ccf")(
        ctypes.byref(cfg), ctypes.byref(lay), _fp(sbj), _fp(ref), p, q,
        None if b is None else _fp(b), cast(out))
    if rc:
        raise RuntimeError("oracle pair_ccf failed")
    return out


def multi_ref_align(cfg, lay, sbj, ref, base_shifts=None, precision="f64", threads=0):
    """Returns (peak_list [R][P][4] float32, d [R][P])."""
    dt, cast = _real(precision)
    P, R = cfg.sbj_num, cfg.ref_num
    sbj = np.ascontiguousarray(sbj, np.float32)
    ref = np.ascontiguousarray(ref, np.float32)
    assert sbj.shape[0] == P and ref.shape[0] == R
    peak = np.zeros((R, P, 4), np.float32)
    d = np.zeros((R, P), dt)
    b = None if base_shifts is None else np.ascontiguousarray(base_shifts, np.float32)
    rc = getattr(lib(), f"orc_{precision}_multi_ref_align")(
        ctypes.byref(cfg), ctypes.byref(lay), _fp(sbj), _fp(ref),
        None if b is None else _fp(b), _fp(peak), cast(d), P, threads)
    if rc:
        raise RuntimeError("oracle multi_ref_align failed")
    return peak, d


def peak_search(ccf: np.ndarray):
    """First-strict-max search + parabola on ccf [2*S][L] (FP64)."""
    ccf = np.ascontiguousarray(ccf, np.float64)
    two_s, L = ccf.shape
    out = np.zeros(4, np.float32)
    pk = ctypes.c_double()
    tau = ctypes.c_uint()
    lib().orc_f64_peak_search(_dp(ccf), two_s // 2, L, _fp(out), ctypes.byref(pk), ctypes.byref(tau))
    return out, pk.value, tau.value


def pre_align_param(ccf: np.ndarray, shifts: np.ndarray, base, img_dim: int, ring_num: int):
    """The pre-alignment's parameter update of one particle from its table
    c[mirror][shift][tau] (FP64 restatement): first strict maximum from 0 at
    index 0 over (mirror, shift, tau) (cu_max_idx_silly,
    cuda/gpu_aln_noref.cu:1624-1665; the table's two padding values per block
    are not part of the correlation and are left out), the 7-point parabola
    and the angle in double precision (interpolate_angle, :2535-2577), the
    shift added to the base shift in float and clamped to
    +-(img_dim - ring_num - 2) computed in unsigned arithmetic
    (compute_alignment_param, :2463-2513).  Returns (shift_x, shift_y, angle,
    mirror) as float32 / bool."""
    c = np.asarray(ccf, np.float64)
    n_mir, S, L = c.shape
    flat = c.reshape(-1)
    best, idx = 0.0, 0
    for i in range(flat.size):   # strict >, first occurrence
        if flat[i] > best:
            best, idx = flat[i], i
    m, rest = divmod(idx, S * L)
    s, tau = divmod(rest, L)
    x = [c[m, s, (tau + i) % L] for i in range(-3, 4)]
    c2 = 49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6]
    c3 = 5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6]
    step = 360.0 / float(L)
    a = step * tau
    if c3 != 0.0:
        a = a + step * (c2 / (2.0 * c3) - 4)
    angle = np.float32(360.0 - a)
    if m:
        angle = np.float32(float(angle) + 180.0)
        if angle >= 360.0:
            angle = np.float32(float(angle) - 360.0)
    limit = np.float32((img_dim - ring_num - 2) % (1 << 32))
    sx = np.float32(np.float32(base[0]) + np.float32(shifts[s][0]))
    sy = np.float32(np.float32(base[1]) + np.float32(shifts[s][1]))
    sx = min(max(sx, -limit), limit)
    sy = min(max(sy, -limit), limit)
    return np.float32(sx), np.float32(sy), np.float32(angle), bool(m)


def assign_groups(d: np.ndarray, nref: int, nima: int) -> np.ndarray:
    """The equal-size group assignment on d[ref * nima + particle]
    (assign_oracle.cpp restates EMAN2's Util::assign_groups, which
    bin/sp_isac2_gpu.py:1119 calls): returns id_list_long, nima + 1 ints."""
    d = np.ascontiguousarray(np.asarray(d, np.float32).reshape(-1))
    if d.size != nref * nima:
        raise ValueError("d must hold nref * nima peaks")
    out = np.zeros(nima + 1, np.int32)
    rc = lib().orc_assign_groups(_fp(d), nref, nima, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc:
        raise ValueError(f"oracle assign_groups rejected its input ({rc})")
    return out


def belongsto_from_id_list(id_list_long, numref: int, nima: int) -> np.ndarray:
    """The caller's reading of the assignment (bin/sp_isac2_gpu.py:1121-1136):
    the first maxasi * numref entries fill the groups maxasi at a time, the
    next nima % maxasi entries join the group named by the last entry, and
    belongsto[particle] is its group.  (When nima % numref >= maxasi the
    caller reads fewer extras than the assignment lists and those particles
    keep group 0; that is the caller's arithmetic, restated as it is.)"""
    ids = [int(x) for x in id_list_long]
    maxasi = nima // numref
    groups = [[] for _ in range(numref)]
    for i in range(maxasi * numref):
        groups[i // maxasi].append(ids[i])
    for i in range(nima % maxasi):
        groups[ids[-1]].append(ids[maxasi * numref + i])
    belongsto = np.zeros(nima, np.int32)
    for k in range(numref):
        for i in sorted(groups[k]):
            belongsto[i] = k
    return belongsto


def class_ranges(cid_list) -> np.ndarray:
    """Class index ranges of sorted class runs 0..R-1 (the reference's
    u_cid_idx, cuda/gpu_aln_noref.cu:825-835)."""
    cid = np.asarray(cid_list, np.int64)
    R = int(cid[-1]) + 1
    idx = np.searchsorted(cid, np.arange(R + 1), side="left").astype(np.uint32)
    idx[R] = cid.size
    return idx


def multigroup_averages(stack, params, mirror, cid_list, tex: int) -> np.ndarray:
    """Class averages of the particles transformed by (angle, shift_x,
    shift_y, mirror) -- cu_transform_batch + cu_average_batch restated
    (isac_oracle.c orc_multigroup_averages).  tex: images per texture."""
    st = np.ascontiguousarray(stack, np.float32)
    n, D = st.shape[0], st.shape[1]
    prm = np.ascontiguousarray(np.asarray(params, np.float32).reshape(n, 3))
    mir = np.ascontiguousarray(np.asarray(mirror).astype(np.int32).reshape(n))
    idx = class_ranges(cid_list)
    R = idx.size - 1
    out = np.zeros((R, D, D), np.float32)
    rc = lib().orc_multigroup_averages(_fp(st), n, D, tex, _fp(prm), mir.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), R, _fp(out))
    if rc:
        raise ValueError("oracle multigroup_averages rejected its input")
    return out


def tanl_filter_averages(avg, cutoff: float, falloff: float) -> np.ndarray:
    """The averages low-passed as BatchHandler::apply_tangent_filter does it
    (cuda/gpu_aln_noref.cu:2203-2266, cu_apply_tanl_filter_to_tex :1007-1037),
    in FP64 with numpy's real FFT: factor 0.5 (tanh(c (d + fc)) - tanh(c (d -
    fc))) on the half spectrum, c = pi / (2 falloff fc), d = |(x, y)| with
    x = kx / (D/2 + 1) / 2 and y = min(ky, D - ky) / (D/2) / 2, computed in
    float as the kernel does; then the reference's host rescaling, which
    reaches only the first image: image 0 divided by D^2, the others
    multiplied by D^2."""
    a = np.asarray(avg, np.float64)
    R, D = a.shape[0], a.shape[1]
    H = D // 2 + 1
    f32 = np.float32
    c = f32(f32(3.141592653589793) / (f32(2.0) * f32(falloff) * f32(cutoff)))
    fx = (np.arange(H).astype(f32) / f32(H)) * f32(0.5)
    half = f32(D) / f32(2.0)
    ky = np.arange(D)
    fy = np.where(ky.astype(f32) < half, ky, D - ky).astype(f32)
    fy = (fy / half) * f32(0.5)
    d = np.sqrt(fx[None, :] * fx[None, :] + fy[:, None] * fy[:, None]).astype(f32)
    fc = f32(cutoff)
    h = f32(0.5) * (np.tanh(c * (d + fc)) - np.tanh(c * (d - fc)))
    out = np.fft.irfft2(np.fft.rfft2(a) * h.astype(np.float64)[None], s=(D, D))
    n = float(D * D)
    out[0] /= n
    out[1:] *= n
    return out


def normalize_mask(imgs, mask, no_sigma: bool) -> np.ndarray:
    """The caller-side masked normalisation before each alignment call
    (bin/sp_isac2_gpu.py:925-931, EMAN2's "normalize.mask" processor, restated
    from its published description; EMAN2 is not in the reference tree, so
    parity with it is unpinned): per image, the mean and population standard
    deviation (FP64) of the pixels where mask > 0.5; x <- (x - mean) / sigma,
    or x <- x - mean with no_sigma or when sigma is 0."""
    x = np.asarray(imgs, np.float64)
    sel = np.asarray(mask) > 0.5
    v = x[:, sel]
    n = max(int(sel.sum()), 1)
    mean = v.sum(1) / n
    var = (v * v).sum(1) / n - mean * mean
    sd = np.sqrt(np.maximum(var, 0.0))
    out = x - mean[:, None, None]
    if not no_sigma:
        ok = sd > 0
        out[ok] /= sd[ok][:, None, None]
    return out


def ormq_post(peak, base=None):
    """The caller's conversion of the peak parameters (bin/sp_isac2_gpu.py:
    1015-1022, the end of ormq() in bin/sp_isac_alignment.py:443-447): the
    negated shift rotated by the negated angle.  peak [..., 4] = (angle, sx,
    sy, mirror) with sx, sy relative to the search centre.  Returns (ang,
    sxs, sys, mirror) in FP64."""
    peak = np.asarray(peak, np.float64)
    ang = peak[..., 0]
    sxn, syn = -peak[..., 1], -peak[..., 2]
    c, s = np.cos(np.radians(ang)), -np.sin(np.radians(ang))
    return ang, sxn * c - syn * s, sxn * s + syn * c, peak[..., 3]


def quadri(img, xo, yo) -> np.ndarray:
    """Quadratic interpolation of one image [D][D] at 0-based coordinates
    (xo, yo) in [0, D), neighbours taken periodically: the six-point scheme of
    SPIDER's QUADRI as EMAN2's Util::quadri implements it (the interpolation
    that rot_shift2D uses by default), restated from its published definition
    in FP64.  With f00 at (i, j) = floor, dx, dy the fractions:
    f = f00 + dx (c1 + (dx - 1) c2 + dy c5) + dy (c3 + (dy - 1) c4), c1, c3
    the forward differences along x, y, c2, c4 half the second differences,
    c5 the cross term through (i + 1, j + 1).  Exact for every quadratic
    a + bx + cx^2 + dy + ey^2 + gxy away from the wrap."""
    f = np.asarray(img, np.float64)
    D = f.shape[0]
    xo = np.asarray(xo, np.float64)
    yo = np.asarray(yo, np.float64)
    i = np.floor(xo).astype(np.int64)
    j = np.floor(yo).astype(np.int64)
    dx, dy = xo - i, yo - j
    i %= D
    j %= D
    ip, im, jp, jm = (i + 1) % D, (i - 1) % D, (j + 1) % D, (j - 1) % D
    f00 = f[j, i]
    c1 = f[j, ip] - f00
    c2 = (c1 - f00 + f[j, im]) * 0.5
    c3 = f[jp, i] - f00
    c4 = (c3 - f00 + f[jm, i]) * 0.5
    c5 = f[jp, ip] - f00 - c1 - c3
    return f00 + dx * (c1 + (dx - 1.0) * c2 + dy * c5) + dy * (c3 + (dy - 1.0) * c4)


def rot_shift2d_coords(D: int, c, s, sx, sy, mirror):
    """Source coordinates (xo, yo) [D][D] (float32) that rot_shift2D(img, ang,
    sx, sy, mirror) samples for each output pixel, as EMAN2's
    rot_scale_trans2D_background (the default "background" mode) and the
    x-mirror after it define them: output column ix comes from the rotation's
    column ixs = (D - ix) mod D when mirrored (the mirror about column D/2
    keeps column 0), x = ixs - (D/2 + sx), y = iy - (D/2 + sy) and
    xo = (x c - y s) + D/2, yo = (x s + y c) + D/2 with c = cos(ang),
    s = sin(ang); a source point outside [0, D)^2 is replaced by the pixel
    (ixs, iy) itself.  Every step is one float32 operation in this order; the
    GPU kernel rounds the same operations."""
    f32 = np.float32
    h = f32(D // 2)
    c, s = f32(c), f32(s)
    iy, ix = np.meshgrid(np.arange(D), np.arange(D), indexing="ij")
    ixs = (D - ix) % D if mirror else ix
    x = ixs.astype(f32) - (h + f32(sx))
    y = iy.astype(f32) - (h + f32(sy))
    xo = (x * c - y * s) + h
    yo = (x * s + y * c) + h
    out = (xo < 0) | (xo >= f32(D)) | (yo < 0) | (yo >= f32(D))
    return np.where(out, ixs.astype(f32), xo), np.where(out, iy.astype(f32), yo)


def rot_shift2d(img, ang, sx, sy, mirror) -> np.ndarray:
    """rot_shift2D(img, ang, sx, sy, mirror) with quadratic interpolation,
    background mode (FP64 values, float32 coordinates): rotate by ang degrees
    about (D/2, D/2), shift by (sx, sy), then mirror in x.  cos and sin of the
    angle in FP64, rounded to float32."""
    D = np.asarray(img).shape[0]
    t = np.radians(np.float64(ang))
    xo, yo = rot_shift2d_coords(D, np.cos(t), np.sin(t), sx, sy, int(mirror))
    return quadri(img, xo, yo)


def tanl_fshift(img, fl: float, ff: float, dx: float, dy: float) -> np.ndarray:
    """filt_tanl(img, fl, ff) followed by fshift(img, dx, dy) on one image
    [D][D], both on its real FFT in FP64 (numpy's rfft2 / irfft2): the
    half spectrum times 0.5 (tanh(k (r + fl)) - tanh(k (r - fl))),
    k = pi / (2 ff fl), r = |(kx, ky)| / D in cycles per pixel (ky signed,
    ky > D/2 taken as ky - D),
    no filter when fl <= 0, a step at fl when ff = 0; times
    exp(-2 pi i (kx dx + ky dy) / D), the image moved by (+dx, +dy)."""
    a = np.asarray(img, np.float64)
    D = a.shape[0]
    kx = np.arange(D // 2 + 1, dtype=np.float64)
    ky = np.arange(D, dtype=np.float64)
    ky[ky > D // 2] -= D  # ky = D/2 (even D) counts as +D/2
    h = np.ones((D, D // 2 + 1))
    if fl > 0:
        r = np.sqrt((kx[None, :] / D) ** 2 + (ky[:, None] / D) ** 2)
        if ff > 0:
            k = np.pi / (2.0 * ff * fl)
            h = 0.5 * (np.tanh(k * (r + fl)) - np.tanh(k * (r - fl)))
        else:  # the limit ff -> 0: a step at fl
            h = np.where(r < fl, 1.0, np.where(r == fl, 0.5, 0.0))
    ph = np.exp(-2j * np.pi * (kx[None, :] * dx + ky[:, None] * dy) / D)
    return np.fft.irfft2(np.fft.rfft2(a) * h * ph, s=(D, D))


def class_averages(imgs, peaks, belongsto, fl: float, ff: float, center: bool = True):
    """The averaging step after the group assignment
    (bin/sp_isac2_gpu.py:1153-1234), restated in FP64 for one process:
    each particle i of group r = belongsto[i] takes the alignment parameters
    of its pair (peaks[r][i], converted as the caller does, ormq_post; stored
    as float32 like the caller's peak_list); its image rot_shift2D'd by them
    is added to the group's sum; the group's shift sums (sx subtracted for a
    mirrored particle) are summed in FP64 in particle order, rounded to
    float32 (the MPI_FLOAT reduction) and divided by the member count; every
    particle's parameters become (ang, sx -/+ mean sx, sy - mean sy, mirror);
    each sum times float32(1 / members) is low-passed (filt_tanl(fl, ff)) and
    moved by minus its mean shift (fshift), when center.
    Returns (averages [R][D][D] FP64, params [P][4] FP64 rounded to float32,
    members [R], shifts [R][2])."""
    imgs = np.asarray(imgs, np.float32)
    P, D = imgs.shape[0], imgs.shape[1]
    pk = np.asarray(peaks, np.float32)
    R = pk.shape[0]
    bel = np.asarray(belongsto, np.int64)
    f32 = np.float32
    ang, sxc, syc, mir = ormq_post(pk[bel, np.arange(P)])
    ang = ang.astype(f32)
    sxc, syc = sxc.astype(f32), syc.astype(f32)
    mir = mir.astype(np.int64)
    sums = np.zeros((R, D, D))
    members = np.zeros(R, np.int64)
    ssx, ssy = np.zeros(R), np.zeros(R)
    for i in range(P):
        r = bel[i]
        sums[r] += rot_shift2d(imgs[i], ang[i], sxc[i], syc[i], mir[i])
        members[r] += 1
        ssx[r] += -float(sxc[i]) if mir[i] else float(sxc[i])
        ssy[r] += float(syc[i])
    with np.errstate(divide="ignore", invalid="ignore"):
        mx = np.where(members > 0, ssx.astype(f32).astype(np.float64) / members, 0.0)
        my = np.where(members > 0, ssy.astype(f32).astype(np.float64) / members, 0.0)
    params = np.zeros((P, 4))
    params[:, 0] = ang
    params[:, 1] = np.where(mir == 0, sxc - mx[bel], sxc + mx[bel]).astype(f32)
    params[:, 2] = (syc - my[bel]).astype(f32)
    params[:, 3] = mir
    avg = np.zeros((R, D, D))
    for r in range(R):
        if members[r] == 0:
            continue
        a = sums[r] * np.float64(f32(1.0 / members[r]))
        if fl > 0 or center:
            a = tanl_fshift(a, fl, ff, -mx[r] if center else 0.0, -my[r] if center else 0.0)
        avg[r] = a
    return avg, params, members, np.stack([mx, my], 1)
