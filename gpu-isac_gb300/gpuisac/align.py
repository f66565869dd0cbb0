"""Python host side of the multi-reference alignment, mirroring the calls
bin/sp_isac2_gpu.py:937-1032 makes (init, fill base shifts, align, clear),
on numpy arrays or torch tensors instead of EMData lists.
"""
from __future__ import annotations

import contextlib
import ctypes

import numpy as np

from . import _lib
from ._lib import AlignConfig, GpuIsacError, float_ptr


def make_config(sbj_num, ref_num, img_dim, ring_num, ring_len=256, shift_step=1.0, shift_rng_x=1.0,
                shift_rng_y=1.0, aln_type=b"mref_aln") -> AlignConfig:
    return AlignConfig(sbj_num, ref_num, img_dim, ring_num, ring_len, shift_step, shift_rng_x, shift_rng_y,
                       aln_type)


# arithmetic of the ring-summed contraction (gpuisac_set_contraction)
CONTRACTIONS = {"fp32": 0, "bf16x3": 1}


@contextlib.contextmanager
def contraction(mode: str | None):
    """Run the enclosed calls with the contraction in `mode`: "fp32" (FP32 on
    the CUDA cores, the drop-in default) or "bf16x3" (BF16 hi/lo split on the
    tensor cores); None leaves the current mode."""
    if mode is None:
        yield
        return
    if mode not in CONTRACTIONS:
        raise ValueError(f"unknown contraction {mode!r} (one of {sorted(CONTRACTIONS)})")
    L = _lib.load()
    prev = L.gpuisac_set_contraction(CONTRACTIONS[mode])
    if prev < 0:
        _lib.check(L)
    try:
        yield
    finally:
        L.gpuisac_set_contraction(prev)


SPLIT_PLAN_FIELDS = ("n_blocks", "block", "zw", "kg", "rga", "rblock", "n_rtiles", "n_cols", "n_stages",
                     "fft_groups")


def split_plan(ring_num: int, n_shift: int, n_ref: int) -> dict:
    """The tensor-core contraction's tile plan for a shape (gpuisac_split_plan)."""
    L = _lib.load()
    f = (ctypes.c_uint * len(SPLIT_PLAN_FIELDS))()
    if L.gpuisac_split_plan(ring_num, n_shift, n_ref, f, len(SPLIT_PLAN_FIELDS)):
        _lib.check(L)
    return dict(zip(SPLIT_PLAN_FIELDS, list(f)))


def ptr_array(stack: np.ndarray):
    """float** over the images of a C-contiguous float32 [n][D][D] stack (the
    reference's get_c_ptr_array, bin/sp_isac2_gpu.py:166-174)."""
    assert stack.flags["C_CONTIGUOUS"] and stack.dtype == np.float32
    n = stack.shape[0]
    step = stack.strides[0]
    base = stack.ctypes.data
    arr = (float_ptr * max(n, 1))()
    for i in range(n):
        arr[i] = ctypes.cast(base + i * step, float_ptr)
    return arr


def multi_ref_align(particles: np.ndarray, refs: np.ndarray, ring_num: int, shift_rng_x: float,
                    shift_rng_y: float, shift_step: float = 1.0, base_shifts: np.ndarray | None = None,
                    ring_len: int = 256, device: int = 0, mem_request: float = 0.9, d_pitch: int | None = None,
                    contraction_mode: str | None = None):
    """Align every particle against every reference through the C-ABI.

    Returns (peak_list, d): peak_list [ref][4*sbj] float32 laid out as the
    reference's caller expects (angle, sx, sy, mirror per particle), d
    [ref][sbj] float32 peak correlations.  contraction_mode: "fp32" or
    "bf16x3" for this call (None: the library's current mode).
    """
    with contraction(contraction_mode):
        return _multi_ref_align(particles, refs, ring_num, shift_rng_x, shift_rng_y, shift_step, base_shifts,
                                ring_len, device, mem_request, d_pitch)


def _multi_ref_align(particles, refs, ring_num, shift_rng_x, shift_rng_y, shift_step, base_shifts, ring_len,
                     device, mem_request, d_pitch):
    L = _lib.load()
    particles = np.ascontiguousarray(particles, np.float32)
    refs = np.ascontiguousarray(refs, np.float32)
    P, D = particles.shape[0], particles.shape[1]
    R = refs.shape[0]
    if particles.shape[1:] != (D, D) or refs.shape[1:] != (D, D):
        raise ValueError("particles and refs must be [n][D][D] with the same D")
    cfg = make_config(P, R, D, ring_num, ring_len, shift_step, shift_rng_x, shift_rng_y)
    pitch = d_pitch or P
    peak_list = np.zeros((R, 4 * P), np.float32)
    d = np.zeros((R, pitch), np.float32)
    params = L.multi_ref_align_init(ctypes.byref(cfg), device)
    if not params:
        _lib.check(L)
        raise GpuIsacError("multi_ref_align_init returned NULL")
    try:
        if base_shifts is not None:
            bs = np.asarray(base_shifts, np.float32).reshape(P, 2)
            for i in range(P):
                params[i].shift_x = float(bs[i, 0])
                params[i].shift_y = float(bs[i, 1])
        sp, rp = ptr_array(particles), ptr_array(refs)
        L.multi_ref_align(sp, rp, peak_list.ctypes.data_as(float_ptr), d.ctypes.data_as(float_ptr), pitch,
                          mem_request)
        _lib.check(L)
    finally:
        L.gpu_clear()
    return peak_list, d[:, :P]


def multi_ref_align_device(particles, refs, ring_num: int, shift_rng_x: float, shift_rng_y: float,
                           shift_step: float = 1.0, base_shifts=None, stream=None, d_out=None, peak_out=None,
                           contraction_mode: str | None = None, ring_len: int = 256):
    """Device-resident form on torch CUDA tensors: returns (d [R][P], peak [R][P][4]).
    contraction_mode: "fp32" or "bf16x3" for this call (None: the current mode);
    ring_len: 256 or 512 samples per ring (512 computes in FP32 whatever the mode)."""
    with contraction(contraction_mode):
        return _multi_ref_align_device(particles, refs, ring_num, shift_rng_x, shift_rng_y, shift_step,
                                       base_shifts, stream, d_out, peak_out, ring_len)


def _multi_ref_align_device(particles, refs, ring_num, shift_rng_x, shift_rng_y, shift_step, base_shifts, stream,
                            d_out, peak_out, ring_len=256):
    import torch

    if not (particles.is_cuda and refs.is_cuda):
        raise GpuIsacError("multi_ref_align_device needs CUDA tensors")
    particles = particles.contiguous().float()
    refs = refs.contiguous().float()
    P, D = particles.shape[0], particles.shape[1]
    R = refs.shape[0]
    cfg = make_config(P, R, D, ring_num, ring_len, shift_step, shift_rng_x, shift_rng_y)
    if d_out is None:
        d_out = torch.empty((R, P), dtype=torch.float32, device=particles.device)
    if peak_out is None:
        peak_out = torch.empty((R, P, 4), dtype=torch.float32, device=particles.device)
    base_ptr = None
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
        base_ptr = base_shifts.data_ptr()
    st = stream if stream is not None else torch.cuda.current_stream(particles.device)
    L = _lib.load()
    rc = L.gpuisac_multi_ref_align_device(ctypes.byref(cfg), particles.data_ptr(), refs.data_ptr(), base_ptr,
                                          d_out.data_ptr(), peak_out.data_ptr(), st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_multi_ref_align_device failed ({rc})")
    return d_out, peak_out


def spectra_device(imgs, ring_num: int, shift_rng_x: float, shift_rng_y: float, shift_step: float = 1.0,
                   is_ref: bool = False, base_shifts=None, sbj_num: int | None = None):
    """Ring spectra of a device image stack as the CCF kernel consumes them:
    [n][n_shift][ring][128][2] float32 (n_shift = 1 for references)."""
    import torch

    imgs = imgs.contiguous().float()
    n, D = imgs.shape[0], imgs.shape[1]
    cfg = make_config(sbj_num or n, n if is_ref else 1, D, ring_num, 256, shift_step, shift_rng_x, shift_rng_y)
    L = _lib.load()
    S = 1 if is_ref else L.gpuisac_shift_count(ctypes.byref(cfg))
    out = torch.empty((n, S, ring_num, 128, 2), dtype=torch.float32, device=imgs.device)
    base_ptr = None
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
        base_ptr = base_shifts.data_ptr()
    st = torch.cuda.current_stream(imgs.device)
    rc = L.gpuisac_spectra_device(ctypes.byref(cfg), imgs.data_ptr(), n, int(is_ref), base_ptr, out.data_ptr(),
                                  st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_spectra_device failed ({rc})")
    return out


def peak_tuples(peak_list: np.ndarray) -> np.ndarray:
    """[ref][4*sbj] -> [ref][sbj][4]"""
    R = peak_list.shape[0]
    return peak_list.reshape(R, -1, 4)


def multi_ref_align_groups_device(particles, refs, groups, ring_num: int, shift_rng_x: float, shift_rng_y: float,
                                  shift_step: float = 1.0, base_shifts=None, stream=None):
    """Many independent groups in one pass (gpuisac_multi_ref_align_groups_device).

    particles, refs: CUDA tensors [n][D][D]; groups: list of
    (sbj_offset, sbj_num, ref_offset, ref_num).  Returns (d, peak, offsets):
    flat result tensors and each group's element offset; group i's results are
    d[off:off+R*P].view(R, P) and peak[off:off+R*P].view(R, P, 4).
    """
    import torch

    from ._lib import GpuisacGroup

    particles = particles.contiguous().float()
    refs = refs.contiguous().float()
    P, D = particles.shape[0], particles.shape[1]
    R = refs.shape[0]
    cfg = make_config(P, R, D, ring_num, 256, shift_step, shift_rng_x, shift_rng_y)
    tbl = (GpuisacGroup * max(len(groups), 1))()
    offsets, off = [], 0
    for i, (so, sn, ro, rn) in enumerate(groups):
        tbl[i] = GpuisacGroup(so, sn, ro, rn, off)
        offsets.append(off)
        off += sn * rn
    d = torch.empty(max(off, 1), dtype=torch.float32, device=particles.device)
    pk = torch.empty((max(off, 1), 4), dtype=torch.float32, device=particles.device)
    base_ptr = None
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
        base_ptr = base_shifts.data_ptr()
    st = stream if stream is not None else torch.cuda.current_stream(particles.device)
    L = _lib.load()
    rc = L.gpuisac_multi_ref_align_groups_device(ctypes.byref(cfg), tbl, len(groups), particles.data_ptr(),
                                                 refs.data_ptr(), base_ptr, d.data_ptr(), pk.data_ptr(),
                                                 st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_multi_ref_align_groups_device failed ({rc})")
    return d, pk, offsets


def groups_stats() -> dict:
    """What the last multi_ref_align_groups_device call did
    (gpuisac_groups_stats): host plan time, graph recording time (0 when a
    recorded graph was replayed), waves, launches in the graph."""
    from ._lib import GpuisacGroupStats
    L = _lib.load()
    s = GpuisacGroupStats()
    if L.gpuisac_groups_stats(ctypes.byref(s)):
        _lib.check(L)
    return {"plan_ms": s.plan_ms, "record_ms": s.record_ms, "waves": s.waves,
            "graph_launches": s.graph_launches, "graph_recorded": bool(s.graphs_recorded)}


def align_proposals_device(particles, refs, proposals, ring_num: int, shift_rng_x: float, shift_rng_y: float,
                           shift_step: float = 1.0, part_idx=None, base_shifts=None, stream=None):
    """Search selected particles against their own reference lists
    (gpuisac_align_proposals_device).

    particles, refs: CUDA tensors [n][D][D] (the whole stacks); proposals:
    int32 CUDA tensor [n_sel][k] of reference indices; part_idx: int32 CUDA
    tensor [n_sel] of particle indices (None: every particle, in order).
    Returns (d [n_sel][k], peak [n_sel][k][4]); entry (i, j) equals the full
    alignment's entry for (reference proposals[i][j], particle part_idx[i]).
    """
    import torch

    particles = particles.contiguous().float()
    refs = refs.contiguous().float()
    proposals = proposals.contiguous()
    if proposals.dtype != torch.int32 or proposals.dim() != 2:
        raise ValueError("proposals must be an int32 [n_sel][k] tensor")
    P, D = particles.shape[0], particles.shape[1]
    R = refs.shape[0]
    n_sel, k = proposals.shape
    idx_ptr = None
    if part_idx is not None:
        part_idx = part_idx.contiguous()
        if part_idx.dtype != torch.int32 or part_idx.numel() != n_sel:
            raise ValueError("part_idx must be an int32 tensor with one entry per proposal row")
        idx_ptr = part_idx.data_ptr()
    cfg = make_config(P, R, D, ring_num, 256, shift_step, shift_rng_x, shift_rng_y)
    d = torch.empty((n_sel, k), dtype=torch.float32, device=particles.device)
    pk = torch.empty((n_sel, k, 4), dtype=torch.float32, device=particles.device)
    base_ptr = None
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
        base_ptr = base_shifts.data_ptr()
    st = stream if stream is not None else torch.cuda.current_stream(particles.device)
    L = _lib.load()
    rc = L.gpuisac_align_proposals_device(ctypes.byref(cfg), particles.data_ptr(), refs.data_ptr(), base_ptr,
                                          idx_ptr, n_sel, proposals.data_ptr(), k, d.data_ptr(), pk.data_ptr(),
                                          st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_align_proposals_device failed ({rc})")
    return d, pk


def autotune_ccf(particles, refs, ring_num: int, shift_rng_x: float, shift_rng_y: float, shift_step: float = 1.0,
                 n_sample: int = 2048, stream=None) -> str:
    """Time the CCF launch's tile shapes on a sample of these stacks and keep
    the fastest for this ring count and shift count (gpuisac_autotune_ccf).
    Returns the tuner's report line."""
    import torch

    particles = particles.contiguous().float()
    refs = refs.contiguous().float()
    P, D = particles.shape[0], particles.shape[1]
    cfg = make_config(P, refs.shape[0], D, ring_num, 256, shift_step, shift_rng_x, shift_rng_y)
    buf = ctypes.create_string_buffer(2048)
    st = stream if stream is not None else torch.cuda.current_stream(particles.device)
    L = _lib.load()
    rc = L.gpuisac_autotune_ccf(ctypes.byref(cfg), particles.data_ptr(), refs.data_ptr(), n_sample, buf, len(buf),
                                st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_autotune_ccf failed ({rc})")
    return buf.value.decode()


def ccf_tile_name(ring_num: int, n_shift: int) -> str:
    """The tile shape CCF launches of this ring count and shift count use."""
    buf = ctypes.create_string_buffer(64)
    _lib.load().gpuisac_ccf_tile_name(ring_num, n_shift, buf, len(buf))
    return buf.value.decode()
