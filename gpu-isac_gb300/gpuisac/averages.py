"""The averaging step of ISAC's main iteration on the GPU.

After the multi-reference alignment and the group assignment, ISAC
(bin/sp_isac2_gpu.py:1153-1234) converts each particle's peak parameters
(:1015-1022), rot_shift2D's every particle by those of its group's pair and
adds it to the group's sum, re-centres the particles' parameters by their
group's mean shift, and turns each sum into the next reference: divided by the
member count, low-passed with filt_tanl and moved by minus the mean shift with
fshift.  `class_averages_device` runs all of it in one call of
gpuisac_class_averages on device tensors; `class_averages` takes and returns
host arrays.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import GpuIsacError


def class_averages_device(particles, peaks, belongsto, fl: float, ff: float, center: bool = True, stream=None):
    """particles: CUDA float32 [P][D][D]; peaks: CUDA float32 [R][P][4] (or
    [R][pitch][4] rows of a wider array) as multi_ref_align_device returns
    them; belongsto: CUDA int32 [P].  fl, ff: filt_tanl's cut-off and fall-off
    (fl <= 0: no filter).  Returns (averages [R][D][D], params [P][4] = (angle,
    sx, sy, mirror) re-centred, members int32 [R], shifts [R][2] the groups'
    mean shifts), all CUDA tensors.  Raises GpuIsacError for a belongsto entry
    outside [0, R) or a group without members (its average is zero)."""
    import torch

    if not (particles.is_cuda and particles.dtype == torch.float32 and particles.dim() == 3
            and particles.is_contiguous()):
        raise GpuIsacError("class_averages_device needs a contiguous float32 CUDA stack [P][D][D]")
    P, D = particles.shape[0], particles.shape[1]
    if particles.shape[2] != D:
        raise GpuIsacError("images must be square")
    if not (peaks.is_cuda and peaks.dtype == torch.float32 and peaks.dim() == 3 and peaks.shape[1] >= P
            and peaks.shape[2] == 4 and peaks.stride(2) == 1 and peaks.stride(1) == 4):
        raise GpuIsacError("peaks must be a float32 CUDA tensor [R][>= P][4] with packed rows")
    bel = belongsto.to(device=particles.device, dtype=torch.int32).contiguous()
    if bel.numel() != P:
        raise GpuIsacError("belongsto must hold one group per particle")
    R = peaks.shape[0]
    dev = particles.device
    avg = torch.empty((R, D, D), dtype=torch.float32, device=dev)
    params = torch.empty((P, 4), dtype=torch.float32, device=dev)
    members = torch.empty(R, dtype=torch.int32, device=dev)
    shifts = torch.empty((R, 2), dtype=torch.float32, device=dev)
    L = _lib.load()
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    rc = L.gpuisac_class_averages(particles.data_ptr(), P, D, peaks.data_ptr(), peaks.stride(0) // 4,
                                  bel.data_ptr(), R, float(fl), float(ff), int(bool(center)), avg.data_ptr(),
                                  params.data_ptr(), members.data_ptr(), shifts.data_ptr(), st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_class_averages failed ({rc})")
    return avg, params, members, shifts


def class_averages(particles, peaks, belongsto, fl: float, ff: float, center: bool = True):
    """The same on host arrays: particles [P][D][D], peaks [R][P][4] (the
    multi_ref_align peak list), belongsto [P].  Returns numpy arrays."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    parts = torch.from_numpy(np.ascontiguousarray(particles, np.float32)).to(dev)
    pk = np.ascontiguousarray(peaks, np.float32)
    pk = torch.from_numpy(pk.reshape(pk.shape[0], parts.shape[0], 4)).to(dev)
    bel = torch.from_numpy(np.ascontiguousarray(belongsto, np.int32)).to(dev)
    out = class_averages_device(parts, pk, bel, fl, ff, center)
    return tuple(t.cpu().numpy() for t in out)
