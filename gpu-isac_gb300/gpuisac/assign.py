"""Equal-size group assignment on the alignment's peak matrix, on the GPU.

ISAC assigns particles to groups right after the multi-reference alignment
(bin/sp_isac2_gpu.py:1114-1136) with EMAN2's Util::assign_groups on the host.
`assign_groups(d, numref, nima)` takes the same arguments (d as a numpy array,
a torch tensor, or the host address the reference passes as a string) and
returns the same list of nima + 1 ints; `assign_groups_device` keeps d and the
result on the GPU and also returns belongsto.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GpuIsacError


def _fail(L, name, rc):
    _lib.check(L)
    raise GpuIsacError(f"{name} failed ({rc})")


def assign_groups(d, numref: int, nima: int) -> list:
    """Util.assign_groups(d, numref, nima): d[ref * nima + particle] peaks.
    Returns id_list_long (each group's nima // numref members, best pair
    first, group after group; the nima % numref leftovers of the group that
    closed last; that group's index)."""
    L = _lib.load()
    if hasattr(d, "is_cuda") and d.is_cuda:
        ids, _, _ = assign_groups_device(d.reshape(numref, nima), with_belongsto=False)
        return ids.cpu().tolist()
    if isinstance(d, (str, int)):
        ptr, keep = int(d), None
    else:
        keep = np.ascontiguousarray(np.asarray(d, np.float32).reshape(-1))
        if keep.size != numref * nima:
            raise GpuIsacError("d must hold numref * nima peaks")
        ptr = keep.ctypes.data
    out = np.zeros(nima + 1, np.int32)
    rc = L.gpuisac_assign_groups(ptr, numref, nima, out.ctypes.data)
    if rc:
        _fail(L, "gpuisac_assign_groups", rc)
    return out.tolist()


def assign_groups_device(d, with_belongsto: bool = True, with_id_list: bool = True, stream=None):
    """d: CUDA tensor [numref][nima] (or [numref][pitch] rows with nima
    columns viewed from a wider array).  Returns (id_list_long int32 tensor or
    None, belongsto int32 tensor or None, rounds)."""
    import torch

    if not d.is_cuda or d.dim() != 2 or d.dtype != torch.float32 or d.stride(1) != 1:
        raise GpuIsacError("assign_groups_device needs a float32 CUDA tensor [numref][nima] with unit column stride")
    numref, nima = d.shape
    ids = torch.empty(nima + 1, dtype=torch.int32, device=d.device) if with_id_list else None
    bel = torch.empty(nima, dtype=torch.int32, device=d.device) if with_belongsto else None
    rounds = ctypes.c_uint()
    st = stream if stream is not None else torch.cuda.current_stream(d.device)
    L = _lib.load()
    rc = L.gpuisac_assign_groups_device(d.data_ptr(), d.stride(0), numref, nima,
                                        bel.data_ptr() if bel is not None else None,
                                        ids.data_ptr() if ids is not None else None, ctypes.byref(rounds),
                                        st.cuda_stream)
    if rc:
        _fail(L, "gpuisac_assign_groups_device", rc)
    return ids, bel, rounds.value
