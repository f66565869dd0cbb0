"""One ISAC main iteration on the GPU, in the order of bin/sp_isac2_gpu.py:
the masked normalisation of the references and the particles (:925-931), the
multi-reference alignment with every particle's base shift taken from its
current parameters (:956-1008), the equal-size group assignment on the peak
matrix (:1119-1136) and the averaging step that makes the next references
and parameters (:1153-1234) -- each on device tensors through this library's
kernels, the peak matrix and the groups never leaving the GPU.  The
"experimental centring" after the averages (:1236-1289, a CPU alignment of
the references in sp_applications, outside the reference tree) is left to
the caller, as are the MPI reductions (one process per GPU).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .align import multi_ref_align_device
from .assign import assign_groups_device
from .averages import class_averages_device
from .ormq import normalize_mask


def base_shifts_of(params) -> np.ndarray:
    """Each particle's base shift for the next alignment from its parameters
    (alpha, sx, sy, mirror): the inverse of the caller's conversion of the
    peak (bin/sp_isac2_gpu.py:1015-1022, sx = -x c - y s, sy = x s - y c with
    c, s = cos, sin alpha), x = -c sx + s sy, y = -s sx - c sy -- what
    inverse_transform2(alpha, sx, sy) gives the caller at :979-983 (mirror
    not passed).  FP64, returned as float32 [P][2]."""
    p = np.asarray(params, np.float64).reshape(-1, 4)
    a = np.radians(p[:, 0])
    c, s = np.cos(a), np.sin(a)
    return np.stack([-c * p[:, 1] + s * p[:, 2], -s * p[:, 1] - c * p[:, 2]], 1).astype(np.float32)


@dataclass
class IsacIteration:
    refs: object          # [R][D][D] the next references (before the experimental centring)
    params: object        # [P][4] (alpha, sx, sy, mirror): what the caller stores with set_params2D
    belongsto: object     # [P] int32 group of each particle
    id_list_long: object  # [P + 1] int32, Util::assign_groups' list
    d: object             # [R][P] peak correlations
    peak: object          # [R][P][4] the alignment's peak parameters (base shift included)
    members: object       # [R] int32
    shifts: object        # [R][2] the groups' mean shifts


def main_iteration(particles, refs, mask, ring_num: int, xrng: float, yrng: float, step: float, fl: float,
                   ff: float, params=None, contraction_mode: str | None = None, stream=None) -> IsacIteration:
    """particles [P][D][D], refs [R][D][D], mask [D][D]: contiguous float32
    CUDA tensors; particles and refs are normalised in place as the caller
    does (references without the division by sigma).  params: the particles'
    current (alpha, sx, sy, mirror) [P][4] (host or device), None for zero
    base shifts.  xrng, yrng, step: the search range around each base shift;
    fl, ff: filt_tanl's cut-off and fall-off for the new references."""
    import torch

    normalize_mask(refs, mask, no_sigma=True, stream=stream)
    normalize_mask(particles, mask, no_sigma=False, stream=stream)
    base = None
    if params is not None:
        prm = params.cpu().numpy() if hasattr(params, "cpu") else params
        base = torch.from_numpy(base_shifts_of(prm)).to(particles.device)
    d, peak = multi_ref_align_device(particles, refs, ring_num, xrng, yrng, step, base_shifts=base, stream=stream,
                                     contraction_mode=contraction_mode)
    ids, bel, _ = assign_groups_device(d, stream=stream)
    avg, prm_new, members, shifts = class_averages_device(particles, peak, bel, fl, ff, center=True, stream=stream)
    return IsacIteration(avg, prm_new, bel, ids, d, peak, members, shifts)
