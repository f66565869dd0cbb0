"""The CCF autotuner: it times every tile shape on the caller's stacks,
records the fastest, and the recorded choice changes no result (every
candidate runs the same arithmetic in the same order)."""
import numpy as np
import pytest

from gpuisac import synth
from gpuisac.align import (autotune_ccf, ccf_tile_name, multi_ref_align_device, multi_ref_align_groups_device)

pytestmark = pytest.mark.gpu


def test_autotune_records_a_choice_and_keeps_results(gpulib, cuda):
    import torch
    st = synth.make_stack(300, 64, 12, 2, 0.1, 28.0, seed=61)
    parts, refs = torch.from_numpy(st.particles).to(cuda), torch.from_numpy(st.refs).to(cuda)
    d0, p0 = multi_ref_align_device(parts, refs, 29, 2.0, 2.0)
    groups = [(0, 120, 0, 5), (100, 150, 4, 8), (250, 50, 0, 12)]
    g0 = multi_ref_align_groups_device(parts, refs, groups, 29, 2.0, 2.0)
    rep = autotune_ccf(parts, refs, 29, 2.0, 2.0, n_sample=128)
    entries = [e for e in rep.split("; ") if not e.startswith("chosen")]
    assert len(entries) == 9 and all(e.endswith(" ms") for e in entries), rep
    chosen = rep.split("chosen ")[1]
    assert ccf_tile_name(29, 25) == chosen
    d1, p1 = multi_ref_align_device(parts, refs, 29, 2.0, 2.0)
    assert np.array_equal(d0.cpu().numpy(), d1.cpu().numpy())
    assert np.array_equal(p0.cpu().numpy(), p1.cpu().numpy())
    g1 = multi_ref_align_groups_device(parts, refs, groups, 29, 2.0, 2.0)
    assert np.array_equal(g0[0].cpu().numpy(), g1[0].cpu().numpy())
    assert np.array_equal(g0[1].cpu().numpy(), g1[1].cpu().numpy())


def test_tile_name_default_and_wide_rings(gpulib):
    # up to 64 rings the warp-specialised kernel (2 shifts per group beyond
    # 36 rings); beyond, the general kernel
    assert ccf_tile_name(61, 81).startswith("ws")
    assert ccf_tile_name(88, 81).startswith("general/")
