"""Uneven groups aligned in one pass (gpuisac_multi_ref_align_groups_device):
every group's results must equal a separate alignment of that group, and a
repeated call (replayed CUDA graph) must give the same results."""
import numpy as np
import pytest

from gpuisac import synth

pytestmark = pytest.mark.gpu


def run_groups(cuda, st, groups, NR, rng, base=None):
    import torch

    from gpuisac.align import multi_ref_align_groups_device
    parts = torch.from_numpy(st.particles).to(cuda)
    refs = torch.from_numpy(st.refs).to(cuda)
    bt = None if base is None else torch.from_numpy(base).to(cuda)
    d, pk, offs = multi_ref_align_groups_device(parts, refs, groups, NR, rng, rng, base_shifts=bt)
    return d.cpu().numpy(), pk.cpu().numpy(), offs


def per_group(cuda, st, g, NR, rng, base=None):
    import torch

    from gpuisac import multi_ref_align_device
    so, sn, ro, rn = g
    parts = torch.from_numpy(np.ascontiguousarray(st.particles[so:so + sn])).to(cuda)
    refs = torch.from_numpy(np.ascontiguousarray(st.refs[ro:ro + rn])).to(cuda)
    bt = None if base is None else torch.from_numpy(np.ascontiguousarray(base[so:so + sn])).to(cuda)
    d, pk = multi_ref_align_device(parts, refs, NR, rng, rng, base_shifts=bt)
    return d.cpu().numpy(), pk.cpu().numpy()


@pytest.mark.parametrize("D,NR,rng", [(64, 29, 2.0), (96, 45, 1.0)])
def test_groups_equal_separate_runs(gpulib, cuda, D, NR, rng):
    st = synth.make_stack(260, D, 30, int(rng), 0.1, D * 0.4, 91)
    base = np.random.default_rng(2).uniform(-1.0, 1.0, (260, 2)).astype(np.float32)
    groups = [(0, 1, 0, 1), (1, 13, 1, 3), (14, 40, 4, 7), (54, 100, 11, 10), (154, 5, 21, 4), (159, 64, 25, 5),
              (223, 37, 0, 30)]
    d, pk, offs = run_groups(cuda, st, groups, NR, rng, base)
    for (so, sn, ro, rn), off in zip(groups, offs):
        dg, pg = per_group(cuda, st, (so, sn, ro, rn), NR, rng, base)
        assert np.array_equal(d[off:off + rn * sn].reshape(rn, sn), dg)
        assert np.array_equal(pk[off:off + rn * sn].reshape(rn, sn, 4), pg)
    # the identical call again replays the recorded graph
    d2, pk2, _ = run_groups(cuda, st, groups, NR, rng, base)
    assert np.array_equal(d, d2) and np.array_equal(pk, pk2)


def test_groups_match_oracle(gpulib, cuda, oracle_mod):
    st = synth.make_stack(30, 64, 6, 2, 0.1, 28.0, 92)
    groups = [(0, 12, 0, 3), (12, 18, 3, 3)]
    d, pk, offs = run_groups(cuda, st, groups, 29, 2.0)
    tex = gpulib.get_texture_limit(64)
    for (so, sn, ro, rn), off in zip(groups, offs):
        cfg = oracle_mod.make_cfg(sn, rn, 64, 29, 256, 1.0, 2.0, 2.0)
        lay = oracle_mod.reference_layout(cfg)
        lay = oracle_mod.OrcLayout(lay.sbj_batch, tex, lay.ref_batch)
        po, do = oracle_mod.multi_ref_align(cfg, lay, st.particles[so:so + sn], st.refs[ro:ro + rn])
        rel = np.abs(d[off:off + rn * sn].reshape(rn, sn) - do) / np.abs(do)
        assert rel.max() <= 1e-4
        assert (pk[off:off + rn * sn].reshape(rn, sn, 4)[..., 1:] == po[..., 1:]).mean() >= 0.99
