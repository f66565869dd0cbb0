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


def _separate_equal(cuda, st, groups, NR, rng, d, pk, offs, base=None):
    for (so, sn, ro, rn), off in zip(groups, offs):
        dg, pg = per_group(cuda, st, (so, sn, ro, rn), NR, rng, base)
        if not (np.array_equal(d[off:off + rn * sn].reshape(rn, sn), dg) and
                np.array_equal(pk[off:off + rn * sn].reshape(rn, sn, 4), pg)):
            return False
    return True


def test_new_groups_replay_without_recording(gpulib, cuda, monkeypatch):
    """Several waves of particles (a small wave set through GPUISAC_GROUP_WAVE):
    a call with different groups but the same number of waves replays the
    recorded launch graph, 1 + 2 x waves launches, and every group still
    equals its own separate run."""
    from gpuisac.align import groups_stats
    monkeypatch.setenv("GPUISAC_GROUP_WAVE", "60")
    st = synth.make_stack(300, 64, 40, 2, 0.1, 26.0, 93)
    base = np.random.default_rng(5).uniform(-1.0, 1.0, (300, 2)).astype(np.float32)
    ga = [(0, 70, 0, 5), (70, 3, 5, 1), (73, 90, 6, 12), (163, 47, 18, 9), (210, 90, 27, 13)]
    gb = [(5, 33, 2, 7), (38, 120, 9, 4), (158, 1, 39, 1), (159, 99, 13, 20), (258, 42, 0, 40), (10, 5, 3, 3)]
    assert sum(g[1] for g in ga) == 300 and sum(g[1] for g in gb) == 300  # 5 waves of 60 each
    n0 = gpulib.gpuisac_launch_count()
    d, pk, offs = run_groups(cuda, st, ga, 29, 2.0, base)
    s1 = groups_stats()
    assert s1["waves"] == 5 and s1["graph_launches"] == 11
    assert gpulib.gpuisac_launch_count() - n0 == 11
    assert _separate_equal(cuda, st, ga, 29, 2.0, d, pk, offs, base)
    n0 = gpulib.gpuisac_launch_count()
    d, pk, offs = run_groups(cuda, st, gb, 29, 2.0, base)
    s2 = groups_stats()
    assert s2["waves"] == 5 and not s2["graph_recorded"] and s2["record_ms"] == 0.0
    assert gpulib.gpuisac_launch_count() - n0 == 11
    assert _separate_equal(cuda, st, gb, 29, 2.0, d, pk, offs, base)


def test_groups_emulated_sampling(gpulib, cuda, monkeypatch):
    """Without textures (GPUISAC_TEXTURE=0) the spectra jobs sample with the
    emulation and no fill is launched; every group equals its own separate
    run sampled the same way."""
    from gpuisac.align import groups_stats
    monkeypatch.setenv("GPUISAC_TEXTURE", "0")
    st = synth.make_stack(120, 64, 10, 2, 0.1, 26.0, 94)
    groups = [(0, 50, 0, 4), (50, 70, 4, 6), (20, 33, 1, 9)]
    d, pk, offs = run_groups(cuda, st, groups, 29, 2.0)
    assert groups_stats()["graph_launches"] == 2
    assert _separate_equal(cuda, st, groups, 29, 2.0, d, pk, offs)
