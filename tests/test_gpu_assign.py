"""The equal-size group assignment on the GPU (gpuisac_assign_groups_device,
gpuisac_assign_groups) against the oracle's restatement of EMAN2's
Util::assign_groups (bin/sp_isac2_gpu.py:1114-1136): the returned list is
identical (integer work: bit-exact), belongsto agrees with it, at small and
ragged sizes, with equal peaks, signed zeros and infinities, on a strided d,
on a real alignment's peak matrix, and -- at 100,000 particles x 500 groups,
where the oracle's sort takes tens of seconds -- through the properties that
define the result (group sizes, joining order, no blocking pair)."""
import ctypes

import numpy as np
import pytest

from gpuisac import GpuIsacError, synth
from gpuisac.align import multi_ref_align_device
from gpuisac.assign import assign_groups, assign_groups_device

pytestmark = pytest.mark.gpu


def synth_peaks(nref, nima, seed, kind="classes"):
    rng = np.random.default_rng(seed)
    if kind == "classes":           # each particle near one class and its neighbour
        cls = rng.integers(0, nref, nima)
        d = rng.normal(size=(nref, nima)).astype(np.float32) * 0.05 + 0.5
        d[cls, np.arange(nima)] += 0.3 * rng.random(nima).astype(np.float32)
        d[(cls + 1) % nref, np.arange(nima)] += 0.15 * rng.random(nima).astype(np.float32)
        return d
    d = rng.normal(size=(nref, nima)).astype(np.float32)
    if kind == "ties":
        d = np.round(d * 2) / 2
    elif kind == "signed":
        d = np.where(rng.random(d.shape) < 0.2, np.float32(-0.0), d)
        d[0, 0] = np.inf
        d[-1, -1] = -np.inf
    elif kind == "dominant":        # every particle ranks group 0 first, then 1, ...
        d = rng.random((nref, nima), dtype=np.float32) + np.linspace(3, 0, nref, dtype=np.float32)[:, None]
    return d


def groups_of(ids, nref, nima):
    maxasi = nima // nref
    bel = np.full(nima, -1, np.int64)
    for g in range(nref):
        bel[ids[g * maxasi:(g + 1) * maxasi]] = g
    bel[ids[nref * maxasi:nima]] = ids[-1]
    return bel


def run_device(d_np, cuda):
    import torch
    d = torch.from_numpy(d_np).to(cuda)
    ids, bel, rounds = assign_groups_device(d)
    return ids.cpu().numpy(), bel.cpu().numpy(), rounds


@pytest.mark.parametrize("nref,nima", [(1, 1), (1, 9), (3, 3), (2, 5), (4, 13), (5, 7), (7, 50), (16, 333),
                                       (64, 64), (200, 4099), (333, 20000)])
@pytest.mark.parametrize("kind", ["classes", "ties", "signed", "dominant"])
def test_list_equals_oracle(oracle_mod, gpulib, cuda, nref, nima, kind):
    d = synth_peaks(nref, nima, nref * 7 + nima, kind)
    want = oracle_mod.assign_groups(d, nref, nima)
    ids, bel, rounds = run_device(d, cuda)
    assert rounds >= 1
    np.testing.assert_array_equal(ids, want)
    np.testing.assert_array_equal(bel, groups_of(want, nref, nima))


def test_host_entry_point_and_address_string(oracle_mod, gpulib, cuda):
    d = synth_peaks(50, 1234, 3)
    want = oracle_mod.assign_groups(d, 50, 1234).tolist()
    assert assign_groups(d, 50, 1234) == want
    flat = np.ascontiguousarray(d.reshape(-1))
    # the reference passes str(d.__array_interface__['data'][0])
    assert assign_groups(str(flat.__array_interface__["data"][0]), 50, 1234) == want
    import torch
    assert assign_groups(torch.from_numpy(flat).to(cuda), 50, 1234) == want


def test_strided_rows(oracle_mod, gpulib, cuda):
    import torch
    d = synth_peaks(40, 3000, 5)
    wide = torch.zeros((40, 3000 + 37), dtype=torch.float32, device=cuda)
    wide[:, :3000] = torch.from_numpy(d).to(cuda)
    ids, bel, _ = assign_groups_device(wide[:, :3000])
    np.testing.assert_array_equal(ids.cpu().numpy(), oracle_mod.assign_groups(d, 40, 3000))


def test_on_an_alignment_peak_matrix(oracle_mod, gpulib, cuda):
    import torch
    st = synth.make_stack(600, 64, 12, 8, 0.2, 28.0, 99)
    d, _ = multi_ref_align_device(torch.from_numpy(st.particles).to(cuda), torch.from_numpy(st.refs).to(cuda),
                                  29, 2.0, 2.0)
    ids, bel, _ = assign_groups_device(d)
    want = oracle_mod.assign_groups(d.cpu().numpy(), 12, 600)
    np.testing.assert_array_equal(ids.cpu().numpy(), want)
    np.testing.assert_array_equal(bel.cpu().numpy(), oracle_mod.belongsto_from_id_list(want, 12, 600))


def test_headline_size_equals_oracle(oracle_mod, gpulib, cuda):
    d = synth_peaks(200, 50000, 11)
    ids, _, rounds = run_device(d, cuda)
    np.testing.assert_array_equal(ids, oracle_mod.assign_groups(d, 200, 50000))


@pytest.mark.parametrize("kind", ["classes", "dominant"])
def test_full_size_properties(gpulib, cuda, kind):
    """100,000 x 500: sizes, joining order and no blocking pair, checked on
    the GPU with pair ranks from a stable sort of (-peak)."""
    import torch
    nref, nima = 500, 100000
    maxasi, extra = nima // nref, nima % nref
    d = torch.from_numpy(synth_peaks(nref, nima, 21, kind)).to(cuda)
    ids, bel, rounds = assign_groups_device(d)
    ids = ids.long()
    assert torch.equal(torch.sort(ids[:nima]).values, torch.arange(nima, device=cuda))
    flat = d.reshape(-1).double() + 0.0
    order = torch.sort(-flat, stable=True).indices
    rank = torch.empty_like(order)
    rank[order] = torch.arange(flat.numel(), device=cuda)
    rank = rank.reshape(nref, nima)
    core = ids[:nref * maxasi].reshape(nref, maxasi)
    core_rank = torch.gather(rank, 1, core)
    assert (core_rank[:, 1:] > core_rank[:, :-1]).all()          # joining order
    worst = core_rank[:, -1]
    last = int(ids[-1])
    assert int(worst.argmax()) == last                          # the last group closes last
    own = torch.full((nima,), 2 ** 62, dtype=torch.long, device=cuda)
    own[core.reshape(-1)] = core_rank.reshape(-1)
    assert not ((rank < own[None, :]) & (rank < worst[:, None])).any()
    assert int(ids[nref * maxasi:nima].numel()) == extra
    expect = torch.empty(nima, dtype=torch.long, device=cuda)
    expect[core.reshape(-1)] = torch.arange(nref, device=cuda).repeat_interleave(maxasi)
    assert torch.equal(bel.long(), expect)


def test_argument_errors_are_reported(gpulib, cuda, oracle_mod):
    import torch
    from gpuisac import _lib
    with pytest.raises(GpuIsacError):
        assign_groups(np.zeros((3, 2), np.float32), 3, 2)            # nima < nref
    d = torch.zeros((2, 4), dtype=torch.float32, device=cuda)
    d[1, 2] = float("nan")
    gpulib.gpuisac_clear_error()
    with pytest.raises(GpuIsacError):
        assign_groups_device(d)
    gpulib.gpuisac_clear_error()
    rc = gpulib.gpuisac_assign_groups_device(d.data_ptr(), 0, 2, 4, None, None, None, None)
    assert rc == 2
    gpulib.gpuisac_clear_error()
    # the workspace recovers for the next call
    good = synth_peaks(2, 4, 1)
    ids, _, _ = run_device(good, cuda)
    np.testing.assert_array_equal(ids, oracle_mod.assign_groups(good, 2, 4))
    assert _lib.last_error(gpulib)[0] == 0
