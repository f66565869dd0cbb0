"""One ISAC main iteration on the GPU (gpuisac.isac.main_iteration): the
same results as its steps called one by one (normalisation, alignment with
base shifts, group assignment, averaging), bit for bit; and the true class
phantoms are a fixed point: two iterations from them, on noisy particles of
those classes, give references that still match them (the alignment, the
conversion of its parameters, the base shifts of the next alignment and the
centring of the averages agree with one another)."""
import numpy as np
import pytest

from gpuisac import synth

pytestmark = pytest.mark.gpu


def test_main_iteration_equals_its_steps_and_keeps_true_classes(gpulib, cuda):
    import torch

    from gpuisac import multi_ref_align_device
    from gpuisac.assign import assign_groups_device
    from gpuisac.averages import class_averages_device
    from gpuisac.isac import base_shifts_of, main_iteration
    from gpuisac.ormq import normalize_mask
    P, R, D, NR = 900, 6, 64, 25
    st = synth.make_stack(P, D, R, 2, 0.3, 24.0, 91)
    mask = torch.from_numpy(synth._mask(D, 24).astype(np.float32)).to(cuda)
    refs0 = torch.from_numpy(st.refs.copy()).to(cuda)
    params0 = np.zeros((P, 4), np.float32)
    params0[:, 1:3] = np.random.default_rng(3).uniform(-1, 1, (P, 2))
    # the steps one by one
    parts_a, refs_a = torch.from_numpy(st.particles.copy()).to(cuda), refs0.clone()
    normalize_mask(refs_a, mask, True)
    normalize_mask(parts_a, mask, False)
    base = torch.from_numpy(base_shifts_of(params0)).to(cuda)
    d, pk = multi_ref_align_device(parts_a, refs_a, NR, 2.0, 2.0, 1.0, base_shifts=base)
    ids, bel, _ = assign_groups_device(d)
    avg, prm, mem, sh = class_averages_device(parts_a, pk, bel, 0.2, 0.2, True)
    # the same through main_iteration
    parts_b, refs_b = torch.from_numpy(st.particles.copy()).to(cuda), refs0.clone()
    it = main_iteration(parts_b, refs_b, mask, NR, 2.0, 2.0, 1.0, 0.2, 0.2, params=params0)
    for x, y in [(avg, it.refs), (prm, it.params), (bel, it.belongsto), (ids, it.id_list_long), (d, it.d),
                 (pk, it.peak), (mem, it.members), (sh, it.shifts)]:
        assert torch.equal(x, y)
    # a second iteration from the new references and parameters
    it2 = main_iteration(parts_b, it.refs.clone(), mask, NR, 2.0, 2.0, 1.0, 0.3, 0.2, params=it.params)
    m = synth._mask(D, 24)
    new = it2.refs.cpu().numpy()
    corr = [np.corrcoef(new[r][m], st.refs[r][m])[0, 1] for r in range(R)]
    print("correlation of each reference with its class after two iterations:", np.round(corr, 4))
    assert min(corr) > 0.97
    assert int(it2.members.sum()) == P
    # most particles stay in their true class (the groups are equal-sized, the classes not)
    assert (it2.belongsto.cpu().numpy() == st.cls).mean() > 0.9
