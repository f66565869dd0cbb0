"""The ormq-shaped entry point and the masked normalisation on the GPU,
against the FP64 oracle (the same bar as the alignment tests)."""
import numpy as np
import pytest

from gpuisac import synth

from test_gpu_align import ANGLE_TOL, PEAK_RTOL, circ_diff, oracle_run
from test_ormq_host import numrinit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D,no_sigma", [(76, False), (76, True), (33, False)])
def test_normalize_mask_matches_oracle(gpulib, cuda, D, no_sigma):
    import torch

    import oracle
    from gpuisac.ormq import normalize_mask
    rng = np.random.default_rng(D)
    x = rng.normal(1.5, 3.0, (40, D, D)).astype(np.float32)
    yy, xx = np.mgrid[:D, :D]
    mask = ((xx - D // 2) ** 2 + (yy - D // 2) ** 2 <= (0.45 * D) ** 2).astype(np.float32)
    t = torch.from_numpy(x).to(cuda)
    normalize_mask(t, mask, no_sigma)
    got = t.cpu().numpy().astype(np.float64)
    want = oracle.normalize_mask(x, mask, no_sigma)
    assert np.abs(got - want).max() <= 2e-6 * max(1.0, np.abs(want).max())


def test_normalize_mask_empty_mask_and_stream_order(gpulib, cuda):
    import torch

    from gpuisac.ormq import normalize_mask
    x = torch.full((3, 16, 16), 4.0, device=cuda)
    normalize_mask(x, np.zeros((16, 16), np.float32), False)  # no masked pixel: nothing to take off
    assert torch.equal(x, torch.full_like(x, 4.0))


@pytest.mark.parametrize("device,centre_off", [(False, 0.0), (True, 0.0), (False, 0.75)])
def test_ormq_matches_oracle(gpulib, cuda, oracle_mod, device, centre_off):
    import torch

    import oracle
    from gpuisac.ormq import ormq
    P, R, D, NR, rng = 30, 8, 64, 29, 2.0
    st = synth.make_stack(P, D, R, 2, 0.1, 26.0, 515)
    cnx = cny = D // 2 + 1 + centre_off
    imgs = torch.from_numpy(st.particles).to(cuda) if device else st.particles
    refs = torch.from_numpy(st.refs).to(cuda) if device else st.refs
    ang, sxs, sys_, mir, peak = ormq(imgs, refs, [rng, rng], [rng, rng], 1.0, "F", numrinit(1, NR), cnx, cny)
    assert ang.shape == (R, P)
    base = np.full((P, 2), centre_off, np.float32)
    pk_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, NR, rng, base=base, tex=gpulib.get_texture_limit(D))
    pk_o = np.asarray(pk_o, np.float64).copy()
    pk_o[..., 1:3] -= centre_off  # ormq's shift: the search shift alone
    a_o, sx_o, sy_o, m_o = oracle.ormq_post(pk_o)
    rel = np.abs(peak - d_o) / np.maximum(np.abs(d_o), 1e-30)
    assert rel.max() <= PEAK_RTOL
    same = (mir == m_o) & (circ_diff(ang, a_o) < ANGLE_TOL) & (np.abs(sxs - sx_o) < 0.01) & (np.abs(sys_ - sy_o) < 0.01)
    assert same.mean() >= 0.99
    # one reference: arrays per image
    a1, *_ = ormq(imgs, refs[3], [rng, rng], [rng, rng], 1.0, "F", numrinit(1, NR), cnx, cny)
    assert a1.shape == (P,)
