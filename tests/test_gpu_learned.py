"""Learned reference proposal on the GPU: the network kernels against the FP64
CPU oracle (forward, gradients, AdamW, top-k, GEMM strides, features), the
proposal search against the full search (bit-exact entries), and what the
trained network gains over the search without it."""
import numpy as np
import pytest

import nn_oracle as nno
from gpuisac import learned, synth
from gpuisac.align import align_proposals_device, multi_ref_align_device, spectra_device

pytestmark = pytest.mark.gpu


def _t(a, cuda, dtype=None):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype or torch.float32, device=cuda)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (65, 130, 17), (128, 64, 300), (7, 200, 64)])
@pytest.mark.parametrize("trans_a,trans_b", [(False, False), (True, False), (False, True), (True, True)])
def test_gemm_strides(gpulib, cuda, M, N, K, trans_a, trans_b):
    import ctypes
    rng = np.random.Generator(np.random.PCG64(M * 1000 + N + K))
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    As = A.T.copy() if trans_a else A          # stored [K][M] when transposed
    Bs = B.T.copy() if trans_b else B          # stored [N][K] when transposed
    sam, sak = (1, M) if trans_a else (K, 1)
    sbk, sbn = (1, K) if trans_b else (N, 1)
    dA, dB, dC = _t(As, cuda), _t(Bs, cuda), _t(C0, cuda)
    import torch
    rc = gpulib.gpuisac_nn_gemm(M, N, K, ctypes.c_float(0.5), dA.data_ptr(), sam, sak, dB.data_ptr(), sbk, sbn,
                                ctypes.c_float(2.0), dC.data_ptr(), N, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    want = 0.5 * A.astype(np.float64) @ B.astype(np.float64) + 2.0 * C0
    assert _rel(dC.cpu().numpy(), want) < 1e-5


def _net(cuda, ring_num=5, nk=60, hidden=64, emb=32, seed=4):
    net = learned.ProposalNet(ring_num, nk=nk, hidden=hidden, emb=emb, scale=7.0, seed=seed, device=cuda)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    p = net.params()
    p["b1"] = 0.05 * rng.standard_normal(p["b1"].shape).astype(np.float32)
    p["b2"] = 0.05 * rng.standard_normal(p["b2"].shape).astype(np.float32)
    net.load_params(p)
    return net, p


def test_forward_and_gradients_match_oracle(gpulib, cuda):
    import torch
    net, p = _net(cuda)
    rng = np.random.Generator(np.random.PCG64(12))
    B, R = 96, 37
    Xp = np.abs(rng.standard_normal((B, net.n_in))).astype(np.float32)
    Xr = np.abs(rng.standard_normal((R, net.n_in))).astype(np.float32)
    labels = rng.integers(0, R, B).astype(np.int32)
    loss = net.loss_and_grad(_t(Xp, cuda), _t(labels, cuda, torch.int32), _t(Xr, cuda))
    torch.cuda.synchronize()
    want_loss, want_g, aux = nno.loss_and_grads(p, Xp, Xr, labels, net.scale)
    assert abs(loss.cpu().numpy().mean() - want_loss) < 1e-5 * max(1.0, abs(want_loss))
    g = net.grads()
    for k in ("W1", "b1", "W2", "b2"):
        assert _rel(g[k], want_g[k]) < 1e-4, k
    # embeddings and scores
    Ep = net.embed(_t(Xp, cuda))
    Er = net.embed(_t(Xr, cuda))
    S = net.scores(Ep, Er).cpu().numpy()
    assert _rel(S, aux["S"]) < 1e-5


def test_adam_matches_oracle(gpulib, cuda):
    net, p = _net(cuda)
    rng = np.random.Generator(np.random.PCG64(2))
    g = rng.standard_normal(net.n_params).astype(np.float32)
    net.grad.copy_(_t(g, cuda))
    p0 = net.flat.cpu().numpy().astype(np.float64)
    m, v = np.zeros(net.n_params), np.zeros(net.n_params)
    want = p0
    for step in (1, 2, 3):
        net.adam(1e-3, wd=1e-2)
        want, m, v = nno.adam_step(want, g, m, v, step, lr=1e-3, wd=1e-2)
    assert _rel(net.flat.cpu().numpy() - p0, want - p0) < 1e-4


@pytest.mark.parametrize("R,k", [(500, 8), (1024, 64), (3, 3), (33, 1)])
def test_topk_matches_oracle(gpulib, cuda, R, k):
    import torch
    rng = np.random.Generator(np.random.PCG64(R + k))
    S = rng.permutation(257 * R)[: 40 * R].reshape(40, R).astype(np.float32) / 7.0
    S[3, :] = 1.0                                  # all tied: 0..k-1
    S[5, ::2] = 2.0                                # ties among even columns
    idx = torch.empty((40, k), dtype=torch.int32, device=cuda)
    rc = gpulib.gpuisac_nn_topk(_t(S, cuda).data_ptr(), 40, R, k, idx.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    assert np.array_equal(idx.cpu().numpy(), nno.topk(S, k))


def test_topk_rejects_out_of_range(gpulib, cuda):
    assert gpulib.gpuisac_nn_topk(1, 1, 1025, 8, 1, None) == 2
    assert gpulib.gpuisac_nn_topk(1, 1, 100, 65, 1, None) == 2


def test_features_match_oracle(gpulib, cuda):
    st = synth.make_stack(30, 64, 5, 2, 0.1, 28.0, seed=77)
    parts = _t(st.particles, cuda)
    sp = spectra_device(parts, 29, 0.0, 0.0)                 # [n][1][29][128][2]
    f = learned.ring_features(parts, 29, 64)
    want = nno.features(sp[:, 0].cpu().numpy(), 64)
    assert _rel(f.cpu().numpy(), want) < 1e-5


@pytest.mark.parametrize("base", [False, True])
def test_proposal_search_entries_equal_full_search(gpulib, cuda, base):
    """Every (particle, reference) entry of the proposal search is the full
    search's entry, bit for bit, whichever particles are selected and in
    whatever order the references are listed."""
    import torch
    P, R, D, NR, rng_s = 44, 13, 64, 29, 2.0
    st = synth.make_stack(P, D, R, 2, 0.1, 28.0, seed=91)
    parts, refs = _t(st.particles, cuda), _t(st.refs, cuda)
    bs = None
    if base:
        g = np.random.Generator(np.random.PCG64(5))
        bs = _t(np.round((g.uniform(-1.5, 1.5, (P, 2))) * 64) / 64, cuda)
    d_full, pk_full = multi_ref_align_device(parts, refs, NR, rng_s, rng_s, base_shifts=bs)
    g = np.random.Generator(np.random.PCG64(6))
    sel = g.choice(P, 29, replace=False).astype(np.int32)
    sel[-1] = sel[0]                                    # a particle may appear twice
    prop = np.stack([g.choice(R, 5, replace=False) for _ in sel]).astype(np.int32)
    d, pk = align_proposals_device(parts, refs, _t(prop, cuda, torch.int32), NR, rng_s, rng_s,
                                   part_idx=_t(sel, cuda, torch.int32), base_shifts=bs)
    d_full, pk_full = d_full.cpu().numpy(), pk_full.cpu().numpy()
    want_d = d_full[prop, sel[:, None]]
    want_pk = pk_full[prop, sel[:, None]]
    assert np.array_equal(d.cpu().numpy(), want_d)
    assert np.array_equal(pk.cpu().numpy(), want_pk)
    # no particle list: every particle in order
    allp = np.stack([g.choice(R, 3, replace=False) for _ in range(P)]).astype(np.int32)
    d2, _ = align_proposals_device(parts, refs, _t(allp, cuda, torch.int32), NR, rng_s, rng_s, base_shifts=bs)
    assert np.array_equal(d2.cpu().numpy(), d_full[allp, np.arange(P)[:, None]])


def test_proposal_search_rejects_bad_indices(gpulib, cuda):
    import torch
    st = synth.make_stack(6, 32, 4, 1, 0.1, 14.0, seed=3)
    parts, refs = _t(st.particles, cuda), _t(st.refs, cuda)
    bad = _t(np.array([[0, 4]], np.int32), cuda, torch.int32)
    with pytest.raises(Exception):
        align_proposals_device(parts, refs, bad, 13, 1.0, 1.0, part_idx=_t(np.array([1], np.int32), cuda,
                                                                            torch.int32))
    ok = _t(np.array([[0, 3]], np.int32), cuda, torch.int32)
    with pytest.raises(Exception):
        align_proposals_device(parts, refs, ok, 13, 1.0, 1.0, part_idx=_t(np.array([6], np.int32), cuda,
                                                                           torch.int32))


def _full(parts, refs, NR, s, base=None):
    d, pk = multi_ref_align_device(parts, refs, NR, s, s, base_shifts=base)
    return d, pk


@pytest.mark.parametrize("base", [False, True])
def test_learned_search_limits_equal_full_search(gpulib, cuda, base):
    """With every particle sent to the fallback (margin +inf), or with every
    reference proposed (k = R), the learned search returns the full search's
    best entry for every particle, bit for bit; with the fallback off it runs
    exactly P x k alignments and each result is the full search's entry for
    the reference it names."""
    import torch
    P, R, D, NR, s = 70, 12, 64, 29, 2.0
    st = synth.make_stack(P, D, R, 2, 0.1, 28.0, seed=17)
    parts, refs = _t(st.particles, cuda), _t(st.refs, cuda)
    bs = None
    if base:
        g = np.random.Generator(np.random.PCG64(8))
        bs = _t(np.round(g.uniform(-1.5, 1.5, (P, 2)) * 64) / 64, cuda)
    d, pk = _full(parts, refs, NR, s, bs)
    d, pk = d.cpu().numpy(), pk.cpu().numpy()
    best = d.argmax(0)
    idx = np.arange(P)
    net = learned.ProposalNet(NR, device=cuda, seed=3)          # untrained: arbitrary proposals
    for k, margin in ((4, float("inf")), (R, 0.0)):
        res = learned.learned_align(parts, refs, net, NR, s, s, k=k, gap_margin=margin, base_shifts=bs)
        assert np.array_equal(res.ref.cpu().numpy(), best)
        assert np.array_equal(res.peak.cpu().numpy(), d[best, idx])
        assert np.array_equal(res.params.cpu().numpy(), pk[best, idx])
    assert res.pairs == P * R
    res = learned.learned_align(parts, refs, net, NR, s, s, k=3, gap_margin=-float("inf"), base_shifts=bs)
    assert res.pairs == P * 3 and not res.fallback.cpu().numpy().any()
    r = res.ref.cpu().numpy()
    assert np.array_equal(res.peak.cpu().numpy(), d[r, idx])
    assert np.array_equal(res.params.cpu().numpy(), pk[r, idx])


def test_trained_network_gain(gpulib, cuda):
    """Trained on the full search's own results, the network proposes the
    full search's best reference among its top 8 far more often than the same
    network untrained, and the learned search then reproduces the full
    search's assignment on >= 99.5% of held-out particles while running a
    fraction of its particle x reference alignments."""
    R, D, NR, s = 64, 64, 29, 2.0
    train = synth.make_stack(8000, D, R, 2, 0.1, 28.0, seed=404, particle_seed=405)
    held = synth.make_stack(2000, D, R, 2, 0.1, 28.0, seed=404, particle_seed=406)
    refs = _t(train.refs, cuda)
    tp, hp = _t(train.particles, cuda), _t(held.particles, cuda)
    d_tr, pk_tr = _full(tp, refs, NR, s)
    d_he, pk_he = _full(hp, refs, NR, s)
    d_he, pk_he = d_he.cpu().numpy(), pk_he.cpu().numpy()
    lab = d_he.argmax(0)
    P = hp.shape[0]

    def recall(net):
        res = learned.learned_align(hp, refs, net, NR, s, s, k=8, gap_margin=-float("inf"))
        return (res.ref.cpu().numpy() == lab).mean()

    untrained = learned.ProposalNet(NR, device=cuda, seed=11)
    net = learned.ProposalNet(NR, device=cuda, seed=11)
    rep = learned.train_from_full_search(net, tp, refs, d_tr, pk_tr, NR, s, s, k=8, calib_frac=0.2)
    untrained.mu.copy_(net.mu)
    untrained.inv_sd.copy_(net.inv_sd)
    before, after = recall(untrained), recall(net)
    assert rep.loss[-1] < 0.5 * rep.loss[0]
    assert after >= 0.97 and after > before + 0.2, (before, after)

    res = learned.learned_align(hp, refs, net, NR, s, s, k=8, gap_margin=rep.gap_margin)
    r = res.ref.cpu().numpy()
    same = r == lab
    assert same.mean() >= 0.995, (same.mean(), rep)
    idx = np.arange(P)
    assert np.array_equal(res.peak.cpu().numpy(), d_he[r, idx])
    assert np.array_equal(res.params.cpu().numpy(), pk_he[r, idx])
    assert res.pairs <= 0.5 * P * R, (res.pairs, rep)
