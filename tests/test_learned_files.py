"""Saving and loading the learned proposal network (ProposalNet.save / load):
weights and feature statistics in an .npz, the architecture, a format name,
a version and the weights' digest in a .json beside it.  CPU only: the
network's tensors live on the host here."""
import json

import numpy as np
import pytest


def _net():
    import torch

    from gpuisac import learned
    net = learned.ProposalNet(7, nk=4, hidden=16, emb=8, seed=5, device="cpu")
    g = torch.Generator().manual_seed(1)
    net.mu.copy_(torch.randn(net.n_in, generator=g))
    net.inv_sd.copy_(torch.rand(net.n_in, generator=g) + 0.5)
    return net


def test_round_trip(tmp_path):
    from gpuisac import learned
    net = _net()
    path = str(tmp_path / "proposal")
    net.save(path, gap_margin=0.25, k=16, note="test")
    back, meta = learned.ProposalNet.load(path, device="cpu")
    assert meta == {"gap_margin": 0.25, "k": 16, "note": "test"}
    assert (back.ring_num, back.nk, back.hidden, back.emb, back.scale) == (7, 4, 16, 8, net.scale)
    for k, v in net.params().items():
        assert np.array_equal(back.params()[k], v)
    assert np.array_equal(back.mu.numpy(), net.mu.numpy())
    assert np.array_equal(back.inv_sd.numpy(), net.inv_sd.numpy())


def test_refuses_other_versions_and_damaged_weights(tmp_path):
    from gpuisac import learned
    path = str(tmp_path / "proposal")
    _net().save(path)
    doc = json.load(open(path + ".json"))
    json.dump(dict(doc, version=doc["version"] + 1), open(path + ".json", "w"))
    with pytest.raises(ValueError, match="version"):
        learned.ProposalNet.load(path, device="cpu")
    json.dump(doc, open(path + ".json", "w"))
    raw = bytearray(open(path + ".npz", "rb").read())
    raw[-40] ^= 0xFF
    open(path + ".npz", "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="digest"):
        learned.ProposalNet.load(path, device="cpu")
