"""Learned reference proposal in front of the exhaustive multi-reference search.

The reference aligns every particle against every reference
(cuda/gpu_aln_noref.cu:multi_ref_align, called from
bin/sp_isac2_gpu.py:959-1006).  Here a small network embeds each image's
rotation- and mirror-invariant ring magnitudes; a particle's top-k references
by embedding similarity are searched exhaustively (every shift, angle and
mirror, by the same kernels as the full search), and particles whose result
is not clearly separated fall back to the search over every reference.

Every result the proposal path returns is an entry of the full search: for a
(particle, reference) pair both give the same peak bit for bit, so the
proposal path can only differ from the full search in WHICH reference wins,
and only when the true winner was not proposed and the fallback test passed.

The network is trained on the GPU by the kernels of csrc/nn.cu on labels the
full search produced (each particle's best reference).  torch only allocates
device memory and hands out streams; every arithmetic step is one of the
library's kernels.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import GpuIsacError
from .align import align_proposals_device, make_config

NK = 16            # angular harmonics per ring fed to the network
MODEL_FORMAT = "gpuisac-proposal-net"  # ProposalNet.save / load
MODEL_VERSION = 1
HIDDEN = 256
EMB = 128
SCALE = 16.0       # score = SCALE * cosine similarity of embeddings
FEATURE_CHUNK = 16384


def _call(L, name, *args):
    rc = getattr(L, name)(*args)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"{name} failed ({rc})")


def _stream(dev):
    import torch
    return torch.cuda.current_stream(dev).cuda_stream


def init_params(n_in: int, hidden: int, emb: int, seed: int) -> dict:
    """He-uniform weights, zero biases, from a seeded PCG64 stream."""
    rng = np.random.Generator(np.random.PCG64(seed))
    l1 = np.sqrt(6.0 / n_in)
    l2 = np.sqrt(6.0 / hidden)
    return {"W1": rng.uniform(-l1, l1, (hidden, n_in)).astype(np.float32),
            "b1": np.zeros(hidden, np.float32),
            "W2": rng.uniform(-l2, l2, (emb, hidden)).astype(np.float32),
            "b2": np.zeros(emb, np.float32)}


def ring_features(imgs, ring_num: int, nk: int = NK, mu=None, inv_sd=None, base_shifts=None,
                  chunk: int = FEATURE_CHUNK):
    """[n][ring_num*nk] ring features of a CUDA image stack, centred on each
    image's base shift (zero when None): the ring spectra of that single
    position (gpuisac_spectra_device, subject basis for particles and
    references alike) reduced by gpuisac_nn_features, standardised when mu
    and inv_sd are given."""
    import torch

    imgs = imgs.contiguous().float()
    n, D = imgs.shape[0], imgs.shape[1]
    L = _lib.load()
    feat = torch.empty((n, ring_num * nk), dtype=torch.float32, device=imgs.device)
    st = _stream(imgs.device)
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
    sp = None
    for c0 in range(0, n, chunk):
        c = min(chunk, n - c0)
        cfg = make_config(c, 1, D, ring_num, 256, 1.0, 0.0, 0.0)
        if sp is None or sp.shape[0] < c:
            sp = torch.empty((c, 1, ring_num, 128, 2), dtype=torch.float32, device=imgs.device)
        bp = base_shifts[c0:c0 + c].data_ptr() if base_shifts is not None else None
        _call(L, "gpuisac_spectra_device", ctypes.byref(cfg), imgs[c0:c0 + c].data_ptr(), c, 0, bp,
              sp.data_ptr(), st)
        _call(L, "gpuisac_nn_features", sp.data_ptr(), c, ring_num, nk,
              mu.data_ptr() if mu is not None else None, inv_sd.data_ptr() if inv_sd is not None else None,
              feat[c0:c0 + c].data_ptr(), st)
    return feat


class ProposalNet:
    """Embedding network x -> L2norm(W2 relu(W1 x + b1) + b2) shared by
    particles and references; score(i, j) = scale * e_p[i] . e_r[j].

    Parameters live in one flat device buffer (W1 | b1 | W2 | b2) so that one
    AdamW launch updates them all; gradients and moments mirror it.
    """

    def __init__(self, ring_num: int, nk: int = NK, hidden: int = HIDDEN, emb: int = EMB, scale: float = SCALE,
                 seed: int = 20261203, device=None):
        import torch

        self.ring_num, self.nk, self.hidden, self.emb, self.scale = ring_num, nk, hidden, emb, float(scale)
        self.n_in = ring_num * nk
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.shapes = {"W1": (hidden, self.n_in), "b1": (hidden,), "W2": (emb, hidden), "b2": (emb,)}
        self.offsets, off = {}, 0
        for k, shp in self.shapes.items():
            self.offsets[k] = off
            off += int(np.prod(shp))
        self.n_params = off
        self.flat = torch.empty(off, dtype=torch.float32, device=self.device)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.step_count = 0
        self.load_params(init_params(self.n_in, hidden, emb, seed))
        # feature standardisation (set from training features by set_feature_stats)
        self.mu = torch.zeros(self.n_in, dtype=torch.float32, device=self.device)
        self.inv_sd = torch.ones(self.n_in, dtype=torch.float32, device=self.device)
        self._ws = {}

    # ---------------------------------------------------------------- params
    def view(self, buf, name):
        o = self.offsets[name]
        shp = self.shapes[name]
        return buf[o:o + int(np.prod(shp))].view(shp)

    def load_params(self, params: dict):
        import torch
        for k in self.shapes:
            self.view(self.flat, k).copy_(torch.as_tensor(np.asarray(params[k], np.float32)))

    def params(self) -> dict:
        return {k: self.view(self.flat, k).cpu().numpy().copy() for k in self.shapes}

    # ---------------------------------------------------------------- files
    def save(self, path: str, **meta) -> None:
        """Weights and feature statistics to path + ".npz" (float32), the
        architecture and any caller metadata (gap_margin, k, training notes:
        JSON values) to path + ".json", with a format name and version."""
        import hashlib
        import json

        arrays = dict(self.params(), mu=self.mu.cpu().numpy(), inv_sd=self.inv_sd.cpu().numpy())
        np.savez(path + ".npz", **arrays)
        with open(path + ".npz", "rb") as f:
            digest = hashlib.sha256(f.read()).hexdigest()
        doc = {"format": MODEL_FORMAT, "version": MODEL_VERSION, "ring_num": self.ring_num, "nk": self.nk,
               "hidden": self.hidden, "emb": self.emb, "scale": self.scale, "n_params": self.n_params,
               "weights_sha256": digest, "meta": meta}
        with open(path + ".json", "w") as f:
            json.dump(doc, f, indent=1, sort_keys=True)

    @classmethod
    def load(cls, path: str, device=None):
        """The network save() wrote at path (".json" + ".npz"), on device.
        Returns (net, meta).  Raises ValueError for another format or
        version, weights that do not match their recorded digest, or arrays
        of the wrong shapes."""
        import hashlib
        import json

        with open(path + ".json") as f:
            doc = json.load(f)
        if doc.get("format") != MODEL_FORMAT or doc.get("version") != MODEL_VERSION:
            raise ValueError(f"{path}.json: not a {MODEL_FORMAT} file of version {MODEL_VERSION}")
        with open(path + ".npz", "rb") as f:
            if hashlib.sha256(f.read()).hexdigest() != doc["weights_sha256"]:
                raise ValueError(f"{path}.npz does not match the digest recorded in {path}.json")
        net = cls(doc["ring_num"], nk=doc["nk"], hidden=doc["hidden"], emb=doc["emb"], scale=doc["scale"],
                  device=device)
        with np.load(path + ".npz") as z:
            arrays = {k: z[k] for k in z.files}
        want = dict(net.shapes, mu=(net.n_in,), inv_sd=(net.n_in,))
        for k, shp in want.items():
            if k not in arrays or tuple(arrays[k].shape) != tuple(shp):
                raise ValueError(f"{path}.npz: {k} missing or not of shape {shp}")
        net.load_params(arrays)
        import torch
        net.mu.copy_(torch.as_tensor(arrays["mu"].astype(np.float32)))
        net.inv_sd.copy_(torch.as_tensor(arrays["inv_sd"].astype(np.float32)))
        return net, doc["meta"]

    def grads(self) -> dict:
        return {k: self.view(self.grad, k).cpu().numpy().copy() for k in self.shapes}

    def set_feature_stats(self, X_raw, eps: float = 1e-6):
        """mu / inv_sd from raw (unstandardised) training feature rows"""
        _call(_lib.load(), "gpuisac_nn_col_stats", X_raw.data_ptr(), X_raw.shape[0], self.n_in, eps,
              self.mu.data_ptr(), self.inv_sd.data_ptr(), _stream(self.device))

    def standardise(self, X_raw):
        """standardise feature rows in place"""
        _call(_lib.load(), "gpuisac_nn_affine_cols", X_raw.data_ptr(), X_raw.shape[0], self.n_in,
              self.mu.data_ptr(), self.inv_sd.data_ptr(), _stream(self.device))
        return X_raw

    def features(self, imgs, ring_num: int, base_shifts=None):
        """standardised network inputs of an image stack"""
        return ring_features(imgs, ring_num, self.nk, self.mu, self.inv_sd, base_shifts)

    def c_struct(self):
        from ._lib import GpuisacProposalNet
        v = lambda name: self.view(self.flat, name).data_ptr()
        return GpuisacProposalNet(self.nk, self.hidden, self.emb, self.mu.data_ptr(), self.inv_sd.data_ptr(),
                                  v("W1"), v("b1"), v("W2"), v("b2"))

    # ---------------------------------------------------------------- workspace
    def _buf(self, key, shape, dtype=None):
        import torch
        n = int(np.prod(shape))
        b = self._ws.get(key)
        if b is None or b.numel() < n:
            b = torch.empty(max(n, 1), dtype=dtype or torch.float32, device=self.device)
            self._ws[key] = b
        return b[:n].view(shape)

    # ---------------------------------------------------------------- forward
    def _forward(self, X, tag):
        """H, Z, E, norm of one batch (buffers keyed by tag)"""
        L = _lib.load()
        st = _stream(self.device)
        n = X.shape[0]
        H = self._buf(tag + "H", (n, self.hidden))
        Z = self._buf(tag + "Z", (n, self.emb))
        E = self._buf(tag + "E", (n, self.emb))
        nrm = self._buf(tag + "N", (n,))
        W1, b1 = self.view(self.flat, "W1"), self.view(self.flat, "b1")
        W2, b2 = self.view(self.flat, "W2"), self.view(self.flat, "b2")
        # H = X W1^T: A = X (n x n_in), B(k, j) = W1[j][k]
        _call(L, "gpuisac_nn_gemm", n, self.hidden, self.n_in, 1.0, X.data_ptr(), self.n_in, 1, W1.data_ptr(), 1,
              self.n_in, 0.0, H.data_ptr(), self.hidden, st)
        _call(L, "gpuisac_nn_bias_act", H.data_ptr(), b1.data_ptr(), n, self.hidden, 1, st)
        _call(L, "gpuisac_nn_gemm", n, self.emb, self.hidden, 1.0, H.data_ptr(), self.hidden, 1, W2.data_ptr(), 1,
              self.hidden, 0.0, Z.data_ptr(), self.emb, st)
        _call(L, "gpuisac_nn_bias_act", Z.data_ptr(), b2.data_ptr(), n, self.emb, 0, st)
        _call(L, "gpuisac_nn_l2norm", Z.data_ptr(), n, self.emb, E.data_ptr(), nrm.data_ptr(), st)
        return H, Z, E, nrm

    def embed(self, X, out=None):
        """unit embeddings [n][emb] of feature rows X (copied out of the workspace)"""
        import torch
        out = out if out is not None else torch.empty((X.shape[0], self.emb), dtype=torch.float32,
                                                      device=self.device)
        for c0 in range(0, X.shape[0], FEATURE_CHUNK):
            c1 = min(X.shape[0], c0 + FEATURE_CHUNK)
            _, _, E, _ = self._forward(X[c0:c1], "e")
            out[c0:c1].copy_(E)
        return out

    def scores(self, Ep, Er, out=None):
        """scale * Ep Er^T  [n_p][n_r]"""
        import torch
        L = _lib.load()
        n, r = Ep.shape[0], Er.shape[0]
        out = out if out is not None else torch.empty((n, r), dtype=torch.float32, device=self.device)
        _call(L, "gpuisac_nn_gemm", n, r, self.emb, self.scale, Ep.data_ptr(), self.emb, 1, Er.data_ptr(), 1,
              self.emb, 0.0, out.data_ptr(), r, _stream(self.device))
        return out

    # ---------------------------------------------------------------- training
    def _backward_batch(self, X, H, E, nrm, dE, tag, accumulate):
        """gradients of one batch's embeddings dE into self.grad"""
        L = _lib.load()
        st = _stream(self.device)
        n = X.shape[0]
        acc = 1.0 if accumulate else 0.0
        W2 = self.view(self.flat, "W2")
        gW1, gb1 = self.view(self.grad, "W1"), self.view(self.grad, "b1")
        gW2, gb2 = self.view(self.grad, "W2"), self.view(self.grad, "b2")
        dZ = self._buf(tag + "dZ", (n, self.emb))
        dH = self._buf(tag + "dH", (n, self.hidden))
        _call(L, "gpuisac_nn_l2norm_backward", E.data_ptr(), dE.data_ptr(), nrm.data_ptr(), n, self.emb,
              dZ.data_ptr(), st)
        # gW2 (+)= dZ^T H: A(m, k) = dZ[k][m], B(k, j) = H[k][j]
        _call(L, "gpuisac_nn_gemm", self.emb, self.hidden, n, 1.0, dZ.data_ptr(), 1, self.emb, H.data_ptr(),
              self.hidden, 1, acc, gW2.data_ptr(), self.hidden, st)
        _call(L, "gpuisac_nn_colsum", dZ.data_ptr(), n, self.emb, gb2.data_ptr(), int(accumulate), st)
        # dH = dZ W2: B(k, j) = W2[k][j]
        _call(L, "gpuisac_nn_gemm", n, self.hidden, self.emb, 1.0, dZ.data_ptr(), self.emb, 1, W2.data_ptr(),
              self.hidden, 1, 0.0, dH.data_ptr(), self.hidden, st)
        _call(L, "gpuisac_nn_relu_backward", dH.data_ptr(), H.data_ptr(), n * self.hidden, st)
        # gW1 (+)= dH^T X
        _call(L, "gpuisac_nn_gemm", self.hidden, self.n_in, n, 1.0, dH.data_ptr(), 1, self.hidden, X.data_ptr(),
              self.n_in, 1, acc, gW1.data_ptr(), self.n_in, st)
        _call(L, "gpuisac_nn_colsum", dH.data_ptr(), n, self.hidden, gb1.data_ptr(), int(accumulate), st)

    def loss_and_grad(self, Xp, labels, Xr):
        """mean cross-entropy of one particle batch against every reference;
        leaves the gradient in self.grad and returns the per-particle loss
        (device tensor)."""
        L = _lib.load()
        st = _stream(self.device)
        B, R = Xp.shape[0], Xr.shape[0]
        Hp, _, Ep, np_ = self._forward(Xp, "p")
        Hr, _, Er, nr_ = self._forward(Xr, "r")
        S = self._buf("S", (B, R))
        dS = self._buf("dS", (B, R))
        loss = self._buf("loss", (B,))
        dEp = self._buf("dEp", (B, self.emb))
        dEr = self._buf("dEr", (R, self.emb))
        self.scores(Ep, Er, out=S)
        _call(L, "gpuisac_nn_softmax_xent", S.data_ptr(), labels.data_ptr(), B, R, loss.data_ptr(), dS.data_ptr(),
              st)
        # dEp = scale dS Er;  dEr = scale dS^T Ep
        _call(L, "gpuisac_nn_gemm", B, self.emb, R, self.scale, dS.data_ptr(), R, 1, Er.data_ptr(), self.emb, 1,
              0.0, dEp.data_ptr(), self.emb, st)
        _call(L, "gpuisac_nn_gemm", R, self.emb, B, self.scale, dS.data_ptr(), 1, R, Ep.data_ptr(), self.emb, 1,
              0.0, dEr.data_ptr(), self.emb, st)
        self._backward_batch(Xp, Hp, Ep, np_, dEp, "p", False)
        self._backward_batch(Xr, Hr, Er, nr_, dEr, "r", True)
        return loss

    def adam(self, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8, wd: float = 0.0):
        self.step_count += 1
        _call(_lib.load(), "gpuisac_nn_adam", self.flat.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(),
              self.v.data_ptr(), self.n_params, lr, b1, b2, eps, wd, self.step_count, _stream(self.device))

    def fit(self, Xp, labels, Xr, epochs: int = 8, batch: int = 2048, lr: float = 2e-3, lr_end: float = 1e-4,
            wd: float = 1e-4, seed: int = 7):
        """Adam on mini-batches of consecutive rows; each epoch starts at a
        different seeded offset so batch boundaries move.  Returns the mean
        training loss per epoch (one device->host read per epoch)."""
        import torch

        n = Xp.shape[0]
        if labels.dtype != torch.int32:
            raise ValueError("labels must be int32")
        rng = np.random.Generator(np.random.PCG64(seed))
        nb = max(1, n // batch)
        total = epochs * nb
        hist = []
        acc = self._buf("loss_acc", (1,))
        t = 0
        for ep in range(epochs):
            off = int(rng.integers(0, max(1, n - nb * batch + 1)))
            acc.zero_()
            for b in range(nb):
                s0 = off + b * batch
                loss = self.loss_and_grad(Xp[s0:s0 + batch], labels[s0:s0 + batch], Xr)
                # cosine decay from lr to lr_end
                cur = lr_end + 0.5 * (lr - lr_end) * (1.0 + np.cos(np.pi * t / max(1, total - 1)))
                self.adam(float(cur), wd=wd)
                _call(_lib.load(), "gpuisac_nn_colsum", loss.data_ptr(), loss.shape[0], 1, acc.data_ptr(), 1,
                      _stream(self.device))
                t += 1
            hist.append(float(acc.item()) / (nb * batch))
        return hist

    # ---------------------------------------------------------------- inference
    def propose(self, Xp, Er, k: int, out=None):
        """top-k references per particle (int32 [n][k], best first) from
        feature rows Xp against reference embeddings Er"""
        import torch
        L = _lib.load()
        st = _stream(self.device)
        n, R = Xp.shape[0], Er.shape[0]
        out = out if out is not None else torch.empty((n, k), dtype=torch.int32, device=self.device)
        for c0 in range(0, n, FEATURE_CHUNK):
            c1 = min(n, c0 + FEATURE_CHUNK)
            _, _, E, _ = self._forward(Xp[c0:c1], "e")
            S = self._buf("Sprop", (c1 - c0, R))
            self.scores(E, Er, out=S)
            _call(L, "gpuisac_nn_topk", S.data_ptr(), c1 - c0, R, k, out[c0:c1].data_ptr(), st)
        return out




# ==================================================================== search

def best_of(d: np.ndarray, cand: np.ndarray):
    """Host restatement of the search's choice among candidates: per row the
    candidate with the largest d (ties: the smaller reference index, as the
    full search's first-maximum scan over references picks).  d, cand: [n][k].
    Returns (position in row, reference, peak, runner-up peak)."""
    d = np.asarray(d, np.float64)
    cand = np.asarray(cand, np.int64)
    mx = d.max(1)
    big = np.iinfo(np.int64).max
    best_ref = np.where(d == mx[:, None], cand, big).min(1)
    pos = (cand == best_ref[:, None]).argmax(1)
    rest = d.copy()
    rest[np.arange(d.shape[0]), pos] = -np.inf
    second = rest.max(1) if d.shape[1] > 1 else np.full(d.shape[0], -np.inf)
    return pos, best_ref, mx, second


def calibrate_margin(gaps: np.ndarray, correct: np.ndarray, max_wrong: float = 1e-3) -> float:
    """Smallest gap margin at which at most a fraction max_wrong of the
    calibration particles keep a proposed result that is not the full
    search's (gaps: best minus runner-up proposed peak; correct: the proposed
    best is the full search's best)."""
    gaps = np.asarray(gaps, np.float64)
    wrong = ~np.asarray(correct, bool)
    budget = int(np.floor(max_wrong * len(gaps)))
    wg = np.sort(gaps[wrong])[::-1]
    if len(wg) <= budget:
        return 0.0
    # accept strictly above the (budget+1)-th largest wrong gap
    return float(np.nextafter(wg[budget], np.inf))


@dataclass
class LearnedResult:
    ref: object        # [P] int32 best reference (device tensor)
    peak: object       # [P] float32 its peak correlation
    params: object     # [P][4] angle, sx, sy, mirror (as the full search reports them)
    gap: object        # [P] best minus runner-up proposed peak
    fallback: object   # [P] uint8: 1 where every reference was searched
    pairs: int         # particle x reference alignments run


def reference_embeddings(net: ProposalNet, refs, ring_num: int):
    """unit embeddings [R][emb] of the references (zero shift)"""
    return net.embed(net.features(refs, ring_num))


def learned_align(particles, refs, net: ProposalNet, ring_num: int, shift_rng_x: float, shift_rng_y: float,
                  shift_step: float = 1.0, k: int = 8, gap_margin: float = 0.0, base_shifts=None,
                  ref_embed=None, stream=None) -> LearnedResult:
    """Best reference and alignment of every particle by the learned search
    (gpuisac_learned_align_device); gap_margin = -inf disables the fallback."""
    import torch

    particles = particles.contiguous().float()
    refs = refs.contiguous().float()
    P, D = particles.shape[0], particles.shape[1]
    R = refs.shape[0]
    dev = particles.device
    Er = ref_embed if ref_embed is not None else reference_embeddings(net, refs, ring_num)
    cfg = make_config(P, R, D, ring_num, 256, shift_step, shift_rng_x, shift_rng_y)
    ref_o = torch.empty(P, dtype=torch.int32, device=dev)
    peak = torch.empty(P, dtype=torch.float32, device=dev)
    params = torch.empty((P, 4), dtype=torch.float32, device=dev)
    gap = torch.empty(P, dtype=torch.float32, device=dev)
    fb = torch.empty(P, dtype=torch.int32, device=dev)
    base_ptr = None
    if base_shifts is not None:
        base_shifts = base_shifts.contiguous().float()
        base_ptr = base_shifts.data_ptr()
    pairs = ctypes.c_ulonglong(0)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    L = _lib.load()
    net_c = net.c_struct()
    rc = L.gpuisac_learned_align_device(ctypes.byref(cfg), particles.data_ptr(), refs.data_ptr(), base_ptr,
                                        ctypes.byref(net_c), Er.data_ptr(), k, float(gap_margin), ref_o.data_ptr(),
                                        peak.data_ptr(), params.data_ptr(), gap.data_ptr(), fb.data_ptr(),
                                        ctypes.byref(pairs), st.cuda_stream)
    if rc:
        _lib.check(L)
        raise GpuIsacError(f"gpuisac_learned_align_device failed ({rc})")
    return LearnedResult(ref_o, peak, params, gap, fb, int(pairs.value))


@dataclass
class TrainReport:
    loss: list           # mean training loss per epoch
    gap_margin: float    # calibrated fallback margin
    recall: float        # calibration particles whose full-search best was proposed and won
    fallback_rate: float  # calibration particles below the margin


def train_from_full_search(net: ProposalNet, particles, refs, d_full, peak_full, ring_num: int,
                           shift_rng_x: float, shift_rng_y: float, shift_step: float = 1.0, k: int = 8,
                           calib_frac: float = 0.1, max_wrong: float = 1e-3, epochs: int = 15, batch: int = 500,
                           lr: float = 2e-3, wd: float = 1e-2, seed: int = 7) -> TrainReport:
    """Train the network on the full search's own results for `particles`
    (d_full [R][P], peak_full [R][P][4] from multi_ref_align_device): label =
    the best reference, input = the particle's ring features centred on that
    reference's best shift.  The last calib_frac of the particles stay out of
    training and calibrate the fallback margin."""
    import torch

    dev = particles.device
    P = particles.shape[0]
    d_h = d_full.cpu().numpy() if hasattr(d_full, "cpu") else np.asarray(d_full)
    labels = d_h.argmax(0).astype(np.int32)
    pk = peak_full.reshape(d_h.shape[0], P, 4)
    lab_t = torch.as_tensor(labels, device=dev)
    best_shift = pk[lab_t.long(), torch.arange(P, device=dev), 1:3].contiguous()
    n_fit = max(1, int(round(P * (1.0 - calib_frac))))
    X = ring_features(particles, ring_num, net.nk, base_shifts=best_shift)
    net.set_feature_stats(X[:n_fit])
    net.standardise(X)
    Xr = net.features(refs, ring_num)
    hist = net.fit(X[:n_fit], lab_t[:n_fit], Xr, epochs=epochs, batch=batch, lr=lr, wd=wd, seed=seed)
    if n_fit >= P:
        return TrainReport(hist, 0.0, float("nan"), 0.0)
    cal = particles[n_fit:]
    res = learned_align(cal, refs, net, ring_num, shift_rng_x, shift_rng_y, shift_step, k=k,
                        gap_margin=-float("inf"), ref_embed=reference_embeddings(net, refs, ring_num))
    correct = res.ref.cpu().numpy() == labels[n_fit:]
    gaps = res.gap.cpu().numpy()
    margin = calibrate_margin(gaps, correct, max_wrong)
    return TrainReport(hist, margin, float(correct.mean()), float((gaps < margin).mean()))
