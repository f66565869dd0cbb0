"""512 samples per ring (ring512.cu) against the FP64 oracle, which takes the
ring length from the configuration as the reference's library does
(cuda/gpu_aln_noref.cu: every ring sampled at cfg->ring_len angles; Numrinit,
bin/sp_isac_alignment.py:713-747, gives 512 for a last ring of 41..81).
Edge shapes: an odd ring count (a ring pair with one ring), a single shift
(one busy peak-search warp), fewer shifts than a CCF block, base shifts."""
import numpy as np
import pytest

from gpuisac import synth

from test_gpu_align import compare

pytestmark = pytest.mark.gpu


def oracle_512(oracle_mod, parts, refs, NR, rng, tex, base=None):
    import oracle
    P, D = parts.shape[0], parts.shape[1]
    cfg = oracle.make_cfg(P, refs.shape[0], D, NR, 512, 1.0, rng, rng)
    lay = oracle.reference_layout(cfg)
    lay = oracle.OrcLayout(lay.sbj_batch, tex, lay.ref_batch)
    peak, d = oracle_mod.multi_ref_align(cfg, lay, parts, refs, base_shifts=base, precision="f64")
    return np.asarray(peak), np.asarray(d, np.float64).reshape(refs.shape[0], P)


@pytest.mark.parametrize("D,NR,rng", [(64, 29, 2.0), (64, 7, 0.0), (96, 45, 1.0), (72, 40, 3.0)])
def test_l512_matches_oracle(gpulib, cuda, oracle_mod, D, NR, rng):
    from gpuisac import multi_ref_align
    st = synth.make_stack(40, D, 6, int(rng), 0.1, D * 0.4, 501 + NR)
    base = np.random.default_rng(NR).uniform(-1.5, 1.5, (40, 2)).astype(np.float32)
    pl, d = multi_ref_align(st.particles, st.refs, NR, rng, rng, base_shifts=base, ring_len=512)
    peak_o, d_o = oracle_512(oracle_mod, st.particles, st.refs, NR, rng, gpulib.get_texture_limit(D), base)
    rel, best, pairs = compare(pl.reshape(6, 40, 4), d, peak_o, d_o, ring_num=NR, ring_len=512)
    print(f"D={D} NR={NR} shifts +-{rng}: rel {rel:.2e}, best {best:.3f}, tuples {pairs:.3f}")


def test_l512_device_entry_equals_host_entry(gpulib, cuda):
    import torch

    from gpuisac import multi_ref_align
    from gpuisac.align import multi_ref_align_device
    st = synth.make_stack(70, 64, 5, 2, 0.1, 26.0, 512)
    pl, d = multi_ref_align(st.particles, st.refs, 29, 2.0, 2.0, ring_len=512)
    dd, pk = multi_ref_align_device(torch.from_numpy(st.particles).to(cuda), torch.from_numpy(st.refs).to(cuda),
                                    29, 2.0, 2.0, ring_len=512)
    assert np.array_equal(d, dd.cpu().numpy())
    assert np.array_equal(pl.reshape(5, 70, 4), pk.cpu().numpy())


def _turned(img, ang, D):
    """img turned by ang degrees about the sampling centre D/2 (bilinear, FP64;
    the direction the search reports as +ang)"""
    t = np.deg2rad(ang)
    c, s = np.cos(t), np.sin(t)
    yy, xx = np.meshgrid(np.arange(D, dtype=float), np.arange(D, dtype=float), indexing="ij")
    x0, y0 = xx - D // 2, yy - D // 2
    xs, ys = c * x0 + s * y0 + D // 2, -s * x0 + c * y0 + D // 2
    img = img.astype(np.float64)
    ix, iy = np.floor(xs).astype(int), np.floor(ys).astype(int)
    fx, fy = xs - ix, ys - iy

    def at(a, b):
        ok = (a >= 0) & (a < D) & (b >= 0) & (b < D)
        return np.where(ok, img[np.clip(b, 0, D - 1), np.clip(a, 0, D - 1)], 0.0)
    return (at(ix, iy) * (1 - fx) * (1 - fy) + at(ix + 1, iy) * fx * (1 - fy) + at(ix, iy + 1) * (1 - fx) * fy +
            at(ix + 1, iy + 1) * fx * fy).astype(np.float32)


@pytest.mark.parametrize("k", [37, 100, 301])
def test_l512_known_turns(gpulib, cuda, oracle_mod, k):
    """A particle equal to a reference turned by k x 360/512 degrees comes
    back as that reference at that angle, no shift, no mirror; at 512 samples
    the angle is closer than at 256 (odd k is a half step of the 256-sample
    grid), and within 1e-3 degrees of the FP64 oracle's."""
    from gpuisac import multi_ref_align
    D = 64
    st = synth.make_stack(4, D, 4, 0, None, 26.0, 77)
    ang = k * 360.0 / 512.0
    rot = _turned(st.refs[2], ang, D)[None]
    res = {}
    for L in (256, 512):
        pl, d = multi_ref_align(rot, st.refs, 29, 0.0, 0.0, ring_len=L)
        q = int(np.argmax(d[:, 0]))
        assert q == 2
        a = pl.reshape(4, 1, 4)[q, 0]
        assert a[1] == 0.0 and a[2] == 0.0 and a[3] == 0.0
        res[L] = float(a[0])
    err = {L: min(abs(v - ang), 360.0 - abs(v - ang)) for L, v in res.items()}
    assert err[512] < 0.5 * 360.0 / 512.0
    assert err[512] <= err[256] + 1e-3
    peak_o, d_o = oracle_512(oracle_mod, rot, st.refs, 29, 0.0, gpulib.get_texture_limit(D))
    assert abs(res[512] - float(peak_o[2, 0, 0])) < 1e-3
    print(f"k={k}: turned {ang:.4f}, found {res[512]:.4f} (512), {res[256]:.4f} (256)")
