"""Host logic of the ormq-shaped entry point and the normalisation oracle
(no GPU): argument meaning of bin/sp_isac_alignment.py:400-447 (ormq) and
:713-747 (Numrinit), the shift conversion of bin/sp_isac2_gpu.py:1015-1022,
and the masked normalisation of bin/sp_isac2_gpu.py:925-931."""
import math

import numpy as np
import pytest


def numrinit(first_ring, last_ring, skip=1, mode="F"):
    """Ring layout restated from Numrinit (bin/sp_isac_alignment.py:713-747):
    per ring (radius, first sample, samples), the sample count a power of two
    that oversamples the circumference, the last ring's rule widened."""
    dpi = 2 * math.pi if mode in ("f", "F") else math.pi
    numr, lcirc = [], 1
    for k in range(first_ring, last_ring + 1, skip):
        jp = int(dpi * k + 0.5)
        ip = 1 << (jp.bit_length())  # smallest power of two above jp
        if k + skip <= last_ring and jp > ip + ip // 2:
            ip = min(32768, 2 * ip)
        if k + skip > last_ring and jp > ip + ip // 5:
            ip = min(32768, 2 * ip)
        numr += [k, lcirc, ip]
        lcirc += ip
    return numr


def test_numr_rings_of_the_workload_layouts():
    from gpuisac.ormq import numr_rings
    assert numr_rings(numrinit(1, 29)) == (29, 256)
    assert numr_rings(numrinit(1, 35)) == (35, 256)
    assert numr_rings(numrinit(1, 61)) == (61, 512)  # the large-box layout
    assert numr_rings(numrinit(1, 90)) == (90, 1024)  # refused below
    with pytest.raises(ValueError):
        numr_rings(numrinit(2, 30))                  # rings must start at 1
    with pytest.raises(ValueError):
        numr_rings([1, 1, 8, 2])                     # not triples


@pytest.mark.parametrize("kw,msg", [(dict(mode="H"), "full-circle"), (dict(delta=1.0), "delta"),
                                    (dict(numr=numrinit(1, 90)), "256"), (dict(xrng=[1.0, 2.0]), "symmetric")])
def test_ormq_refuses_what_the_gpu_path_does_not_compute(kw, msg):
    from gpuisac.ormq import ormq
    args = dict(images=np.zeros((2, 64, 64), np.float32), refs=np.zeros((64, 64), np.float32), xrng=[2.0, 2.0],
                yrng=[2.0, 2.0], step=1.0, mode="F", numr=numrinit(1, 29), cnx=33, cny=33)
    args.update(kw)
    with pytest.raises(ValueError, match=msg):
        ormq(**args)


def test_shift_conversion_is_the_callers():
    """ormq_post restates the caller's conversion: sx' = -sx cos a + sy (-sin a) ... as written at
    bin/sp_isac2_gpu.py:1015-1022; a quarter turn maps (sx, sy) = (1, 0) to (0, 1)."""
    import oracle
    pk = np.array([[90.0, 1.0, 0.0, 0.0], [0.0, 2.0, -3.0, 1.0], [180.0, 1.5, 0.5, 0.0]])
    ang, sxs, sys_, mir = oracle.ormq_post(pk)
    assert np.allclose(sxs, [0.0, -2.0, 1.5], atol=1e-12) and np.allclose(sys_, [1.0, 3.0, 0.5], atol=1e-12)
    assert (mir == pk[:, 3]).all() and (ang == pk[:, 0]).all()


def test_normalize_mask_oracle_properties():
    import oracle
    rng = np.random.default_rng(4)
    x = rng.normal(3.0, 2.5, (5, 40, 40))
    yy, xx = np.mgrid[:40, :40]
    mask = ((xx - 20) ** 2 + (yy - 20) ** 2 <= 15 ** 2).astype(np.float32)
    n = oracle.normalize_mask(x, mask, no_sigma=False)
    sel = mask > 0.5
    assert np.allclose(n[:, sel].mean(1), 0.0, atol=1e-12)
    assert np.allclose(n[:, sel].std(1), 1.0, atol=1e-12)
    m = oracle.normalize_mask(x, mask, no_sigma=True)
    assert np.allclose(m[:, sel].mean(1), 0.0, atol=1e-12)
    assert np.allclose(m - x, (m - x)[:, :1, :1])            # a constant offset per image
    z = oracle.normalize_mask(np.full((1, 8, 8), 2.0), np.ones((8, 8)), no_sigma=False)
    assert np.allclose(z, 0.0)                                # no spread: only the mean is taken off
