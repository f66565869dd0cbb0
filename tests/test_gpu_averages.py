"""The averaging step on the GPU (csrc/averages.cu, gpuisac.averages) against
the FP64 restatement (oracle.class_averages): averages within 2e-5 of the
largest average value, the re-centred parameters within 2e-6 (both round the
same float operations; the conversion and mean shifts are FP64 on both
sides), member counts and mean shifts equal.  Image sides cover the staged
path (even sides up to 160, bulk copies of whole images), odd sides and the
larger sides read from global memory, two passes of output rows (sides above
128), the finish kernel's spectra in global memory (sides above 160) and
sides of 4 and 5 pixels (every neighbour next to the wrap).  Also: more than
1,024 groups (the group scan's carry) and more than 16,384 (the scatter's
running counts in global memory), the chain with the
alignment and the group assignment on one stream, the errors the reference's
caller would meet (a group without members, a group index out of range), and
repeat calls bit-identical."""
import numpy as np
import pytest

from gpuisac import GpuIsacError, synth

pytestmark = pytest.mark.gpu

AVG_TOL = 2e-5  # of the largest |average| value
PARAM_TOL = 2e-6


def _case(P, R, D, seed, mirror_p=0.5, empty=()):
    rng = np.random.default_rng(seed)
    imgs = rng.standard_normal((P, D, D)).astype(np.float32)
    peaks = np.zeros((R, P, 4), np.float32)
    peaks[..., 0] = rng.uniform(0.0, 360.0, (R, P))
    peaks[..., 1:3] = rng.integers(-3, 4, (R, P, 2)) + rng.uniform(-0.5, 0.5, (R, P, 2))
    peaks[..., 3] = rng.uniform(size=(R, P)) < mirror_p
    groups = [g for g in range(R) if g not in empty]
    bel = np.asarray(groups, np.int32)[rng.integers(0, len(groups), P)]
    bel[:len(groups)] = groups[:P]  # every listed group has a member
    return imgs, peaks, bel


def _compare(oracle_mod, imgs, peaks, bel, fl, ff, center, out):
    avg, params, members, shifts = out
    a_o, p_o, m_o, s_o = oracle_mod.class_averages(imgs, peaks, bel, fl, ff, center)
    scale = max(np.abs(a_o).max(), 1e-6)
    err = np.abs(avg - a_o).max() / scale
    assert err < AVG_TOL, err
    assert np.array_equal(members, m_o)
    assert np.abs(params - p_o).max() < PARAM_TOL
    assert np.abs(shifts - s_o).max() < PARAM_TOL
    return err


@pytest.mark.parametrize("P,R,D,fl,ff,center", [
    (300, 6, 64, 0.2, 0.2, True),
    (240, 5, 76, 0.25, 0.1, True),
    (200, 4, 65, 0.2, 0.2, True),    # odd side: images read from global memory
    (120, 3, 128, 0.3, 0.2, True),
    (60, 3, 150, 0.2, 0.2, True),    # two passes of output rows, staged
    (40, 2, 200, 0.2, 0.0, True),    # global-memory images and spectra; the step filter
    (150, 5, 64, 0.0, 0.2, False),   # sums only
    (150, 5, 64, 0.0, 0.2, True),    # centring alone
])
def test_averages_match_oracle(gpulib, cuda, oracle_mod, P, R, D, fl, ff, center):
    from gpuisac.averages import class_averages
    imgs, peaks, bel = _case(P, R, D, 100 + D)
    out = class_averages(imgs, peaks, bel, fl, ff, center)
    err = _compare(oracle_mod, imgs, peaks, bel, fl, ff, center, out)
    print(f"P={P} R={R} D={D}: max |avg - oracle| / max |avg| = {err:.2e}")


@pytest.mark.parametrize("P,R,D", [
    (4000, 1500, 16),    # the group scan's carry over 1,024-group tiles
    (300, 7, 4),         # every source point next to the periodic wrap
    (200, 5, 5),
])
def test_many_groups_and_tiny_images(gpulib, cuda, oracle_mod, P, R, D):
    from gpuisac.averages import class_averages
    imgs, peaks, bel = _case(P, R, D, 9 + D)
    out = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    _compare(oracle_mod, imgs, peaks, bel, 0.2, 0.2, True, out)


def test_more_groups_than_shared_memory_counts(gpulib, cuda, oracle_mod):
    """16,400 groups: the scatter keeps each chunk's running counts in global
    memory.  Every group's peak row holds the same per-particle parameters
    (the matrix is 4.3 GB on the device; the oracle reads a strided view)."""
    import torch

    from gpuisac.averages import class_averages_device
    P, R, D = 16500, 16400, 4
    rng = np.random.default_rng(77)
    imgs = rng.standard_normal((P, D, D)).astype(np.float32)
    row = np.zeros((1, P, 4), np.float32)
    row[..., 0] = rng.uniform(0.0, 360.0, P)
    row[..., 1:3] = rng.uniform(-2.0, 2.0, (P, 2))
    row[..., 3] = rng.uniform(size=P) < 0.5
    bel = rng.integers(0, R, P).astype(np.int32)
    bel[:R] = rng.permutation(R)
    peaks_d = torch.from_numpy(row).to(cuda).expand(R, P, 4).contiguous()
    out = class_averages_device(torch.from_numpy(imgs).to(cuda), peaks_d, torch.from_numpy(bel).to(cuda),
                                0.2, 0.2, True)
    del peaks_d
    out = tuple(t.cpu().numpy() for t in out)
    view = np.lib.stride_tricks.as_strided(row, shape=(R, P, 4), strides=(0,) + row.strides[1:])
    _compare(oracle_mod, imgs, view, bel, 0.2, 0.2, True, out)


def test_repeat_calls_identical(gpulib, cuda):
    """Repeat calls give the same bits, also after gpu_clear released the
    step's work space (and the group assignment's)."""
    from gpuisac.assign import assign_groups
    from gpuisac.averages import class_averages
    imgs, peaks, bel = _case(500, 7, 76, 4)
    a = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    b = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    d = np.random.default_rng(4).uniform(0.0, 1.0, (7, 500)).astype(np.float32)
    ids = assign_groups(d, 7, 500)
    gpulib.gpu_clear()
    c = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    for x, y, z in zip(a, b, c):
        assert np.array_equal(x, y) and np.array_equal(x, z)
    assert assign_groups(d, 7, 500) == ids


def test_errors(gpulib, cuda, oracle_mod):
    from gpuisac.averages import class_averages
    imgs, peaks, bel = _case(100, 4, 32, 5, empty=(2,))
    with pytest.raises(GpuIsacError, match="no members"):
        class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    bad = bel.copy()
    bad[17] = 4
    with pytest.raises(GpuIsacError, match="outside"):
        class_averages(imgs, peaks, bad, 0.2, 0.2, True)
    with pytest.raises(GpuIsacError):
        class_averages(imgs, peaks, bel, 0.2, 0.7, True)
    # the context stays usable, and the groups with members still came out right
    imgs, peaks, bel = _case(100, 4, 32, 6)
    out = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    _compare(oracle_mod, imgs, peaks, bel, 0.2, 0.2, True, out)


def test_chain_with_alignment_and_assignment(gpulib, cuda, oracle_mod):
    """alignment -> group assignment -> averages on device tensors, one stream;
    the averages equal the oracle's on the same peaks and groups, and they
    reproduce the references (correlation inside the mask)."""
    import torch

    from gpuisac import multi_ref_align_device
    from gpuisac.assign import assign_groups_device
    from gpuisac.averages import class_averages_device
    P, R, D = 600, 6, 64
    st = synth.make_stack(P, D, R, 2, 0.5, 24.0, 31)
    parts = torch.from_numpy(st.particles).to(cuda)
    refs = torch.from_numpy(st.refs).to(cuda)
    d, pk = multi_ref_align_device(parts, refs, 25, 2.0, 2.0)
    _, bel, _ = assign_groups_device(d, with_id_list=False)
    avg, params, members, shifts = class_averages_device(parts, pk, bel, 0.0, 0.2, center=False)
    out = tuple(t.cpu().numpy() for t in (avg, params, members, shifts))
    _compare(oracle_mod, st.particles, pk.cpu().numpy(), bel.cpu().numpy(), 0.0, 0.2, False, out)
    mask = synth._mask(D, 24)
    for r in range(R):
        assert np.corrcoef(out[0][r][mask], st.refs[r][mask])[0, 1] > 0.9
    assert members.sum().item() == P
