"""gpuisac_multi_ref_align_device_noalloc: the allocation-free entry point,
for callers that cannot call cudaMalloc (their GPU memory belongs to another
allocator, or they cannot afford cudaMalloc's implicit synchronisation).  Its
work space is a 32 MiB array inside the library, so it must give the same
results as the allocating entry point, call after call, and refuse workloads
that do not fit.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from gpuisac import synth

pytestmark = pytest.mark.gpu

PEAK_RTOL = 1e-4   # same tolerance as the other alignment tests
ANGLE_TOL = 0.05


def circ_diff(a, b):
    d = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) % 360.0
    return np.minimum(d, 360.0 - d)


def run(gpulib, fn, cfg, parts, refs, base, cuda, free_delta=None):
    """One call of entry point fn into fresh NaN-filled outputs.  With
    free_delta (a list), the device's free memory right before and right
    after the call (outputs already allocated, the stream idle on both
    sides) is measured and the change appended."""
    import torch

    from gpuisac import _lib
    R, P = refs.shape[0], parts.shape[0]
    d = torch.full((R, P), float("nan"), dtype=torch.float32, device=cuda)
    pk = torch.full((R, P, 4), float("nan"), dtype=torch.float32, device=cuda)
    st = torch.cuda.current_stream(cuda)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(cuda)[0]
    rc = getattr(gpulib, fn)(ctypes.byref(cfg), parts.data_ptr(), refs.data_ptr(), base.data_ptr(), d.data_ptr(),
                             pk.data_ptr(), st.cuda_stream)
    if rc:
        _lib.check(gpulib)
    torch.cuda.synchronize()
    if free_delta is not None:
        free_delta.append(free0 - torch.cuda.mem_get_info(cuda)[0])
    return d.cpu().numpy(), pk.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(gpulib, cuda):
    import torch

    from gpuisac import make_config
    # 300 particles of 1.7 MB spectra each: the 32 MiB array holds ~18 at a
    # time, so the call walks many chunks
    st = synth.make_stack(300, 76, 20, 3, 0.05, 34.0, 777)
    parts = torch.from_numpy(st.particles).to(cuda)
    refs = torch.from_numpy(st.refs).to(cuda)
    base = torch.from_numpy(np.random.default_rng(5).uniform(-1.5, 1.5, (300, 2)).astype(np.float32)).to(cuda)
    cfg = make_config(300, 20, 76, 35, 256, 1.0, 3.0, 3.0)
    d_ref, pk_ref = run(gpulib, "gpuisac_multi_ref_align_device", cfg, parts, refs, base, cuda)
    deltas = []
    for _ in range(2):  # two calls in a row share the array
        d, pk = run(gpulib, "gpuisac_multi_ref_align_device_noalloc", cfg, parts, refs, base, cuda, deltas)
        assert np.isfinite(d).all() and np.isfinite(pk).all()
        rel = np.abs(d.astype(np.float64) - d_ref) / np.maximum(np.abs(d_ref), 1e-30)
        assert rel.max() <= PEAK_RTOL
        assert (pk[..., 1:] == pk_ref[..., 1:]).all()
        assert circ_diff(pk[..., 0], pk_ref[..., 0]).max() < ANGLE_TOL
    # the first call on a device may load the library's device code and its
    # static array (module loading is lazy); the second allocates nothing
    assert deltas[1] == 0, f"device free memory changed by {deltas[1]} bytes across a call"


def test_noalloc_rejects_workloads_beyond_its_array(gpulib, cuda):
    import torch

    from gpuisac import _lib, make_config
    # 1000 references x 35 rings of spectra (35 MB) cannot fit 32 MiB; the
    # buffers are real and sized for the call, and the call must refuse it
    parts = torch.zeros((1, 76, 76), dtype=torch.float32, device=cuda)
    refs = torch.zeros((1000, 76, 76), dtype=torch.float32, device=cuda)
    base = torch.zeros((1, 2), dtype=torch.float32, device=cuda)
    d = torch.zeros((1000, 1), dtype=torch.float32, device=cuda)
    pk = torch.zeros((1000, 1, 4), dtype=torch.float32, device=cuda)
    cfg = make_config(1, 1000, 76, 35, 256, 1.0, 3.0, 3.0)
    gpulib.gpuisac_clear_error()
    rc = gpulib.gpuisac_multi_ref_align_device_noalloc(ctypes.byref(cfg), parts.data_ptr(), refs.data_ptr(),
                                                       base.data_ptr(), d.data_ptr(), pk.data_ptr(), None)
    assert rc == 2
    code, msg = _lib.last_error(gpulib)
    assert code == 2 and "work space" in msg
    gpulib.gpuisac_clear_error()
