"""Host-side checks of the averaging step's Python entry (no GPU): the
arguments it refuses before anything reaches the library."""
import pytest

torch = pytest.importorskip("torch")


def test_refuses_host_tensors_and_bad_shapes():
    from gpuisac import GpuIsacError
    from gpuisac.averages import class_averages_device
    parts = torch.zeros((10, 8, 8))
    peaks = torch.zeros((3, 10, 4))
    bel = torch.zeros(10, dtype=torch.int32)
    with pytest.raises(GpuIsacError, match="CUDA stack"):
        class_averages_device(parts, peaks, bel, 0.2, 0.2)
    with pytest.raises(GpuIsacError, match="CUDA stack"):
        class_averages_device(torch.zeros((10, 8)), peaks, bel, 0.2, 0.2)


def test_base_shifts_shape():
    import numpy as np

    from gpuisac.isac import base_shifts_of
    out = base_shifts_of(np.zeros((5, 4), np.float32))
    assert out.shape == (5, 2) and out.dtype == np.float32 and not out.any()
