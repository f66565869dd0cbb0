"""gpuisac -- GB300 multi-reference 2D alignment (GPU-ISAC's hot path).

The compute path is libgpu_aln_pack.so (hand-written sm_103a CUDA behind the
reference's C-ABI); this package is its Python host side.
"""
from ._lib import AlignConfig, AlignParam, GpuIsacError, load  # noqa: F401
from .align import contraction, make_config, multi_ref_align, multi_ref_align_device, spectra_device  # noqa: F401

__version__ = "0.1.0"
