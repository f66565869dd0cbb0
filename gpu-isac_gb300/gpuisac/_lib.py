"""ctypes binding of libgpu_aln_pack.so.

The structures and argtypes are the ones the reference's drivers declare
(bin/sp_isac2_gpu.py:121-187, bin/sp_isac_applications.py:86-157), so code
written against the reference's gpu_aln_pack.so binds this library unchanged.
There is no fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
# GPUISAC_LIBRARY: another build of the library (the bounds-checked one)
LIB_PATH = os.environ.get("GPUISAC_LIBRARY") or os.path.join(PKG_ROOT, "lib", "libgpu_aln_pack.so")


class AlignConfig(ctypes.Structure):
    """Mirror of AlignConfig (cuda/gpu_aln_common.h:62-76)."""
    _fields_ = [("sbj_num", ctypes.c_uint), ("ref_num", ctypes.c_uint), ("img_dim", ctypes.c_uint),
                ("ring_num", ctypes.c_uint), ("ring_len", ctypes.c_uint),
                ("shift_step", ctypes.c_float), ("shift_rng_x", ctypes.c_float),
                ("shift_rng_y", ctypes.c_float), ("aln_type", ctypes.c_char_p)]


class AlignParam(ctypes.Structure):
    """Mirror of AlignParam (cuda/gpu_aln_common.h:78-85)."""
    _fields_ = [("sbj_id", ctypes.c_int), ("ref_id", ctypes.c_int), ("shift_x", ctypes.c_float),
                ("shift_y", ctypes.c_float), ("angle", ctypes.c_float), ("mirror", ctypes.c_bool)]


aln_cfg_ptr = ctypes.POINTER(AlignConfig)
aln_param_ptr = ctypes.POINTER(AlignParam)
float_ptr = ctypes.POINTER(ctypes.c_float)
float_ptr_ptr = ctypes.POINTER(float_ptr)

# every symbol include/gpu_aln_pack.h declares
EXPORTS = (
    "multi_ref_align_init", "multi_ref_align", "gpu_clear", "reset_shifts", "print_gpu_info",
    "get_texture_limit", "pre_align_init", "pre_align_size_check", "pre_align_fetch", "pre_align_run",
    "ref_free_alignment_2D_init", "ref_free_alignment_2D_size_check", "ref_free_alignment_2D",
    "ref_free_alignment_2D_filter_references", "gpuisac_last_error", "gpuisac_clear_error",
    "gpuisac_version", "gpuisac_multi_ref_align_device", "gpuisac_spectra_device", "gpuisac_spectra_device_layout",
    "gpuisac_ccf_peak_device", "gpuisac_shift_count", "gpuisac_launch_count", "gpuisac_profile",
    "gpuisac_kernel_time", "gpuisac_multi_ref_align_device_noalloc", "gpuisac_multi_ref_align_groups_device",
    "gpuisac_align_proposals_device", "gpuisac_nn_features", "gpuisac_nn_gemm", "gpuisac_nn_bias_act",
    "gpuisac_nn_relu_backward", "gpuisac_nn_colsum", "gpuisac_nn_l2norm", "gpuisac_nn_l2norm_backward",
    "gpuisac_nn_softmax_xent", "gpuisac_nn_adam", "gpuisac_nn_topk", "gpuisac_nn_col_stats",
    "gpuisac_nn_affine_cols", "gpuisac_nn_group_max", "gpuisac_learned_align_device", "gpuisac_autotune_ccf",
    "gpuisac_ccf_tile_name", "gpuisac_nn_gemm_bf16", "gpuisac_assign_groups_device", "gpuisac_assign_groups",
    "gpuisac_ref_free_averages", "gpuisac_set_contraction", "gpuisac_get_contraction", "gpuisac_test_stall_ccf", "gpuisac_normalize_mask",
    "gpuisac_split_plan", "gpuisac_groups_stats", "gpuisac_checked_failures", "gpuisac_class_averages",
    "gpuisac_test_fail_alloc",
)


class GpuisacGroupStats(ctypes.Structure):
    """Mirror of GpuisacGroupStats (include/gpu_aln_pack.h)."""
    _fields_ = [("plan_ms", ctypes.c_double), ("record_ms", ctypes.c_double), ("waves", ctypes.c_uint),
                ("graph_launches", ctypes.c_uint), ("graphs_recorded", ctypes.c_uint)]


class GpuisacGroup(ctypes.Structure):
    """Mirror of GpuisacGroup (include/gpu_aln_pack.h)."""
    _fields_ = [("sbj_offset", ctypes.c_uint), ("sbj_num", ctypes.c_uint), ("ref_offset", ctypes.c_uint),
                ("ref_num", ctypes.c_uint), ("out_offset", ctypes.c_ulonglong)]


class GpuisacProposalNet(ctypes.Structure):
    """Mirror of GpuisacProposalNet (include/gpu_aln_pack.h): device pointers."""
    _fields_ = [("nk", ctypes.c_uint), ("hidden", ctypes.c_uint), ("emb", ctypes.c_uint),
                ("mu", ctypes.c_void_p), ("inv_sd", ctypes.c_void_p), ("W1", ctypes.c_void_p),
                ("b1", ctypes.c_void_p), ("W2", ctypes.c_void_p), ("b2", ctypes.c_void_p)]


class GpuIsacError(RuntimeError):
    pass


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the library (once) and declare its argtypes."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise GpuIsacError(f"{p} is missing: build it with gpu-isac_gb300/build.py")
    L = ctypes.CDLL(p)
    # the reference's own declarations (bin/sp_isac2_gpu.py:183-187)
    L.multi_ref_align_init.argtypes = [aln_cfg_ptr, ctypes.c_uint]
    L.multi_ref_align_init.restype = aln_param_ptr
    L.multi_ref_align.argtypes = [float_ptr_ptr, float_ptr_ptr, float_ptr, float_ptr, ctypes.c_uint, ctypes.c_float]
    L.multi_ref_align.restype = None
    L.gpu_clear.argtypes = []
    L.gpu_clear.restype = None
    L.reset_shifts.argtypes = [ctypes.c_float, ctypes.c_float]
    L.print_gpu_info.argtypes = [ctypes.c_uint]
    L.get_texture_limit.argtypes = [ctypes.c_uint]
    L.get_texture_limit.restype = ctypes.c_int
    # the pre-alignment session, bound as bin/sp_isac_applications.py:86-157 binds it
    L.pre_align_init.argtypes = [ctypes.c_uint, aln_cfg_ptr, ctypes.c_uint]
    L.pre_align_init.restype = ctypes.c_ulonglong
    L.pre_align_size_check.argtypes = [ctypes.c_uint, aln_cfg_ptr, ctypes.c_uint, ctypes.c_float, ctypes.c_bool]
    L.pre_align_size_check.restype = ctypes.c_bool
    L.pre_align_fetch.argtypes = [float_ptr_ptr, ctypes.c_uint, ctypes.c_char_p]
    L.pre_align_fetch.restype = None
    L.pre_align_run.argtypes = [ctypes.c_int, ctypes.c_int]
    L.pre_align_run.restype = None
    # the multigroup session, bound as bin/sp_isac_applications.py:86-157 binds it
    L.ref_free_alignment_2D_init.argtypes = [aln_cfg_ptr, float_ptr_ptr, float_ptr_ptr,
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_uint]
    L.ref_free_alignment_2D_init.restype = ctypes.c_ulonglong
    L.ref_free_alignment_2D_size_check.argtypes = [aln_cfg_ptr, ctypes.c_uint, ctypes.c_float, ctypes.c_bool]
    L.ref_free_alignment_2D_size_check.restype = ctypes.c_bool
    L.ref_free_alignment_2D.argtypes = []
    L.ref_free_alignment_2D.restype = None
    L.ref_free_alignment_2D_filter_references.argtypes = [ctypes.c_float, ctypes.c_float]
    L.ref_free_alignment_2D_filter_references.restype = None
    # additions
    L.gpuisac_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.gpuisac_last_error.restype = ctypes.c_int
    L.gpuisac_clear_error.argtypes = []
    L.gpuisac_version.restype = ctypes.c_char_p
    L.gpuisac_multi_ref_align_device.argtypes = [aln_cfg_ptr, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gpuisac_multi_ref_align_device.restype = ctypes.c_int
    L.gpuisac_multi_ref_align_device_noalloc.argtypes = [aln_cfg_ptr, ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_void_p]
    L.gpuisac_multi_ref_align_device_noalloc.restype = ctypes.c_int
    L.gpuisac_multi_ref_align_groups_device.argtypes = [aln_cfg_ptr, ctypes.POINTER(GpuisacGroup), ctypes.c_uint,
                                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gpuisac_multi_ref_align_groups_device.restype = ctypes.c_int
    L.gpuisac_groups_stats.argtypes = [ctypes.POINTER(GpuisacGroupStats)]
    L.gpuisac_groups_stats.restype = ctypes.c_int
    L.gpuisac_checked_failures.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
    L.gpuisac_checked_failures.restype = ctypes.c_int
    vp, ci, cl, cf, cu = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_uint
    L.gpuisac_align_proposals_device.argtypes = [aln_cfg_ptr, vp, vp, vp, vp, cu, vp, cu, vp, vp, vp]
    L.gpuisac_nn_features.argtypes = [vp, cu, cu, cu, vp, vp, vp, vp]
    L.gpuisac_nn_col_stats.argtypes = [vp, cl, ci, cf, vp, vp, vp]
    L.gpuisac_autotune_ccf.argtypes = [aln_cfg_ptr, vp, vp, cu, ctypes.c_char_p, ctypes.c_size_t, vp]
    L.gpuisac_autotune_ccf.restype = ci
    L.gpuisac_ccf_tile_name.argtypes = [cu, cu, ctypes.c_char_p, ctypes.c_size_t]
    L.gpuisac_ccf_tile_name.restype = ci
    L.gpuisac_nn_affine_cols.argtypes = [vp, cl, ci, vp, vp, vp]
    L.gpuisac_nn_group_max.argtypes = [vp, cl, ci, ci, vp, vp]
    L.gpuisac_learned_align_device.argtypes = [aln_cfg_ptr, vp, vp, vp, ctypes.POINTER(GpuisacProposalNet), vp, cu,
                                               cf, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_ulonglong), vp]
    L.gpuisac_nn_gemm.argtypes = [ci, ci, ci, cf, vp, cl, cl, vp, cl, cl, cf, vp, cl, vp]
    L.gpuisac_nn_gemm_bf16.argtypes = [ci, ci, ci, cf, vp, cl, vp, cl, vp, ci, vp, cl, vp, vp]
    L.gpuisac_nn_gemm_bf16.restype = ci
    L.gpuisac_assign_groups_device.argtypes = [vp, ctypes.c_ulonglong, cu, cu, vp, vp, ctypes.POINTER(cu), vp]
    L.gpuisac_assign_groups_device.restype = ci
    L.gpuisac_assign_groups.argtypes = [vp, cu, cu, vp]
    L.gpuisac_assign_groups.restype = ci
    L.gpuisac_ref_free_averages.argtypes = [vp]
    L.gpuisac_ref_free_averages.restype = ci
    L.gpuisac_nn_bias_act.argtypes = [vp, vp, cl, ci, ci, vp]
    L.gpuisac_nn_relu_backward.argtypes = [vp, vp, cl, vp]
    L.gpuisac_nn_colsum.argtypes = [vp, cl, ci, vp, ci, vp]
    L.gpuisac_nn_l2norm.argtypes = [vp, cl, ci, vp, vp, vp]
    L.gpuisac_nn_l2norm_backward.argtypes = [vp, vp, vp, cl, ci, vp, vp]
    L.gpuisac_nn_softmax_xent.argtypes = [vp, vp, cl, ci, vp, vp, vp]
    L.gpuisac_nn_adam.argtypes = [vp, vp, vp, vp, cl, cf, cf, cf, cf, cf, ci, vp]
    L.gpuisac_nn_topk.argtypes = [vp, cl, ci, ci, vp, vp]
    for name in ("gpuisac_align_proposals_device", "gpuisac_nn_features", "gpuisac_nn_gemm", "gpuisac_nn_bias_act",
                 "gpuisac_nn_relu_backward", "gpuisac_nn_colsum", "gpuisac_nn_l2norm", "gpuisac_nn_l2norm_backward",
                 "gpuisac_nn_softmax_xent", "gpuisac_nn_adam", "gpuisac_nn_topk", "gpuisac_nn_col_stats",
                 "gpuisac_nn_affine_cols", "gpuisac_nn_group_max", "gpuisac_learned_align_device"):
        getattr(L, name).restype = ci
    L.gpuisac_spectra_device.argtypes = [aln_cfg_ptr, ctypes.c_void_p, ctypes.c_uint, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gpuisac_spectra_device.restype = ctypes.c_int
    L.gpuisac_spectra_device_layout.argtypes = [aln_cfg_ptr, ctypes.c_void_p, ctypes.c_uint, ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                                                ctypes.c_void_p]
    L.gpuisac_spectra_device_layout.restype = ctypes.c_int
    L.gpuisac_ccf_peak_device.argtypes = [aln_cfg_ptr, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]
    L.gpuisac_ccf_peak_device.restype = ctypes.c_int
    L.gpuisac_launch_count.argtypes = []
    L.gpuisac_launch_count.restype = ctypes.c_ulonglong
    L.gpuisac_profile.argtypes = [ctypes.c_int]
    L.gpuisac_kernel_time.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_ulonglong),
                                      ctypes.POINTER(ctypes.c_double)]
    L.gpuisac_kernel_time.restype = ctypes.c_int
    L.gpuisac_shift_count.argtypes = [aln_cfg_ptr]
    L.gpuisac_shift_count.restype = ctypes.c_int
    L.gpuisac_set_contraction.argtypes = [ctypes.c_int]
    L.gpuisac_set_contraction.restype = ctypes.c_int
    L.gpuisac_get_contraction.argtypes = []
    L.gpuisac_get_contraction.restype = ctypes.c_int
    L.gpuisac_test_stall_ccf.argtypes = [ctypes.c_uint]
    L.gpuisac_test_stall_ccf.restype = None
    L.gpuisac_test_fail_alloc.argtypes = [ctypes.c_uint]
    L.gpuisac_test_fail_alloc.restype = None
    L.gpuisac_normalize_mask.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p]
    L.gpuisac_normalize_mask.restype = ctypes.c_int
    L.gpuisac_class_averages.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                                         ctypes.c_ulonglong, ctypes.c_void_p, ctypes.c_uint, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gpuisac_class_averages.restype = ctypes.c_int
    L.gpuisac_split_plan.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.POINTER(ctypes.c_uint),
                                     ctypes.c_uint]
    L.gpuisac_split_plan.restype = ctypes.c_int
    if path is None:
        _lib = L
    return L


def last_error(lib: ctypes.CDLL | None = None) -> tuple[int, str]:
    L = lib or load()
    buf = ctypes.create_string_buffer(512)
    code = L.gpuisac_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")


def check(lib: ctypes.CDLL | None = None) -> None:
    """Raise GpuIsacError if the library recorded an error (and clear it)."""
    L = lib or load()
    code, msg = last_error(L)
    if code:
        L.gpuisac_clear_error()
        raise GpuIsacError(f"gpuisac error {code}: {msg}")
