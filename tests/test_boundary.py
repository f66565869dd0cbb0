"""The C-ABI boundary without a GPU: the library loads, exports every symbol
include/gpu_aln_pack.h declares, its structs match the reference's ctypes
mirrors byte for byte, and argument errors are reported, not fatal."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpu_aln_pack.h")


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gpuisac_build", os.path.join(ROOT, "gpu-isac_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    from gpuisac import _lib
    return _lib.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"if", "defined", "sizeof"}
    return sorted({n for n in names if n not in skip})


def test_header_declares_the_reference_exports():
    names = set(declared_functions())
    for ref_export in ("multi_ref_align_init", "multi_ref_align", "gpu_clear", "reset_shifts", "print_gpu_info",
                       "get_texture_limit", "pre_align_init", "pre_align_size_check", "pre_align_fetch",
                       "pre_align_run", "ref_free_alignment_2D_init", "ref_free_alignment_2D_size_check",
                       "ref_free_alignment_2D", "ref_free_alignment_2D_filter_references"):
        assert ref_export in names


def test_every_declared_symbol_is_exported(lib):
    so = os.path.join(ROOT, "gpu-isac_gb300", "lib", "libgpu_aln_pack.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    from gpuisac import _lib
    assert set(_lib.EXPORTS) == set(declared_functions())
    for n in declared_functions():
        getattr(lib, n)


def test_dropin_file_name_exists(lib):
    assert os.path.exists(os.path.join(ROOT, "gpu-isac_gb300", "lib", "gpu_aln_pack.so"))


def test_struct_layout_matches_reference():
    from gpuisac import AlignConfig, AlignParam
    # cuda/gpu_aln_common.h:62-85 on LP64
    assert ctypes.sizeof(AlignConfig) == 40 and AlignConfig.aln_type.offset == 32
    assert ctypes.sizeof(AlignParam) == 24 and AlignParam.mirror.offset == 20


def _cfg(**kw):
    from gpuisac import make_config
    base = dict(sbj_num=10, ref_num=3, img_dim=64, ring_num=29, ring_len=256, shift_step=1.0, shift_rng_x=2.0,
                shift_rng_y=2.0)
    base.update(kw)
    return make_config(**base)


def test_shift_count_host_only(lib):
    assert lib.gpuisac_shift_count(ctypes.byref(_cfg())) == 25
    assert lib.gpuisac_shift_count(ctypes.byref(_cfg(shift_rng_x=3.0, shift_rng_y=3.0))) == 49
    assert lib.gpuisac_shift_count(ctypes.byref(_cfg(shift_rng_x=0.0, shift_rng_y=0.0))) == 1


@pytest.mark.parametrize("kw,code", [(dict(ring_len=128), 4), (dict(ring_num=0), 4), (dict(ring_num=500), 4),
                                     (dict(img_dim=1), 2), (dict(shift_step=0.0), 2),
                                     (dict(aln_type=b"pre_aln"), 4)])
def test_init_rejects_bad_config(lib, kw, code):
    from gpuisac import _lib
    cfg = _cfg(**kw)
    lib.gpuisac_clear_error()
    p = lib.multi_ref_align_init(ctypes.byref(cfg), 0)
    assert not p
    c, msg = _lib.last_error(lib)
    assert c == code and msg
    lib.gpuisac_clear_error()
    assert _lib.last_error(lib)[0] == 0


def test_align_before_init_is_an_error(lib):
    from gpuisac import _lib
    lib.gpu_clear()
    lib.gpuisac_clear_error()
    lib.multi_ref_align(None, None, None, None, 10, ctypes.c_float(0.9))
    assert _lib.last_error(lib)[0] == 3
    lib.gpuisac_clear_error()


def test_multigroup_before_init_fails(lib):
    from gpuisac import _lib
    lib.gpu_clear()
    lib.gpuisac_clear_error()
    lib.ref_free_alignment_2D()
    code, msg = _lib.last_error(lib)
    assert code == 3 and "before ref_free_alignment_2D_init" in msg
    lib.gpuisac_clear_error()
    lib.ref_free_alignment_2D_filter_references(ctypes.c_float(0.3), ctypes.c_float(0.2))
    assert _lib.last_error(lib)[0] == 3
    lib.gpuisac_clear_error()
    assert lib.gpuisac_ref_free_averages(None) == 3
    lib.gpuisac_clear_error()


def test_multigroup_init_rejects_bad_class_lists(lib):
    """Classes must be sorted runs 0 .. ref_num-1 (the reference's class
    index, cuda/gpu_aln_noref.cu:825-835); rejected before any device work."""
    from gpuisac import _lib
    import numpy as np
    from gpuisac.align import make_config, ptr_array
    imgs = np.zeros((4, 16, 16), np.float32)
    refs = np.zeros((2, 16, 16), np.float32)
    for cids in ([1, 1, 0, 0], [0, 0, 2, 2], [0, 1, 0, 1]):
        cfg = make_config(4, 2, 16, 5, 256, 1.0, 1.0, 1.0, b"multigroup_aln")
        lib.gpuisac_clear_error()
        p = lib.ref_free_alignment_2D_init(ctypes.byref(cfg), ptr_array(imgs), ptr_array(refs),
                                           (ctypes.c_int * 4)(*cids), 0)
        assert not p
        assert _lib.last_error(lib)[0] == 2
    lib.gpuisac_clear_error()


def test_pre_align_run_before_init_fails(lib):
    from gpuisac import _lib
    lib.gpuisac_clear_error()
    lib.pre_align_run.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.pre_align_run.restype = None
    lib.pre_align_run(0, 10)
    code, msg = _lib.last_error(lib)
    assert code == 3 and "before pre_align_init" in msg
    lib.gpuisac_clear_error()


def test_python_host_raises_without_library(tmp_path):
    from gpuisac import _lib
    with pytest.raises(_lib.GpuIsacError):
        _lib.load(str(tmp_path / "missing.so"))


def test_assign_groups_rejects_bad_arguments_on_the_host(lib):
    from gpuisac import _lib
    d = (ctypes.c_float * 6)()
    out = (ctypes.c_int * 4)()
    lib.gpuisac_clear_error()
    assert lib.gpuisac_assign_groups(None, 2, 3, ctypes.cast(out, ctypes.c_void_p)) == 2
    assert lib.gpuisac_assign_groups(ctypes.cast(d, ctypes.c_void_p), 0, 3, ctypes.cast(out, ctypes.c_void_p)) == 2
    assert lib.gpuisac_assign_groups(ctypes.cast(d, ctypes.c_void_p), 4, 3, ctypes.cast(out, ctypes.c_void_p)) == 2
    assert lib.gpuisac_assign_groups_device(ctypes.cast(d, ctypes.c_void_p), 0, 2, 3, None, None, None, None) == 2
    code, msg = _lib.last_error(lib)
    assert code == 2 and "assign_groups" in msg
    lib.gpuisac_clear_error()


def test_class_averages_rejects_bad_arguments_on_the_host(lib):
    """gpuisac_class_averages checks its arguments before any device call:
    each refusal is error 2 with a message (the pointers are never read)."""
    from gpuisac import _lib
    p = 1 << 20  # a 16-byte aligned address the refusals never dereference
    f = lib.gpuisac_class_averages
    lib.gpuisac_clear_error()
    assert f(None, 10, 8, p, 0, p, 3, 0.2, 0.2, 1, p, p, None, None, None) == 2   # no images
    assert f(p, 0, 8, p, 0, p, 3, 0.2, 0.2, 1, p, p, None, None, None) == 2      # no particles
    assert f(p, 10, 8, p, 0, p, 0, 0.2, 0.2, 1, p, p, None, None, None) == 2     # no groups
    assert f(p, 10, 300, p, 0, p, 3, 0.2, 0.2, 1, p, p, None, None, None) == 2   # side above 256
    assert f(p, 10, 8, p, 5, p, 3, 0.2, 0.2, 1, p, p, None, None, None) == 2     # pitch below n_img
    assert f(p, 10, 8, p + 4, 0, p, 3, 0.2, 0.2, 1, p, p, None, None, None) == 2  # peaks misaligned
    assert f(p, 10, 8, p, 0, p, 3, 0.7, 0.2, 1, p, p, None, None, None) == 2     # cut-off above Nyquist
    assert f(p, 10, 8, p, 0, p, 3, 0.2, -0.1, 1, p, p, None, None, None) == 2    # negative fall-off
    assert f(p, 10, 8, p, 0, p, 3, 0.2, 0.2, 1, p, p + 8, None, None, None) == 2  # params misaligned
    code, msg = _lib.last_error(lib)
    assert code == 2 and "class_averages" in msg
    lib.gpuisac_clear_error()
