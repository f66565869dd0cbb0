"""The bounds-checked build (gpu-isac_gb300/build.py --checked, -DGPUISAC_CHECKED)
on small cases of every alignment path -- FP32 and tensor-core contractions
at 76^2 / 35 rings and 128^2 / 61 rings (two shift blocks), 512-sample rings,
the grouped launch sequence, the averaging step at four image sides -- run in
a child process that loads the checked library (GPUISAC_LIBRARY).  Every
guarded access of the spectra, operand, contraction, FFT, peak and averaging
kernels must stay inside the extent its kernel was given (no access skipped),
and every result must equal the normal build's bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = r'''
import sys
import numpy as np
import torch
sys.path[:0] = [sys.argv[1]]
from gpuisac import _lib, multi_ref_align, synth
from gpuisac.align import multi_ref_align_groups_device
import ctypes
L = _lib.load()
out = {}
st = synth.make_stack(60, 76, 7, 3, 0.1, 30.0, 301)
for mode in ("fp32", "bf16x3"):
    pl, d = multi_ref_align(st.particles, st.refs, 35, 3.0, 3.0, contraction_mode=mode)
    out[f"mref_{mode}_d"], out[f"mref_{mode}_p"] = d, pl
big = synth.make_stack(10, 128, 4, 4, 0.1, 56.0, 302)
for mode in ("fp32", "bf16x3"):
    pl, d = multi_ref_align(big.particles, big.refs, 61, 4.0, 4.0, contraction_mode=mode)
    out[f"big_{mode}_d"], out[f"big_{mode}_p"] = d, pl
pl, d = multi_ref_align(st.particles[:20], st.refs, 35, 2.0, 2.0, ring_len=512)
out["l512_d"], out["l512_p"] = d, pl
dev = torch.device("cuda:0")
parts, refs = torch.from_numpy(st.particles).to(dev), torch.from_numpy(st.refs).to(dev)
dg, pg, _ = multi_ref_align_groups_device(parts, refs, [(0, 25, 0, 3), (25, 35, 2, 5), (5, 1, 6, 1)], 35, 3.0, 3.0)
out["groups_d"], out["groups_p"] = dg.cpu().numpy(), pg.cpu().numpy()
from gpuisac.averages import class_averages
rng = np.random.default_rng(3)
for D in (64, 65, 150, 200):
    imgs = rng.standard_normal((90, D, D)).astype(np.float32)
    pk = np.concatenate([rng.uniform(0, 360, (3, 90, 1)), rng.uniform(-3, 3, (3, 90, 2)),
                         rng.integers(0, 2, (3, 90, 1))], 2).astype(np.float32)
    avg, prm, mem, sh = class_averages(imgs, pk, np.arange(90) % 3, 0.2, 0.2, True)
    out[f"avg{D}"], out[f"avg{D}_p"] = avg, prm
first = ctypes.c_ulonglong()
out["failures"] = np.array([L.gpuisac_checked_failures(ctypes.byref(first)), first.value], np.int64)
np.savez(sys.argv[2], **out)
'''


def _run(tmp_path, name, lib=None):
    env = dict(os.environ)
    if lib:
        env["GPUISAC_LIBRARY"] = lib
    else:
        env.pop("GPUISAC_LIBRARY", None)
    path = str(tmp_path / f"{name}.npz")
    r = subprocess.run([sys.executable, "-c", CASES, os.path.join(ROOT, "gpu-isac_gb300"), path], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return dict(np.load(path))


def test_checked_build_stays_in_bounds_and_matches(gpulib, tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("gpuisac_build", os.path.join(ROOT, "gpu-isac_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    checked_lib = b.build(checked=True)
    chk = _run(tmp_path, "checked", checked_lib)
    ref = _run(tmp_path, "normal")
    n_fail, first = chk.pop("failures")
    assert n_fail == 0, f"{n_fail} guarded accesses out of range, first site {first >> 48} index {first & (2**48 - 1)}"
    assert ref.pop("failures")[0] == -1  # the normal build has no guards
    for k in ref:
        assert np.array_equal(chk[k], ref[k]), k
