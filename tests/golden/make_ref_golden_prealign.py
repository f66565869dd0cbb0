#!/usr/bin/env python3
"""Golden outputs and run time of the reference's own GPU library for the
pre-alignment path.

    python tests/golden/make_ref_golden_prealign.py --ref-src DIR [--out DIR] [--time]

DIR is the reference repository root (its cuda/ sources).  The library is
built with make_ref_golden.py's recipe (no source edits) and driven as
ali2d_base_gpu_isac_CLEAN drives it (bin/sp_isac_applications.py:1455-1660):
pre_align_init with the batch size, the particles fetched once when one batch
holds them (else per batch), then per shift step reset_shifts and per
iteration the average fetched and pre_align_run over the batches; the
AlignParam array is stored after every run.  Needs a CUDA GPU.  Inputs are
regenerated bit for bit from make_ref_golden.gen_inputs (one reference, its
particles; the average = the reference image); only parameters and outputs
are stored.  --time times one pre_align_run over bench.py's pre-alignment
workload instead.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("make_ref_golden", os.path.join(HERE, "make_ref_golden.py"))
base = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(base)

# (name, P, D, ring_num, batch, [(shift range, step), ...], iterations per step, seed)
CASES = [
    ("pre_p40_d64", 40, 64, 29, 40, [(2.0, 1.0), (1.0, 0.5)], 2, 3001),
    ("pre_p36_d76_batches", 36, 76, 35, 16, [(3.0, 1.0)], 2, 3002),
]


def case_inputs(P, D, seed):
    parts, refs, _ = base.gen_inputs(P, 1, D, seed, False)
    return parts, np.ascontiguousarray(refs[:1])


def bind(lib):
    fp = ctypes.POINTER(ctypes.c_float)
    lib.pre_align_init.argtypes = [ctypes.c_uint, ctypes.POINTER(base.AlignConfig), ctypes.c_uint]
    lib.pre_align_init.restype = ctypes.c_ulonglong
    lib.pre_align_fetch.argtypes = [ctypes.POINTER(fp), ctypes.c_uint, ctypes.c_char_p]
    lib.pre_align_fetch.restype = None
    lib.pre_align_run.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.pre_align_run.restype = None
    lib.reset_shifts.argtypes = [ctypes.c_float, ctypes.c_float]
    lib.reset_shifts.restype = None
    return fp


def run_reference(lib, parts, avg, ring_num, batch, schedule, iters, record=True, timing=None):
    fp = bind(lib)
    P, D = parts.shape[0], parts.shape[1]
    rng0, step0 = schedule[0]
    cfg = base.AlignConfig(batch, 1, D, ring_num, 256, step0, rng0, rng0, b"pre_aln")
    prm = ctypes.cast(lib.pre_align_init(P, ctypes.byref(cfg), 0), ctypes.POINTER(base.AlignParam))
    for i in range(P):                 # every particle starts at zero shift
        prm[i].shift_x = prm[i].shift_y = 0.0
    ptrs = (fp * P)(*[parts[i].ctypes.data_as(fp) for i in range(P)])
    aptr = (fp * 1)(avg[0].ctypes.data_as(fp))
    n_batches = (P + batch - 1) // batch
    if n_batches == 1:
        lib.pre_align_fetch(ptrs, P, b"sbj_batch")
    out = []
    for rng, step in schedule:
        lib.reset_shifts(rng, step)
        for _ in range(iters):
            lib.pre_align_fetch(aptr, 1, b"ref_batch")
            for b in range(n_batches):
                s, e = b * batch, min(P, (b + 1) * batch)
                if n_batches > 1:
                    sub = (fp * (e - s))(*[parts[i].ctypes.data_as(fp) for i in range(s, e)])
                    lib.pre_align_fetch(sub, e - s, b"sbj_batch")
                t = time.perf_counter()
                lib.pre_align_run(s, e)
                if timing is not None:
                    timing.append(time.perf_counter() - t)
            if record:
                out.append([[prm[i].shift_x, prm[i].shift_y, prm[i].angle, float(prm[i].mirror)] for i in range(P)])
    lib.gpu_clear()
    return np.array(out, np.float32)


def time_workload(lib, out_dir):
    """One pre_align_run over bench.py's pre-alignment workload: the 50,000
    particles of the multi-reference workload against their plain mean, 35
    rings, shift range 5 step 1 (121 shifts), one batch."""
    sys.path.insert(0, os.path.join(HERE, "..", "..", "gpu-isac_gb300"))
    from gpuisac import synth
    st = synth.workload_stack(1)
    parts = np.ascontiguousarray(st.particles)
    avg = np.ascontiguousarray(parts.astype(np.float64).mean(0, keepdims=True).astype(np.float32))
    times = []
    run_reference(lib, parts, avg, 35, parts.shape[0], [(5.0, 1.0)], 2, record=False, timing=times)
    res = {"workload": "prealign_50000x76_121shifts", "seconds_per_run": times,
           "particle_alignments_per_s": parts.shape[0] / min(times)}
    with open(os.path.join(out_dir, "ref_gpu_time_prealign.json"), "w") as f:
        json.dump(res, f)
    print(json.dumps(res), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--build-dir", default=os.path.join(HERE, "..", "_build", "ref"))
    ap.add_argument("--time", action="store_true", help="only time bench.py's pre-alignment workload")
    a = ap.parse_args()
    lib = ctypes.CDLL(base.build_ref(a.ref_src, a.build_dir))
    if a.time:
        time_workload(lib, a.out)
        return
    for name, P, D, NR, batch, schedule, iters, seed in CASES:
        parts, avg = case_inputs(P, D, seed)
        params = run_reference(lib, parts, avg, NR, batch, schedule, iters)
        np.savez_compressed(os.path.join(a.out, f"ref_{name}.npz"), params=params, seed=seed,
                            input_sum=np.float64(parts.astype(np.float64).sum() + avg.astype(np.float64).sum()))
        print(name, "done", flush=True)


if __name__ == "__main__":
    main()
