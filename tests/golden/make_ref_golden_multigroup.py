#!/usr/bin/env python3
"""Golden outputs of the reference's own GPU library for the multigroup
alignment of the stability test.

    python tests/golden/make_ref_golden_multigroup.py --ref-src DIR [--out DIR]

DIR is the reference repository root (its cuda/ sources).  The library is
built with make_ref_golden.py's recipe (no source edits) and driven as
multigroup_refinement_gpu (bin/sp_isac_applications.py:4552-4650) drives it:
ref_free_alignment_2D_init with class-sorted particles and their class
averages, the particles' start shifts written into the AlignParam array, then
per iteration the tangent filter (cut-off ramping from 0.1 when a cut-off is
given) and ref_free_alignment_2D; the AlignParam array is stored after every
iteration.  Needs a CUDA GPU.  Inputs are regenerated bit for bit from
make_ref_golden.gen_inputs (particles sorted by class, averages = class means
quantised to 1/4096); only parameters and outputs are stored.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("make_ref_golden", os.path.join(HERE, "make_ref_golden.py"))
base = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(base)

# (name, P, R, D, ring_num, shift range, iterations, cut-off (0: no filter), falloff, start shifts?, seed)
CASES = [
    ("mg_p60_r4_d64", 60, 4, 64, 29, 2.0, 3, 0.0, 0.0, False, 2001),
    ("mg_p48_r3_d76_filter", 48, 3, 76, 35, 2.0, 3, 0.35, 0.2, True, 2002),
]


def class_inputs(P, R, D, seed, start):
    """gen_inputs' particles sorted by the class they were drawn from, the
    class means (quantised) as initial averages, optional start shifts."""
    parts, refs, _ = base.gen_inputs(P, R, D, seed, False)
    u = base._uniform(seed, R * 12 * 4 + P * 8 + P * D * D * 2 + 16)
    cls = np.array([int(u[R * 12 * 4 + 8 * p] * R) % R for p in range(P)])
    order = np.argsort(cls, kind="stable")
    parts, cls = np.ascontiguousarray(parts[order]), cls[order]
    if np.unique(cls).size != R:
        raise ValueError("a class is empty; pick another seed")
    avgs = base._q(np.stack([parts[cls == k].astype(np.float64).mean(0) for k in range(R)]))
    shifts = base._q((base._uniform(seed + 11, P * 2).reshape(P, 2) - 0.5) * 3.0) if start else None
    return parts, cls, avgs, shifts


def run_reference(lib, parts, cls, avgs, shifts, ring_num, rng, n_iter, cutoff, falloff, record=True):
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ref_free_alignment_2D_init.argtypes = [ctypes.POINTER(base.AlignConfig), ctypes.POINTER(fp),
                                               ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.ref_free_alignment_2D_init.restype = ctypes.c_ulonglong
    lib.ref_free_alignment_2D.argtypes = []
    lib.ref_free_alignment_2D.restype = None
    lib.ref_free_alignment_2D_filter_references.argtypes = [ctypes.c_float, ctypes.c_float]
    lib.ref_free_alignment_2D_filter_references.restype = None
    P, D = parts.shape[0], parts.shape[1]
    R = avgs.shape[0]
    cfg = base.AlignConfig(P, R, D, ring_num, 256, 1.0, rng, rng, b"multigroup_aln")
    sp = (fp * P)(*[parts[i].ctypes.data_as(fp) for i in range(P)])
    rp = (fp * R)(*[avgs[i].ctypes.data_as(fp) for i in range(R)])
    addr = lib.ref_free_alignment_2D_init(ctypes.byref(cfg), sp, rp, (ctypes.c_int * P)(*[int(c) for c in cls]), 0)
    prm = ctypes.cast(addr, ctypes.POINTER(base.AlignParam))
    for i in range(P):
        prm[i].shift_x = float(shifts[i, 0]) if shifts is not None else 0.0
        prm[i].shift_y = float(shifts[i, 1]) if shifts is not None else 0.0
    out = []
    for it in range(n_iter):
        if cutoff > 0.0:
            freq = 0.1 + (cutoff - 0.1) * it / float(n_iter - 1)
            lib.ref_free_alignment_2D_filter_references(freq, falloff)
        lib.ref_free_alignment_2D()
        if record:
            out.append([[prm[i].shift_x, prm[i].shift_y, prm[i].angle, float(prm[i].mirror)] for i in range(P)])
    lib.gpu_clear()
    return np.array(out, np.float32)


def time_stability_workload(lib, out_dir):
    """The reference's run time on bench.py's multigroup workload: the
    50,000 particles of the multi-reference workload sorted into classes of
    at most 100, class means as averages, 35 rings, shift range 1, 30
    iterations with the filter ramp 0.1 -> 0.3, fall-off 0.2."""
    import json
    import sys
    import time
    sys.path.insert(0, os.path.join(HERE, "..", "..", "gpu-isac_gb300"))
    from gpuisac import synth
    st = synth.workload_stack(1)
    order, cid = synth.stability_classes(st.cls, 100)
    parts = np.ascontiguousarray(st.particles[order])
    starts = np.flatnonzero(np.r_[True, cid[1:] != cid[:-1]])
    counts = np.diff(np.r_[starts, parts.shape[0]])
    avgs = np.ascontiguousarray((np.add.reduceat(parts.astype(np.float64), starts, axis=0) /
                                 counts[:, None, None]).astype(np.float32))
    times = []
    for _ in range(2):
        t = time.perf_counter()
        run_reference(lib, parts, cid, avgs, None, 35, 1.0, 30, 0.3, 0.2, record=False)
        times.append(time.perf_counter() - t)
    res = {"workload": "multigroup_50000x76_600classes_30it", "seconds_per_call": times,
           "particle_alignments_per_s": parts.shape[0] * 30 / min(times)}
    with open(os.path.join(out_dir, "ref_gpu_time_multigroup.json"), "w") as f:
        json.dump(res, f)
    print(json.dumps(res), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--build-dir", default=os.path.join(HERE, "..", "_build", "ref"))
    ap.add_argument("--time", action="store_true", help="only time bench.py's multigroup workload")
    a = ap.parse_args()
    lib = ctypes.CDLL(base.build_ref(a.ref_src, a.build_dir))
    if a.time:
        time_stability_workload(lib, a.out)
        return
    for name, P, R, D, NR, rng, n_iter, cutoff, falloff, start, seed in CASES:
        parts, cls, avgs, shifts = class_inputs(P, R, D, seed, start)
        params = run_reference(lib, parts, cls, avgs, shifts, NR, rng, n_iter, cutoff, falloff)
        np.savez_compressed(os.path.join(a.out, f"ref_{name}.npz"), params=params, seed=seed,
                            input_sum=np.float64(parts.astype(np.float64).sum() + avgs.astype(np.float64).sum()))
        print(name, "done", flush=True)


if __name__ == "__main__":
    main()
