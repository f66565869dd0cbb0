#!/usr/bin/env python3
"""Golden outputs of the reference's own GPU library for the multi-reference
alignment, and its run time on the 50,000 x 200 workload.

    python tests/golden/make_ref_golden.py --ref-src DIR [--out DIR] [--time]

DIR is the reference repository root (its cuda/ sources).  The library is
built from those sources with oracle/build_ref.sh's command line (no source
edits) and called exactly as bin/sp_isac2_gpu.py:959-1006 calls it:
multi_ref_align_init -> fill AlignParam shifts -> multi_ref_align -> gpu_clear.
Needs a CUDA GPU.  Inputs come from gen_inputs() below (integer hashing and
values quantised to 1/4096, so every machine regenerates them bit for bit);
only parameters and outputs are stored.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (name, P, R, D, ring_num, shift range, step, fractional base shifts?)
CASES = [
    ("mref_p40_r8_d64", 40, 8, 64, 29, 2.0, 1.0, False),
    ("mref_p24_r6_d76_base", 24, 6, 76, 35, 3.0, 1.0, True),
    ("mref_p20_r5_d32_edge", 20, 5, 32, 20, 2.0, 1.0, False),
    ("mref_p10_r130_d34_refbatch", 10, 130, 34, 17, 1.0, 1.0, False),
]


def _mix(x):
    """splitmix64 on uint64 arrays"""
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def _uniform(seed: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = _mix(np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(1_000_003))
    return (x >> np.uint64(11)).astype(np.float64) / float(1 << 53)


def _q(a):
    """quantise to multiples of 1/4096 (exactly representable, platform independent)"""
    return (np.round(np.asarray(a, np.float64) * 4096.0) / 4096.0).astype(np.float32)


def gen_inputs(P: int, R: int, D: int, seed: int, base: bool):
    """Blob phantoms (references) and rotated / shifted / noisy copies (particles)."""
    u = _uniform(seed, R * 12 * 4 + P * 8 + P * D * D * 2 + 16)
    i = 0
    refs = np.zeros((R, D, D))
    c = np.arange(D) - D // 2
    X, Y = np.meshgrid(c, c)
    blobs = []
    for q in range(R):
        bl = []
        for b in range(8):
            rad = 0.4 * D * np.sqrt(u[i]); th = 2 * np.pi * u[i + 1]
            sig = 1.5 + 0.08 * D * u[i + 2]; amp = 0.5 + 0.5 * u[i + 3]
            i += 4
            bl.append((rad * np.cos(th), rad * np.sin(th), sig, amp))
            refs[q] += amp * np.exp(-((X - bl[-1][0]) ** 2 + (Y - bl[-1][1]) ** 2) / (2 * sig * sig))
        blobs.append(bl)
    i = R * 12 * 4
    parts = np.zeros((P, D, D))
    for p in range(P):
        q = int(u[i] * R) % R; ang = 2 * np.pi * u[i + 1]
        dx = int(u[i + 2] * 5) - 2; dy = int(u[i + 3] * 5) - 2; mir = u[i + 4] < 0.5
        i += 8
        for (bx, by, sig, amp) in blobs[q]:
            bx = -bx if mir else bx
            rx = np.cos(ang) * bx - np.sin(ang) * by + dx
            ry = np.sin(ang) * bx + np.cos(ang) * by + dy
            parts[p] += amp * np.exp(-((X - rx) ** 2 + (Y - ry) ** 2) / (2 * sig * sig))
    n = u[R * 12 * 4 + P * 8: R * 12 * 4 + P * 8 + P * D * D * 2].reshape(P, D, D, 2)
    noise = np.sqrt(-2 * np.log(np.maximum(n[..., 0], 1e-12))) * np.cos(2 * np.pi * n[..., 1])
    parts = parts + 0.3 * noise
    bs = None
    if base:
        bs = _q((_uniform(seed + 7, P * 2).reshape(P, 2) - 0.5) * 3.0)
    return _q(parts), _q(refs), bs


def build_ref(ref_src: str, out_dir: str) -> str:
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "gpu_aln_pack.so")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++11", "-shared", "-Xcompiler",
           "-fPIC", "-DCUFFT_PARSE_ERROR=1001", "-DCUFFT_LICENSE_ERROR=1002",
           "-DCUFFT_INCOMPLETE_PARAMETER_LIST=1003", "-DkernelExecTimeoutEnabled=integrated",
           "-I", os.path.join(ref_src, "cuda"), os.path.join(ref_src, "cuda", "gpu_aln_common.cu"),
           os.path.join(ref_src, "cuda", "gpu_aln_noref.cu"), "-o", so, "-lcufft", "-lcublas"]
    subprocess.run(cmd, check=True, capture_output=True)
    return so


class AlignConfig(ctypes.Structure):
    _fields_ = [("sbj_num", ctypes.c_uint), ("ref_num", ctypes.c_uint), ("img_dim", ctypes.c_uint),
                ("ring_num", ctypes.c_uint), ("ring_len", ctypes.c_uint), ("shift_step", ctypes.c_float),
                ("shift_rng_x", ctypes.c_float), ("shift_rng_y", ctypes.c_float), ("aln_type", ctypes.c_char_p)]


class AlignParam(ctypes.Structure):
    _fields_ = [("sbj_id", ctypes.c_int), ("ref_id", ctypes.c_int), ("shift_x", ctypes.c_float),
                ("shift_y", ctypes.c_float), ("angle", ctypes.c_float), ("mirror", ctypes.c_bool)]


def run_reference(lib, parts, refs, ring_num, rng, step, base):
    """the reference driver's call sequence (bin/sp_isac2_gpu.py:959-1006)"""
    fp = ctypes.POINTER(ctypes.c_float)
    lib.multi_ref_align_init.argtypes = [ctypes.POINTER(AlignConfig), ctypes.c_uint]
    lib.multi_ref_align_init.restype = ctypes.POINTER(AlignParam)
    lib.multi_ref_align.argtypes = [ctypes.POINTER(fp), ctypes.POINTER(fp), fp, fp, ctypes.c_uint, ctypes.c_float]
    lib.multi_ref_align.restype = None
    P, D = parts.shape[0], parts.shape[1]
    R = refs.shape[0]
    cfg = AlignConfig(P, R, D, ring_num, 256, step, rng, rng, b"mref_aln")
    prm = lib.multi_ref_align_init(ctypes.byref(cfg), 0)
    for i in range(P):
        prm[i].shift_x = float(base[i, 0]) if base is not None else 0.0
        prm[i].shift_y = float(base[i, 1]) if base is not None else 0.0
    sp = (fp * P)(*[parts[i].ctypes.data_as(fp) for i in range(P)])
    rp = (fp * R)(*[refs[i].ctypes.data_as(fp) for i in range(R)])
    peak = np.zeros((R, 4 * P), np.float32)
    d = np.zeros((R, P), np.float32)
    t = time.perf_counter()
    lib.multi_ref_align(sp, rp, peak.ctypes.data_as(fp), d.ctypes.data_as(fp), P, 0.9)
    dt = time.perf_counter() - t
    lib.gpu_clear()
    return peak.reshape(R, P, 4), d, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--build-dir", default=os.path.join(HERE, "..", "_build", "ref"))
    ap.add_argument("--time", action="store_true", help="also time the 50,000 x 200 workload")
    a = ap.parse_args()
    lib = ctypes.CDLL(build_ref(a.ref_src, a.build_dir))
    os.makedirs(a.out, exist_ok=True)
    for k, (name, P, R, D, NR, rng, step, base) in enumerate(CASES):
        parts, refs, bs = gen_inputs(P, R, D, 1000 + k, base)
        peak, d, _ = run_reference(lib, parts, refs, NR, rng, step, bs)
        np.savez_compressed(os.path.join(a.out, f"ref_{name}.npz"), P=P, R=R, D=D, ring_num=NR, rng=rng, step=step,
                            seed=1000 + k, base=base, d=d, peak=peak,
                            input_sum=np.float64(parts.astype(np.float64).sum() + refs.astype(np.float64).sum()))
        print(name, "done", flush=True)
    if a.time:
        sys.path.insert(0, os.path.join(HERE, "..", "..", "gpu-isac_gb300"))
        from gpuisac import synth
        st = synth.workload_stack(1)
        times = []
        for _ in range(2):
            _, _, dt = run_reference(lib, st.particles, st.refs, 35, 3.0, 1.0, None)
            times.append(dt)
        res = {"workload": "mref_50000x76_200ref", "seconds": times,
               "alignments_per_s": 50000 * 200 / min(times)}
        with open(os.path.join(a.out, "ref_gpu_time.json"), "w") as f:
            json.dump(res, f)
        print(json.dumps(res))


if __name__ == "__main__":
    main()
