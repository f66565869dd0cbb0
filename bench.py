#!/usr/bin/env python3
"""Benchmark of the multi-reference 2D alignment (GPU-ISAC's hot path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: 50,000 synthetic 76x76 float32 particles from 200 seeded phantom
classes against 200 references, rings 1..35, shifts +/-3 step 1 (49 shifts),
mirror on.  One step = one exhaustive search of every particle against every
reference (1.0e7 alignments).  Prints one JSON line (rank 0).

  value    alignments/s, inputs resident in HBM (device C-ABI entry point),
           CUDA events on the library's stream
  e2e      alignments/s through the reference-facing C-ABI (multi_ref_align
           with host image pointers): host->device copies of the images and
           device->host copies of d / peak_list inside every timed step
  roofline the CCF/IFFT/peak kernel: algorithmic contraction FLOPs per launch
           over its average launch time (CUDA events in the timed region)
  cpu_baseline  the CPU oracle (FP32 restatement of the reference's
           arithmetic) on all host cores, on a bounded particle sample

Multi-GPU (torchrun): each rank aligns its own stack on its own GPU (weak
scaling, no collective on the data path); value = all ranks' alignments over
the slowest rank's time.

--impl reference: the reference's CPU path for this workload (the CPU
oracle port; the reference's own CPU implementation lives in the un-vendored
EMAN2 library) on the host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gpu-isac_gb300"))

import numpy as np  # noqa: E402

METRIC = "particle x ref alignments/s (exhaustive: 49 shifts x 256 angles x 2 mirrors)"
UNIT = "alignments/s"
WORKLOAD = dict(workload="mref_50000x76_200ref", particles=50000, refs=200, img_dim=76, rings=35,
                ring_len=256, shift_range=3, shift_step=1.0, n_shifts=49, mirror=True, snr=0.05)
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            j = json.load(open(p))
            hbm = j.get("hbm_gbs") or j.get("hbm_GBs")
            bf16 = j.get("bf16_tflops")
            if hbm and bf16:
                return float(hbm), float(bf16), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, FALLBACK_BF16_TFLOPS, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_oracle_rate(parts, refs, target_s=15.0, threads=None):
    """alignments/s of the CPU oracle (FP32, reference arithmetic) on a sample
    of particles sized to take about target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or cpu_threads()
    R = refs.shape[0]
    w = WORKLOAD

    def run(n):
        cfg = oracle.make_cfg(n, R, w["img_dim"], w["rings"], 256, 1.0, 3.0, 3.0)
        lay = oracle.reference_layout(cfg)
        t = time.perf_counter()
        oracle.multi_ref_align(cfg, lay, parts[:n], refs, precision="f32", threads=threads)
        return time.perf_counter() - t

    n0 = max(threads, 4)
    t0 = run(n0)
    n = int(min(parts.shape[0], max(n0, n0 * target_s / max(t0, 1e-3))))
    n = max(threads, n // threads * threads)
    t = run(n)
    return n * R / t, n, t, threads


def bench_reference(args):
    world, rank, local = dist_setup(args.gpus)
    if rank != 0:
        return
    from gpuisac import synth
    st = synth.make_stack(args.cpu_particles, WORKLOAD["img_dim"], WORKLOAD["refs"], WORKLOAD["shift_range"],
                          WORKLOAD["snr"], 34.0, synth.SEED_BASE + 1)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = cpu_threads()
    R = st.refs.shape[0]
    w = WORKLOAD
    # size one step to ~args.step_seconds of CPU work
    rate, n_cal, t_cal, _ = cpu_oracle_rate(st.particles, st.refs, target_s=3.0, threads=threads)
    n = int(max(threads, min(st.particles.shape[0], rate * args.step_seconds / R)))
    cfg = oracle.make_cfg(n, R, w["img_dim"], w["rings"], 256, 1.0, 3.0, 3.0)
    lay = oracle.reference_layout(cfg)
    times = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        oracle.multi_ref_align(cfg, lay, st.particles[:n], st.refs, precision="f32", threads=threads)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.mean(times)
    value = n * R / (ms / 1000.0)
    sample = f"{n} of {w['particles']} particles x {R} refs per step (FP32 oracle port, OpenMP)"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantoms)",
            "config": dict(WORKLOAD, sample_particles=n, l2="cpu run"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def bench_ours(args):
    import torch

    world, rank, local = dist_setup(args.gpus)
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    from gpuisac import _lib, multi_ref_align, synth
    from gpuisac.align import make_config, ptr_array
    L = _lib.load()
    w = WORKLOAD
    P = args.particles
    st = synth.make_stack(P, w["img_dim"], w["refs"], w["shift_range"], w["snr"], 34.0,
                          synth.SEED_BASE + 1 + 1000 * rank)
    R = st.refs.shape[0]
    parts_d = torch.from_numpy(st.particles).to(dev)
    refs_d = torch.from_numpy(st.refs).to(dev)
    base_d = torch.zeros((P, 2), dtype=torch.float32, device=dev)
    d_out = torch.empty((R, P), dtype=torch.float32, device=dev)
    peak_out = torch.empty((R, P, 4), dtype=torch.float32, device=dev)
    cfg = make_config(P, R, w["img_dim"], w["rings"], 256, 1.0, 3.0, 3.0)
    stream = torch.cuda.Stream(dev)

    def step():
        rc = L.gpuisac_multi_ref_align_device(ctypes.byref(cfg), parts_d.data_ptr(), refs_d.data_ptr(),
                                              base_d.data_ptr(), d_out.data_ptr(), peak_out.data_ptr(),
                                              stream.cuda_stream)
        if rc:
            _lib.check(L)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    clocks = ClockSampler(local)
    L.gpuisac_profile(1)
    launches0 = L.gpuisac_launch_count()
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = L.gpuisac_launch_count() - launches0
    ms_total = ev0.elapsed_time(ev1)
    n_l, t_l = ctypes.c_ulonglong(), ctypes.c_double()
    L.gpuisac_kernel_time(b"ccf_peak", ctypes.byref(n_l), ctypes.byref(t_l))
    ccf_launches, ccf_ms = n_l.value, t_l.value
    L.gpuisac_kernel_time(b"polar_spectra", ctypes.byref(n_l), ctypes.byref(t_l))
    spec_launches, spec_ms = n_l.value, t_l.value
    L.gpuisac_profile(0)
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps
    alignments = P * R
    value = world * alignments / (ms_step / 1000.0)

    # ---- roofline of the CCF / IFFT / peak kernel ----
    hbm_peak, bf16_peak, peak_kind = peaks()
    S = w["n_shifts"]
    flops_per_alignment = 8.0 * S * (w["ring_len"] // 2 + 1) * w["rings"]
    flops_per_launch = flops_per_alignment * alignments * args.steps / max(ccf_launches, 1)
    ccf_avg_ms = ccf_ms / max(ccf_launches, 1)
    achieved_tflops = flops_per_launch / (ccf_avg_ms / 1000.0) / 1e12
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "ccf_peak_traffic.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_particle_ref:"):
                traffic = float(ln.split(":")[1]) * alignments * args.steps / max(ccf_launches, 1)
    roofline = {"bound": "tensor", "achieved": achieved_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved_tflops / bf16_peak, "traffic": traffic, "kernel": "ccf_peak",
                "peak_kind": f"bf16 dense, {peak_kind}",
                "flops_per_launch": flops_per_launch, "avg_launch_ms": ccf_avg_ms,
                "kernel_share": ccf_ms / max(ccf_ms + spec_ms, 1e-9),
                "spectra_avg_launch_ms": spec_ms / max(spec_launches, 1)}

    # ---- end to end through the reference-facing C-ABI ----
    e2e = None
    if args.e2e_steps > 0:
        sp, rp = ptr_array(st.particles), ptr_array(st.refs)
        pl = np.zeros((R, 4 * P), np.float32)
        dh = np.zeros((R, P), np.float32)
        times = []
        for i in range(args.e2e_warmup + args.e2e_steps):
            barrier()
            t0 = time.perf_counter()
            params = L.multi_ref_align_init(ctypes.byref(cfg), torch.cuda.current_device())
            if not params:
                _lib.check(L)
            L.multi_ref_align(sp, rp, pl.ctypes.data_as(_lib.float_ptr), dh.ctypes.data_as(_lib.float_ptr), P,
                              ctypes.c_float(0.9))
            _lib.check(L)
            L.gpu_clear()
            dt = time.perf_counter() - t0
            if i >= args.e2e_warmup:
                times.append(dt)
        e2e_s = statistics.mean(times)
        if world > 1:
            t = torch.tensor([e2e_s], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = (P + R) * w["img_dim"] ** 2 * 4 + P * 8
        d2h = R * P * 4 + R * P * 16
        e2e = {"value": world * alignments / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * e2e_s, "steps": args.e2e_steps,
               "host_to_device": "pinned staging of the caller's image pointers"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, n, t, thr = cpu_oracle_rate(st.particles, st.refs, target_s=args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{n} particles x {R} refs of the same workload, {t:.1f} s (FP32 oracle, OpenMP)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantoms, 50k particles/GPU)",
                "config": dict(WORKLOAD, path="plain FP32 CUDA-core contraction",
                               l2="inputs (1.16 GB images, spectra chunks of GBs) exceed the 129 MB L2"),
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--particles", type=int, default=WORKLOAD["particles"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-particles", type=int, default=4000)
    ap.add_argument("--step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
