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

METRIC = "particle x ref alignments/s (exhaustive: {S} shifts x 256 angles x 2 mirrors)"


def metric() -> str:
    return METRIC.format(S=WORKLOAD["n_shifts"])
UNIT = "alignments/s"
# the alignment workloads (one per --workload): plain exhaustive search
WORKLOADS = {
    "mref": dict(workload="mref_50000x76_200ref", particles=50000, refs=200, img_dim=76, rings=35, ring_len=256,
                 shift_range=3, shift_step=1.0, n_shifts=49, mirror=True, snr=0.05, blob_radius=34.0, seed_idx=1),
    "cpu2000": dict(workload="cpu_2000x64_16ref", particles=2000, refs=16, img_dim=64, rings=29, ring_len=256,
                    shift_range=2, shift_step=1.0, n_shifts=25, mirror=True, snr=0.1, blob_radius=28.0, seed_idx=0),
    "largebox": dict(workload="largebox_200000x128_500ref", particles=200000, refs=500, img_dim=128, rings=61,
                     ring_len=256, shift_range=4, shift_step=1.0, n_shifts=81, mirror=True, snr=0.03,
                     blob_radius=60.0, seed_idx=4),
}
WORKLOAD = WORKLOADS["mref"]
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


def fp32_nominal_tflops(sm_mhz: float = 2070.0) -> float:
    """nominal FP32 FMA rate of a GB300 (152 SMs x 128 FP32 lanes x 2 flops)"""
    return 152 * 128 * 2 * sm_mhz * 1e6 / 1e12


def fp32_measured_tflops(dev, n: int = 8192, reps: int = 6) -> float:
    """FP32 throughput of the CUDA cores measured on this GPU the way the
    bf16 peak is: a library GEMM (cuBLAS SGEMM, TF32 off), n^3 FMAs per call,
    timed with CUDA events after warm-up."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn((n, n), dtype=torch.float32, device=dev)
        b = torch.randn((n, n), dtype=torch.float32, device=dev)
        for _ in range(2):
            torch.mm(a, b)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        return 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) / 1000.0) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


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
    """(world, rank, local rank) of this process (gpuisac.replicas)."""
    from gpuisac import replicas
    return replicas.rank_env()


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
        sr = float(w["shift_range"])
        cfg = oracle.make_cfg(n, R, w["img_dim"], w["rings"], 256, 1.0, sr, sr)
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
    st = synth.make_stack(min(args.cpu_particles, WORKLOAD["particles"]), WORKLOAD["img_dim"], WORKLOAD["refs"],
                          WORKLOAD["shift_range"], WORKLOAD["snr"], WORKLOAD["blob_radius"],
                          synth.SEED_BASE + WORKLOAD["seed_idx"])
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = cpu_threads()
    R = st.refs.shape[0]
    w = WORKLOAD
    # size one step to ~args.step_seconds of CPU work
    rate, n_cal, t_cal, _ = cpu_oracle_rate(st.particles, st.refs, target_s=3.0, threads=threads)
    n = int(max(threads, min(st.particles.shape[0], rate * args.step_seconds / R)))
    sr = float(w["shift_range"])
    cfg = oracle.make_cfg(n, R, w["img_dim"], w["rings"], 256, 1.0, sr, sr)
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
    line = {"impl": "reference", "metric": metric(), "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantoms)",
            "config": dict(WORKLOAD, sample_particles=n, l2="cpu run"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


LEARNED = dict(workload="learned_100000x76_500ref", synth_idx=3, particles=100000, refs=500, train_alignments=200000,
               img_dim=76, rings=35, shift_range=3, n_shifts=49, snr=0.05, k=32, max_wrong=3e-3, nk=16)
# the same workload with the proposal as the workload text writes it: 64
# harmonics per ring, top-8 references (angles: see bench_learned)
LEARNED_AS_WRITTEN = dict(LEARNED, workload="learned_100000x76_500ref_as_written_64harm_top8", k=8, nk=64)
# the headline workload with the learned proposal in front: the chosen form
# (evaluation particles = the workload's own, training particles an
# independent draw of the same generator)
# (k = 16: 4.2x the plain search at 99.56 % same best with a 3e-3 margin
# calibration, against 3.1x at k = 32; the margin is calibrated to 2e-3 here
# to keep a wider distance from the 99.5 % bar)
LEARNED_MREF = dict(workload="learned_mref_50000x76_200ref", synth_idx=1, particles=None, refs=200,
                    train_alignments=50000, img_dim=76, rings=35, shift_range=3, n_shifts=49, snr=0.05, k=16,
                    max_wrong=2e-3)
# the large-box workload with the learned proposal in front (evaluation
# particles = the workload's own, training particles an independent draw)
LEARNED_LARGEBOX = dict(workload="largebox_learned_x128_500ref", synth_idx=4, particles=None, refs=500,
                        train_alignments=50000, img_dim=128, rings=61, shift_range=4, n_shifts=81, snr=0.03, k=32,
                        max_wrong=3e-3)


def fp64_check(L, parts, refs, NR, s, best_ref, best_peak):
    """The search's best reference and peak value per particle against the
    FP64 oracle's full search on the first particles of the same stack.  The
    oracle stacks only these particles, so the last one's texture neighbour
    differs from the full run's and it is left out.  Peak errors are relative
    to max(|d|, 1% of the Cauchy-Schwarz bound L^2 sum(r+1)); a peak below
    that is a near-total cancellation (see tests/test_gpu_configs.py)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    n, D, R = parts.shape[0], parts.shape[1], refs.shape[0]
    cfg = oracle.make_cfg(n, R, D, NR, 256, 1.0, s, s)
    lay = oracle.reference_layout(cfg)
    lay = oracle.OrcLayout(lay.sbj_batch, L.get_texture_limit(D), lay.ref_batch)
    t = time.perf_counter()
    _, od = oracle.multi_ref_align(cfg, lay, parts, refs, precision="f64", threads=cpu_threads())
    t = time.perf_counter() - t
    od = np.asarray(od, np.float64).reshape(R, n)[:, :n - 1]
    best_o = od.argmax(0)
    same = best_o == np.asarray(best_ref)[:n - 1]
    po = od[best_o, np.arange(n - 1)]
    floor = 0.01 * 256.0 * 256.0 * NR * (NR + 1) / 2.0
    err = np.abs(np.asarray(best_peak, np.float64)[:n - 1] - po) / np.maximum(np.abs(po), floor)
    return {"sample_particles": n - 1, "refs": R, "same_best_ref": float(same.mean()),
            "max_rel_peak_err_agreeing": float(err[same].max()) if same.any() else None,
            "oracle_seconds": t}


def bench_learned(args, dev, L, spec=None, resident=None):
    """The learned search against the plain FP32 full search on the learned
    workload: 100,000 held-out particles x 500 references, the network
    trained (untimed) on 200,000 particles the full search labelled.  Both
    timed with CUDA events on the same resident inputs; throughput counts
    particle x reference pairs covered (P x R) per second."""
    import torch

    from gpuisac import learned, synth
    from gpuisac.align import multi_ref_align_device
    w = spec or LEARNED
    if w["synth_idx"] == LEARNED["synth_idx"]:
        P, n_train = args.learned_particles, args.learned_train
    else:
        P, n_train = (w["particles"] or args.particles), (args.learned_train_largebox or w["train_alignments"])
    R, NR, s = w["refs"], w["rings"], float(w["shift_range"])
    t0 = time.perf_counter()
    tr = synth.workload_stack(w["synth_idx"], n_particles=n_train, n_refs=R, split=1)
    n_chk = min(args.fp64_sample, P)
    if resident is not None and resident[1].shape[0] == P:
        # the evaluation particles are the workload's own, already resident
        # (the same generator and seed)
        ev_np, ep, refs = resident
        chk_parts, chk_refs = ev_np.particles[:n_chk].copy(), ev_np.refs.copy()
    else:
        ev = synth.workload_stack(w["synth_idx"], n_particles=P, n_refs=R)
        ep = torch.from_numpy(ev.particles).to(dev)
        refs = torch.from_numpy(tr.refs).to(dev)
        chk_parts, chk_refs = ev.particles[:n_chk].copy(), tr.refs.copy()
        del ev
    t_gen = time.perf_counter() - t0
    tp = torch.from_numpy(tr.particles).to(dev)
    del tr
    t0 = time.perf_counter()
    d_tr, pk_tr = multi_ref_align_device(tp, refs, NR, s, s, contraction_mode="fp32")
    net = learned.ProposalNet(NR, nk=w.get("nk", learned.NK), device=dev, seed=11)
    rep = learned.train_from_full_search(net, tp, refs, d_tr, pk_tr, NR, s, s, k=w["k"], calib_frac=0.1,
                                         max_wrong=w["max_wrong"])
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del d_tr, pk_tr, tp
    stream = torch.cuda.current_stream(dev)

    def timed(fn, warm, steps):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1) / steps

    launches0 = L.gpuisac_launch_count()
    res, ms_l = timed(lambda: learned.learned_align(ep, refs, net, NR, s, s, k=w["k"], gap_margin=rep.gap_margin),
                      args.warmup, args.steps)
    launches = (L.gpuisac_launch_count() - launches0) // (args.warmup + args.steps)
    full_steps = max(1, min(args.steps, 3))
    (d_ev, pk_ev), ms_f = timed(lambda: multi_ref_align_device(ep, refs, NR, s, s, contraction_mode="fp32"), 1,
                                full_steps)
    d_ev = d_ev.cpu().numpy()
    lab = d_ev.argmax(0)
    r = res.ref.cpu().numpy()
    same = r == lab
    full_best = pk_ev.cpu().numpy()[lab, np.arange(P)]
    same_all = same & np.all(res.params.cpu().numpy() == full_best, axis=1)
    peak_err = np.abs(res.peak.cpu().numpy().astype(np.float64) - d_ev[lab, np.arange(P)]) / \
        np.maximum(np.abs(d_ev[lab, np.arange(P)]), 1e-30)
    fp64 = None
    if n_chk > 1 and not args.no_cpu:
        fp64 = fp64_check(L, chk_parts, chk_refs, NR, s, r[:n_chk], res.peak.cpu().numpy()[:n_chk])
    return {"workload": w["workload"], "value": P * R / (ms_l / 1000.0), "unit": UNIT,
            "vs_fp64_oracle": fp64,
            "ms_per_step": ms_l, "steps": args.steps, "warmup": args.warmup,
            "plain_fp32": {"value": P * R / (ms_f / 1000.0), "ms_per_step": ms_f, "steps": full_steps, "warmup": 1},
            "ratio_vs_plain_fp32": ms_f / ms_l,
            "same_best_ref": float(same.mean()), "same_ref_angle_shift_mirror": float(same_all.mean()),
            "max_rel_peak_err_vs_plain_fp32": float(peak_err.max()),
            "fallback_rate": float(res.fallback.float().mean().item()),
            "alignments_run_fraction": res.pairs / (P * R), "k": w["k"], "harmonics": net.nk,
            "gap_margin": rep.gap_margin,
            "calibration": {"recall_top_k": rep.recall, "fallback_rate": rep.fallback_rate,
                            "max_wrong": w["max_wrong"]},
            "train": {"particles": n_train, "seconds_incl_labelling": t_train, "loss_first_last":
                      [rep.loss[0], rep.loss[-1]], "epochs": len(rep.loss)},
            "gen_seconds": t_gen, "gpu_launches_per_step": launches,
            "dtype": ("f32 network (CUDA cores)" if os.environ.get("GPUISAC_NN_FP32", "0") not in ("", "0")
                      else "bf16 network inference (tcgen05 tensor cores, f32 accumulate; training f32)")
                     + ", f32 search"}


GROUPED = dict(workload="groups_400_loguniform_100_5000_x76_10to60ref", n_groups=400, min_size=100, max_size=5000,
               min_refs=10, max_refs=60, img_dim=76, rings=35, shift_range=3, n_shifts=49)


def bench_grouped(args, dev, L, parts_d, refs_d):
    """400 independent groups per call through gpuisac_multi_ref_align_groups_device
    (one texture fill, then a spectra and a CCF launch per wave, all reading
    device tables; the launch graph recorded once per shape), tile shape from
    the autotuner.  Group sizes are log-uniform in [100, 5000] particles with
    10..60 references each, cut from the 50,000-particle / 200-reference
    stacks already resident (groups may overlap in the pool; each is its own
    stack).  Two such group sets A and B alternate in the timed calls, so that
    every timed call has other groups than the call before it (its tables and
    texture objects are rebuilt; the recorded graph is replayed).  Also timed:
    the first call of the process (recording the graph), both sets as one
    call per group, and the plain path on the same work mix (one call,
    every particle of the pool against the groups' mean reference count)."""
    import torch

    from gpuisac.align import (ccf_tile_name, groups_stats, multi_ref_align_device,
                               multi_ref_align_groups_device)
    g = GROUPED
    P, R = parts_d.shape[0], refs_d.shape[0]
    NR, s = g["rings"], float(g["shift_range"])
    stream = torch.cuda.current_stream(dev)

    def make_groups(seed):
        rng = np.random.Generator(np.random.PCG64(seed))
        sizes = np.exp(rng.uniform(np.log(g["min_size"]), np.log(g["max_size"]), g["n_groups"])).astype(int)
        nrefs = rng.integers(g["min_refs"], g["max_refs"] + 1, g["n_groups"])
        out = []
        for n, r in zip(sizes, nrefs):
            out.append((int(rng.integers(0, P - n + 1)), int(n), int(rng.integers(0, R - r + 1)), int(r)))
        return out

    sets = [make_groups(20261203 + 2), make_groups(20261203 + 3)]
    work = [int(sum(n * r for _, n, _, r in gs)) for gs in sets]

    def run(i):
        return multi_ref_align_groups_device(parts_d, refs_d, sets[i], NR, s, s)

    # the first call of the process for this shape records the graph
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first = run(0)
    torch.cuda.synchronize()
    first_ms = (time.perf_counter() - t0) * 1000.0
    first_stats = groups_stats()
    outs = [first, None]
    for _ in range(max(args.warmup, 3)):
        for i in (1, 0):
            outs[i] = run(i)
    torch.cuda.synchronize()
    steps = max(args.steps, 2)
    launches0 = L.gpuisac_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    done = 0
    recorded = 0
    plan_ms = []
    for k in range(steps):
        i = (k + 1) % 2  # B, A, B, ...: each call's groups differ from the previous call's
        outs[i] = run(i)
        st_k = groups_stats()
        recorded += int(st_k["graph_recorded"])
        plan_ms.append(st_k["plan_ms"])
        done += work[i]
    e1.record(stream)
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1000.0
    ms_g = e0.elapsed_time(e1) / steps
    launches = (L.gpuisac_launch_count() - launches0) / steps
    stats = groups_stats()

    def sequential(i):
        return [multi_ref_align_device(parts_d[so:so + n], refs_d[ro:ro + r], NR, s, s, contraction_mode="fp32")
                for so, n, ro, r in sets[i]]

    same, seq_ms = [], []
    for i in (0, 1):
        torch.cuda.synchronize()
        e0.record(stream)
        seq = sequential(i)
        e1.record(stream)
        torch.cuda.synchronize()
        seq_ms.append(e0.elapsed_time(e1))
        dg, pg, offs = outs[i]
        dg_h, pg_h = dg.cpu().numpy(), pg.cpu().numpy()
        n_same = 0
        for (so, n, ro, r), off, (d1, p1) in zip(sets[i], offs, seq):
            n_same += int(np.array_equal(dg_h[off:off + n * r].reshape(r, n), d1.cpu().numpy()) and
                          np.array_equal(pg_h[off:off + n * r].reshape(r, n, 4), p1.cpu().numpy()))
        same.append(n_same)
        del seq

    # the plain path on the same work mix: every particle of the pool against
    # the groups' mean reference count (one call)
    r_mix = int(round(sum(work) / sum(sum(n for _, n, _, _ in gs) for gs in sets)))
    for _ in range(2):
        multi_ref_align_device(parts_d, refs_d[:r_mix], NR, s, s, contraction_mode="fp32")
    torch.cuda.synchronize()
    e0.record(stream)
    multi_ref_align_device(parts_d, refs_d[:r_mix], NR, s, s, contraction_mode="fp32")
    e1.record(stream)
    torch.cuda.synchronize()
    mix_ms = e0.elapsed_time(e1)
    value = done / (ms_g * steps / 1000.0)
    return {"workload": g["workload"], "value": value, "unit": UNIT, "ms_per_step": ms_g,
            "steps": steps, "warmup": max(args.warmup, 3),
            "alignments_per_step": done / steps, "particles_per_call": [int(sum(n for _, n, _, _ in gs)) for gs in sets],
            "timed_calls": "group sets A and B alternate: every call has other groups than the call before it",
            "host_wall_ms_per_step": wall_ms / steps,
            "plan_ms_per_call": float(np.mean(plan_ms)), "graphs_recorded_in_timed_calls": recorded,
            "first_call": {"ms": first_ms, "record_ms": first_stats["record_ms"], "plan_ms": first_stats["plan_ms"],
                           "note": "first call of the process: allocations, texture layout, graph recording"},
            "waves": stats["waves"], "launches_per_call": launches, "graph_launches": stats["graph_launches"],
            "sequential_per_group_calls": {"value": sum(work) / (sum(seq_ms) / 1000.0), "ms": seq_ms},
            "groups_identical_to_sequential": f"{sum(same)}/{2 * len(sets[0])}",
            "plain_same_mix": {"value": P * r_mix / (mix_ms / 1000.0), "ms": mix_ms, "particles": P, "refs": r_mix,
                               "note": "one plain call, all pool particles x the groups' mean reference count"},
            "tile": ccf_tile_name(NR, g["n_shifts"]),
            "data": "groups cut from the resident 50k-particle / 200-ref synthetic stacks"}


GROUPED_LARGEBOX = dict(workload="largebox_groups_loguniform_500_20000_x128_500ref", min_size=500, max_size=20000,
                        rings=61, shift_range=4, n_shifts=81, checked_groups=3)


def bench_grouped_largebox(args, dev, L, parts_d, refs_d):
    """The large-box stack cut into consecutive groups of log-uniform size in
    [500, 20000] particles (the last group takes the rest), every group
    against all references, in one gpuisac_multi_ref_align_groups_device call
    per step; a few groups compared bit for bit with their own separate
    calls."""
    import torch

    from gpuisac.align import groups_stats, multi_ref_align_device, multi_ref_align_groups_device
    g = GROUPED_LARGEBOX
    P, R = parts_d.shape[0], refs_d.shape[0]
    NR, s = g["rings"], float(g["shift_range"])
    rng = np.random.Generator(np.random.PCG64(20261203 + 4 + 2))
    groups, a = [], 0
    while a < P:
        n = int(np.exp(rng.uniform(np.log(g["min_size"]), np.log(g["max_size"]))))
        n = min(n, P - a)
        groups.append((a, n, 0, R))
        a += n
    stream = torch.cuda.current_stream(dev)
    out = multi_ref_align_groups_device(parts_d, refs_d, groups, NR, s, s)  # first call: records the graph
    first = groups_stats()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 2))
    e0.record(stream)
    for _ in range(steps):
        out = multi_ref_align_groups_device(parts_d, refs_d, groups, NR, s, s)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    stats = groups_stats()
    d, pk, offs = out
    same = 0
    pick = rng.choice(len(groups), size=min(g["checked_groups"], len(groups)), replace=False)
    for i in pick:
        so, n, ro, r = groups[i]
        d1, p1 = multi_ref_align_device(parts_d[so:so + n], refs_d[ro:ro + r], NR, s, s, contraction_mode="fp32")
        off = offs[i]
        same += int(torch.equal(d[off:off + n * r].view(r, n), d1) and
                    torch.equal(pk[off:off + n * r].view(r, n, 4), p1))
    del out, d, pk
    torch.cuda.empty_cache()
    return {"workload": g["workload"], "value": P * R / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms,
            "steps": steps, "groups": len(groups), "particles": P, "refs_per_group": R,
            "waves": stats["waves"], "graph_launches": stats["graph_launches"],
            "first_call_record_ms": first["record_ms"], "plan_ms": stats["plan_ms"],
            "groups_identical_to_separate_calls": f"{same}/{len(pick)} (sampled)",
            "contraction": "fp32 (the grouped launch sequence runs the FP32 CCF kernels)"}


def bench_assign(args, dev, L, d_dev, cpu=True):
    """The equal-size group assignment ISAC runs on the alignment's peak matrix
    (gpuisac_assign_groups_device; EMAN2's Util::assign_groups on the host in
    the reference) on d_dev [R][P] already in HBM, L2 flushed before every
    timed call; the host-buffer C-ABI call with d copied in and the list
    copied out; the oracle's CPU restatement on the same d; and the
    list compared with the oracle's."""
    import torch

    from gpuisac.assign import assign_groups_device
    R, P = d_dev.shape
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)       # 256 MB > L2
    ids = torch.empty(P + 1, dtype=torch.int32, device=dev)
    bel = torch.empty(P, dtype=torch.int32, device=dev)
    rounds = ctypes.c_uint()

    def call():
        rc = L.gpuisac_assign_groups_device(d_dev.data_ptr(), P, R, P, bel.data_ptr(), ids.data_ptr(),
                                            ctypes.byref(rounds), stream.cuda_stream)
        if rc:
            _lib_check(L)

    for _ in range(max(args.warmup, 3)):
        call()
    total = 0.0
    steps = max(args.steps, 3)
    launches0 = L.gpuisac_launch_count()
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    launches = (L.gpuisac_launch_count() - launches0) / steps
    ms = total / steps
    hbm_peak, _, peak_kind = peaks()
    alg_bytes = 4.0 * R * P + 4.0 * P + 4.0 * (P + 1)
    blk = {"workload": f"{P} particles x {R} groups", "ms_per_call": ms, "pairs_per_s": R * P / (ms / 1000.0),
           "rounds": rounds.value, "kernel_launches_per_call": launches,
           "roofline": {"bound": "hbm", "achieved": alg_bytes / (ms / 1000.0) / 1e9, "peak": hbm_peak,
                        "unit": "GB/s", "frac": alg_bytes / (ms / 1000.0) / 1e9 / hbm_peak,
                        "algorithmic_bytes": alg_bytes, "peak_kind": peak_kind},
           "l2": "256 MB buffer written before each timed call"}
    d_host = d_dev.cpu().numpy()
    out = np.zeros(P + 1, np.int32)
    t0 = time.perf_counter()
    rc = L.gpuisac_assign_groups(d_host.ctypes.data, R, P, out.ctypes.data)
    if rc:
        _lib_check(L)
    t_host = time.perf_counter() - t0
    blk["e2e"] = {"ms_per_call": 1000.0 * t_host, "h2d_bytes": 4 * R * P, "d2h_bytes": 4 * (P + 1),
                  "api": "gpuisac_assign_groups (host d, host list)"}
    blk["identical_to_device_call"] = bool(np.array_equal(out, ids.cpu().numpy()))
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        t0 = time.perf_counter()
        want = oracle.assign_groups(d_host, R, P)
        t_cpu = time.perf_counter() - t0
        blk["cpu_baseline"] = {"ms_per_call": 1000.0 * t_cpu, "cores": 1, "kind": "port",
                               "sample": "the whole call (std::sort of the pairs + the serial greedy)"}
        blk["identical_to_oracle"] = bool(np.array_equal(want, out))
    del flush
    return blk


AVERAGES = {"fl": 0.2, "ff": 0.2, "sample_groups": 2}


def bench_averages(args, dev, L, parts_d, d_dev, peak_dev, cpu=True):
    """The averaging step after the group assignment (gpuisac_class_averages:
    rot_shift2D of every particle by its group's pair parameters, group sums,
    mean shifts, re-centred parameters, filt_tanl + fshift of each average)
    on the alignment's own peaks and the assignment's groups, all in HBM, L2
    flushed before every timed call; the host-array call; the FP64 oracle on
    the members of sampled groups (parity and the CPU baseline)."""
    import torch

    from gpuisac.assign import assign_groups_device
    from gpuisac.averages import class_averages, class_averages_device
    R, P = d_dev.shape
    D = parts_d.shape[1]
    fl, ff = AVERAGES["fl"], AVERAGES["ff"]
    _, bel, _ = assign_groups_device(d_dev, with_id_list=False)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)       # 256 MB > L2

    def call():
        return class_averages_device(parts_d, peak_dev, bel, fl, ff, True, stream=stream)

    for _ in range(max(args.warmup, 3)):
        out = call()
    total = 0.0
    steps = max(args.steps, 3)
    launches0 = L.gpuisac_launch_count()
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out2 = call()
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    launches = (L.gpuisac_launch_count() - launches0) / steps
    ms = total / steps
    hbm_peak, _, peak_kind = peaks()
    alg_bytes = 4.0 * P * D * D + 4.0 * R * D * D + 16.0 * P + 4.0 * P + 16.0 * P
    avg, params, members, shifts = (t.cpu().numpy() for t in out)
    blk = {"workload": f"{P} particles ({D}^2) x {R} groups from the assignment on this run's peaks; rot_shift2D "
                       f"(quadratic, background), sums, mean shifts, re-centred parameters, filt_tanl({fl}, {ff}) "
                       "and fshift by minus the mean shift",
           "ms_per_call": ms, "particles_per_s": P / (ms / 1000.0), "kernel_launches_per_call": launches,
           "roofline": {"bound": "issue (the interpolation: about 80 instructions per output pixel and member)",
                        "hbm_achieved": alg_bytes / (ms / 1000.0) / 1e9, "hbm_peak": hbm_peak, "unit": "GB/s",
                        "hbm_frac": alg_bytes / (ms / 1000.0) / 1e9 / hbm_peak, "algorithmic_bytes": alg_bytes,
                        "peak_kind": peak_kind},
           "repeat_identical": all(np.array_equal(a.cpu().numpy(), b.cpu().numpy()) for a, b in zip(out, out2)),
           "l2": "256 MB buffer written before each timed call; the 1.2 GB stack exceeds L2"}
    parts_h, pk_h, bel_h = parts_d.cpu().numpy(), peak_dev.cpu().numpy(), bel.cpu().numpy()
    t0 = time.perf_counter()
    class_averages(parts_h, pk_h, bel_h, fl, ff, True)
    t_host = time.perf_counter() - t0
    blk["e2e"] = {"ms_per_call": 1000.0 * t_host, "h2d_bytes": parts_h.nbytes + pk_h.nbytes + bel_h.nbytes,
                  "d2h_bytes": avg.nbytes + params.nbytes + members.nbytes + shifts.nbytes,
                  "api": "gpuisac.averages.class_averages (host arrays in and out)"}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        groups = np.unique(bel_h)[:AVERAGES["sample_groups"]]
        idx = np.flatnonzero(np.isin(bel_h, groups))
        remap = np.searchsorted(groups, bel_h[idx])
        t0 = time.perf_counter()
        a_o, p_o, m_o, s_o = oracle.class_averages(parts_h[idx], pk_h[groups][:, idx], remap, fl, ff, True)
        t_cpu = time.perf_counter() - t0
        err = float(np.abs(avg[groups] - a_o).max() / max(np.abs(a_o).max(), 1e-6))
        blk["vs_fp64_oracle"] = {"groups": int(groups.size), "particles": int(idx.size),
                                 "max_rel_average_err": err,
                                 "max_param_err": float(np.abs(params[idx] - p_o).max()),
                                 "members_equal": bool(np.array_equal(members[groups], m_o)),
                                 "meets_bar": err < 2e-5 and float(np.abs(params[idx] - p_o).max()) < 2e-6}
        blk["cpu_baseline"] = {"particles_per_s": idx.size / t_cpu, "cores": 1, "kind": "port",
                               "sample": f"the {idx.size} members of {groups.size} groups, FP64 numpy restatement, "
                                         f"{t_cpu:.1f} s"}
    del flush
    return blk


MULTIGROUP = {"workload": "stability-test multigroup alignment: the 50,000 particles (76^2) sorted into classes of "
                          "at most 100 (each true class split into runs), 35 rings, shift range 1 (9 shifts), "
                          "30 iterations with the tangent filter ramp 0.1 -> 0.3, fall-off 0.2 (ISAC's defaults "
                          "maxit=30, FH=0.3, FF=0.2)",
              "class_size": 100, "rings": 35, "shift_range": 1.0, "iterations": 30, "cutoff": 0.3, "falloff": 0.2}


def bench_multigroup(args, dev, L, st):
    """One multigroup_refinement call (ref_free_alignment_2D_init, 30 x
    (_filter_references + ref_free_alignment_2D), gpu_clear) as ISAC's
    stability test makes it per repeat; value = particle alignments (one
    particle against its class average over the shift grid, with the
    averaging) per second over the iterations, e2e including the init's
    upload of the particles and averages.  CPU baseline: one oracle iteration
    (FP32 alignment with OpenMP, transform + average, filter) on 20 classes."""
    import torch

    from gpuisac import _lib
    from gpuisac._lib import AlignParam
    from gpuisac.align import make_config, ptr_array
    from gpuisac import synth
    m = MULTIGROUP
    order, cid = synth.stability_classes(st.cls, m["class_size"])
    parts = np.ascontiguousarray(st.particles[order])
    P, D = parts.shape[0], parts.shape[1]
    R = int(cid[-1]) + 1
    starts = np.flatnonzero(np.r_[True, cid[1:] != cid[:-1]])
    counts = np.diff(np.r_[starts, P])
    avgs = np.ascontiguousarray((np.add.reduceat(parts.astype(np.float64), starts, axis=0) /
                                 counts[:, None, None]).astype(np.float32))
    NR, sr, n_it = m["rings"], float(m["shift_range"]), m["iterations"]
    cfg = make_config(P, R, D, NR, 256, 1.0, sr, sr, b"multigroup_aln")
    cids = (ctypes.c_int * P)(*[int(c) for c in cid])
    sp, rp = ptr_array(parts), ptr_array(avgs)

    def call():
        t0 = time.perf_counter()
        addr = L.ref_free_alignment_2D_init(ctypes.byref(cfg), sp, rp, cids, torch.cuda.current_device())
        if not addr:
            _lib_check(L)
        t_init = time.perf_counter() - t0
        prm = ctypes.cast(addr, ctypes.POINTER(AlignParam))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(n_it):
            L.ref_free_alignment_2D_filter_references(ctypes.c_float(0.1 + (m["cutoff"] - 0.1) * i / (n_it - 1)),
                                                      ctypes.c_float(m["falloff"]))
            L.ref_free_alignment_2D()
        e1.record()
        torch.cuda.synchronize()
        _lib.check(L)
        # the results are in the host AlignParam array when the last call returns
        t_all = time.perf_counter() - t0
        assert prm[P - 1].ref_id == int(cid[-1])
        L.gpu_clear()
        return e0.elapsed_time(e1), t_all, t_init

    for _ in range(max(1, args.warmup - 2)):
        call()
    launches0 = L.gpuisac_launch_count()
    runs = [call() for _ in range(max(2, min(args.steps, 3)))]
    launches = (L.gpuisac_launch_count() - launches0) / len(runs)
    ms = statistics.mean(r[0] for r in runs)
    e2e_s = statistics.mean(r[1] for r in runs)
    blk = {"workload": m["workload"], "classes": R, "particles": P,
           "value": P * n_it / (ms / 1000.0), "unit": "particle alignments/s",
           "ms_per_call": ms, "ms_per_iteration": ms / n_it, "calls": len(runs),
           "kernel_launches_per_call": launches,
           "e2e": {"value": P * n_it / e2e_s, "unit": "particle alignments/s", "ms_per_call": 1000.0 * e2e_s,
                   "init_ms": 1000.0 * statistics.mean(r[2] for r in runs),
                   "h2d_bytes_per_call": int((P + R) * D * D * 4), "api": "ref_free_alignment_2D_* (host images)"}}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        n_cls = 20
        sub = [(int(starts[j]), int(counts[j])) for j in range(n_cls)]
        t0 = time.perf_counter()
        filt = oracle.tanl_filter_averages(avgs[:n_cls], 0.2, m["falloff"]).astype(np.float32)
        n_parts = 0
        prms, mirs, sub_parts, sub_cid = [], [], [], []
        for j, (a, n) in enumerate(sub):
            ccfg = oracle.make_cfg(n, 1, D, NR, 256, 1.0, sr, sr)
            lay = oracle.reference_layout(ccfg)
            pk, _ = oracle.multi_ref_align(ccfg, lay, parts[a:a + n], filt[j:j + 1], precision="f32")
            pk = np.asarray(pk).reshape(n, 4)
            prms.append(pk[:, :3])
            mirs.append(pk[:, 3] != 0)
            sub_parts.append(parts[a:a + n])
            sub_cid += [j] * n
            n_parts += n
        oracle.multigroup_averages(np.concatenate(sub_parts), np.concatenate(prms), np.concatenate(mirs), sub_cid,
                                   65000 // D)
        t_cpu = time.perf_counter() - t0
        blk["cpu_baseline"] = {"value": n_parts / t_cpu, "unit": "particle alignments/s", "cores": cpu_threads(),
                               "kind": "port",
                               "sample": f"one iteration on {n_cls} classes ({n_parts} particles): filter, FP32 "
                                         f"alignment (OpenMP), transform + average, {t_cpu:.1f} s"}
    return blk


PREALIGN = {"workload": "pre-alignment: the 50,000 particles (76^2) against their mean, 35 rings, shift range 5 "
                        "step 1 (121 shifts), one batch",
            "rings": 35, "shift_range": 5.0, "shift_step": 1.0, "runs": 2}


def bench_prealign(args, dev, L, st):
    """pre_align_init, the particles fetched once, then per run the average
    fetched and pre_align_run over all particles (ISAC's pre-alignment
    iteration on one batch); value = particles aligned per second of run."""
    import torch

    from gpuisac import _lib
    from gpuisac.align import make_config, ptr_array
    m = PREALIGN
    parts = np.ascontiguousarray(st.particles)
    P, D = parts.shape[0], parts.shape[1]
    avg = np.ascontiguousarray(parts.astype(np.float64).mean(0, keepdims=True).astype(np.float32))
    cfg = make_config(P, 1, D, m["rings"], 256, m["shift_step"], m["shift_range"], m["shift_range"], b"pre_aln")
    n_shift = L.gpuisac_shift_count(ctypes.byref(cfg))
    t0 = time.perf_counter()
    if not L.pre_align_init(P, ctypes.byref(cfg), torch.cuda.current_device()):
        _lib_check(L)
    L.pre_align_fetch(ptr_array(parts), P, b"sbj_batch")
    _lib.check(L)
    t_setup = time.perf_counter() - t0
    runs = []
    try:
        for i in range(1 + m["runs"]):           # the first run is warm-up
            t = time.perf_counter()
            L.pre_align_fetch(ptr_array(avg), 1, b"ref_batch")
            L.pre_align_run(0, P)
            _lib.check(L)
            if i:
                runs.append(time.perf_counter() - t)
    finally:
        L.gpu_clear()
    s_run = statistics.mean(runs)
    blk = {"workload": m["workload"], "particles": P, "shifts": n_shift,
           "value": P / s_run, "unit": "particles aligned/s (121 shifts x 256 angles x 2 mirrors, one reference)",
           "ms_per_run": 1000.0 * s_run, "runs": len(runs), "init_and_particle_fetch_ms": 1000.0 * t_setup}
    ref_t = os.path.join(ROOT, "tests", "golden", "ref_gpu_time_prealign.json")
    if os.path.exists(ref_t):
        r = json.load(open(ref_t))
        # stored, not measured in this run: the reference's own library timed
        # once on a GB300 of this pool by the fixture script
        blk["reference_library_ms_per_run_stored"] = 1000.0 * min(r["seconds_per_run"])
        blk["reference_library_source"] = "stored: tests/golden/ref_gpu_time_prealign.json"
    return blk


def _lib_check(L):
    from gpuisac import _lib
    _lib.check(L)
    raise RuntimeError("library call failed")


# the parity bar of the tests (tests/test_gpu_align.py, test_gpu_configs.py)
PEAK_RTOL, SAME_BEST, SAME_PAIR, ANGLE_TOL = 1e-4, 0.995, 0.99, 0.05


def precision_vs_fp64(dev, n=256, R=200):
    """Peak values and peak parameters of both contractions against the FP64
    oracle on a stack of the headline workload's shape (the same stack on
    both), with the tests' bar: every peak within 1e-4 relative of the
    oracle's -- relative to max(|d|, 1% of the Cauchy-Schwarz bound L^2
    sum(r+1)), a smaller peak being a near-total cancellation -- the same best
    (reference, angle, sx, sy, mirror) on >= 99.5% of particles, >= 99% of all
    (reference, particle) tuples the same."""
    import torch

    from gpuisac import synth
    from gpuisac.align import multi_ref_align_device
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    w = WORKLOAD
    R = min(R, w["refs"])
    sr = float(w["shift_range"])
    NR = w["rings"]
    st = synth.make_stack(n, w["img_dim"], R, w["shift_range"], w["snr"], w["blob_radius"],
                          synth.SEED_BASE + w["seed_idx"])
    cfg = oracle.make_cfg(n, R, w["img_dim"], NR, 256, 1.0, sr, sr)
    lay = oracle.reference_layout(cfg)
    t = time.perf_counter()
    po, od = oracle.multi_ref_align(cfg, lay, st.particles, st.refs, precision="f64", threads=cpu_threads())
    t = time.perf_counter() - t
    od = np.asarray(od, np.float64).reshape(R, n)
    po = np.asarray(po)
    floor = 0.01 * 256.0 * 256.0 * NR * (NR + 1) / 2.0
    out = {"sample": f"{n} particles x {R} refs, {w['workload']} shape", "oracle_seconds": t,
           "bar": {"peak_rtol": PEAK_RTOL, "near_zero_floor": "1% of L^2 sum(r+1)", "same_best": SAME_BEST,
                   "same_tuples": SAME_PAIR, "angle_tol_deg": ANGLE_TOL}}
    ok_all = True
    for mode in ("fp32", "bf16x3"):
        d, pk = multi_ref_align_device(torch.from_numpy(st.particles).to(dev), torch.from_numpy(st.refs).to(dev),
                                       NR, sr, sr, contraction_mode=mode)
        d, pk = d.cpu().numpy().astype(np.float64), pk.cpu().numpy()
        rel = np.abs(d - od) / np.maximum(np.abs(od), floor)
        ang = np.abs(pk[..., 0].astype(np.float64) - po[..., 0]) % 360.0
        ang = np.minimum(ang, 360.0 - ang)
        same_t = (pk[..., 1:] == po[..., 1:]).all(-1) & (ang < ANGLE_TOL)
        qg, qo = d.argmax(0), od.argmax(0)
        best = (qg == qo) & same_t[qo, np.arange(n)]
        ok = bool(rel.max() <= PEAK_RTOL and best.mean() >= SAME_BEST and same_t.mean() >= SAME_PAIR)
        ok_all = ok_all and ok
        out[mode] = {"max_rel_peak_err": float(rel.max()), "median_rel_peak_err": float(np.median(rel)),
                     "same_best_tuple": float(best.mean()), "same_tuples": float(same_t.mean()),
                     "near_zero_peaks": int((np.abs(od) < floor).sum()), "meets_bar": ok}
    out["meets_bar"] = ok_all
    return out


def spectra_roofline(w, P, steps, spec_ms, spec_launches, hbm_peak, peak_kind, out_bytes_per_row):
    """resample + FFT stage: images read once per shift row, spectra (or
    operands) written"""
    S = w["n_shifts"]
    spec_avg_ms = spec_ms / max(spec_launches, 1)
    spec_bytes = (P * w["img_dim"] ** 2 * 4 * S + P * S * out_bytes_per_row) * steps / max(spec_launches, 1)
    return {"avg_launch_ms": spec_avg_ms, "bytes_per_launch": spec_bytes,
            "achieved_gbs": spec_bytes / (spec_avg_ms / 1000.0) / 1e9 if spec_avg_ms else None,
            "hbm_peak_gbs": hbm_peak, "hbm_peak_kind": peak_kind}


def fp32_roofline(dev, w, P, R, steps, ccf_ms, ccf_launches, spec_ms, spec_launches, hbm_peak, bf16_peak, peak_kind):
    """The fused FP32 CCF / inverse-FFT / peak kernel: algorithmic contraction
    FLOPs per launch over its average launch time, against the FP32 rate of
    the CUDA cores (the plain path's ceiling), measured here with cuBLAS SGEMM
    as the bf16 peak is measured with a bf16 GEMM; the nominal FMA rate (152
    SMs x 128 lanes x 2 flops x max SM clock) and the bf16 tensor peak beside
    it.  Traffic: the 3,000-particle ncu capture's DRAM bytes per alignment
    (profiles/ccf_peak_traffic.txt) scaled to a launch."""
    S = w["n_shifts"]
    alignments = P * R
    flops_per_alignment = 8.0 * S * (w["ring_len"] // 2 + 1) * w["rings"]
    flops_per_launch = flops_per_alignment * alignments * steps / max(ccf_launches, 1)
    ccf_avg_ms = ccf_ms / max(ccf_launches, 1)
    achieved_tflops = flops_per_launch / (ccf_avg_ms / 1000.0) / 1e12
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "ccf_peak_traffic.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_particle_ref:"):
                traffic = float(ln.split(":")[1]) * alignments * steps / max(ccf_launches, 1)
    fp32_nominal = fp32_nominal_tflops()
    fp32_peak = fp32_measured_tflops(dev)
    return {"bound": "fp32-fma", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": achieved_tflops / fp32_peak, "traffic": traffic, "kernel": "ccf_peak",
            "peak_kind": "measured: cuBLAS SGEMM (TF32 off, CUDA cores) on this GPU, 8192^3",
            "fp32_nominal_peak": fp32_nominal, "frac_of_fp32_nominal": achieved_tflops / fp32_nominal,
            "flops_per_launch": flops_per_launch, "avg_launch_ms": ccf_avg_ms,
            "kernel_share": ccf_ms / max(ccf_ms + spec_ms, 1e-9),
            "frac_of_bf16_tensor_peak": achieved_tflops / bf16_peak, "bf16_peak": bf16_peak,
            "bf16_peak_kind": peak_kind,
            "spectra": spectra_roofline(w, P, steps, spec_ms, spec_launches, hbm_peak, peak_kind,
                                        w["rings"] * 128 * 8)}


def split_roofline(L, w, P, R, steps, split_ms, spec_ms, spec_launches, hbm_peak, bf16_peak, peak_kind):
    """The tensor-core contraction's two kernels.  Both move the pair spectra
    Z (2 KB per (particle x shift, reference) pair) through HBM, so both are
    HBM-bound: algorithmic bytes per launch = Z written (ccf_mma_kernel, plus
    the subject operands it reads) or Z read (zfft_peak_kernel, plus d and
    peak_list written), over the average launch time, against the measured
    copy bandwidth.  The MMA kernel's tensor-pipe work is reported beside it:
    3 BF16 products x 2 x 128 x N x 16 FLOPs per tcgen05.mma, and the
    algorithmic contraction FLOPs 8 S (L/2+1) N_r per alignment."""
    from gpuisac.align import split_plan
    S, NR = w["n_shifts"], w["rings"]
    pl = split_plan(NR, S, R)
    alignments = P * R
    z_bytes = float(P) * R * S * 2048
    sop_bytes = float(P) * pl["n_blocks"] * 128 * 2 * pl["kg"] * pl["rga"] * 128
    out_bytes = float(P) * R * 20
    ks = (pl["kg"] + (pl["kg"] & 1)) // 2
    mma_flops = float(P) * pl["n_blocks"] * pl["n_rtiles"] * 128 * ks * 3 * 2 * 128 * pl["n_cols"] * 16
    alg_flops = 8.0 * S * (w["ring_len"] // 2 + 1) * NR * alignments
    kern = {}
    for name, byts in (("ccf_mma", z_bytes + sop_bytes), ("zfft_peak", z_bytes + out_bytes)):
        k = split_ms[name]
        launches = max(k["launches"] // max(steps, 1), 1)
        avg_ms = k["ms_per_step"] / launches
        per_launch = byts / launches
        kern[name] = {"avg_launch_ms": avg_ms, "launches_per_step": launches, "bytes_per_launch": per_launch,
                      "achieved_gbs": per_launch / (avg_ms / 1000.0) / 1e9, "ms_per_step": k["ms_per_step"]}
    mma_s = split_ms["ccf_mma"]["ms_per_step"] / 1000.0
    kern["ccf_mma"]["tensor"] = {
        "mma_flops_per_step": mma_flops, "achieved_tflops": mma_flops / mma_s / 1e12,
        "frac_of_bf16_peak": mma_flops / mma_s / 1e12 / bf16_peak, "bf16_peak": bf16_peak,
        "algorithmic_flops_per_step": alg_flops, "algorithmic_tflops": alg_flops / mma_s / 1e12}
    dom = max(kern, key=lambda n: kern[n]["ms_per_step"])
    d = kern[dom]
    traffic = None
    tfile = os.path.join(ROOT, "profiles", f"{dom}_traffic.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_pair:"):
                traffic = float(ln.split(":")[1]) * alignments * S / d["launches_per_step"]
    total_ms = sum(k["ms_per_step"] for k in kern.values()) + spec_ms / max(steps, 1)
    return {"bound": "hbm", "achieved": d["achieved_gbs"], "peak": hbm_peak, "unit": "GB/s",
            "frac": d["achieved_gbs"] / hbm_peak, "traffic": traffic, "kernel": dom, "peak_kind": peak_kind,
            "avg_launch_ms": d["avg_launch_ms"], "kernel_share": d["ms_per_step"] / max(total_ms, 1e-9),
            "plan": pl, "kernels": kern,
            "spectra": spectra_roofline(w, P, steps, spec_ms, spec_launches, hbm_peak, peak_kind,
                                        2 * 2 * 2 * pl["kg"] * 8 * 128)}


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
    st = synth.make_stack(P, w["img_dim"], w["refs"], w["shift_range"], w["snr"], w["blob_radius"],
                          synth.SEED_BASE + w["seed_idx"] + 1000 * rank)
    sr = float(w["shift_range"])
    R = st.refs.shape[0]
    parts_d = torch.from_numpy(st.particles).to(dev)
    refs_d = torch.from_numpy(st.refs).to(dev)
    base_d = torch.zeros((P, 2), dtype=torch.float32, device=dev)
    d_out = torch.empty((R, P), dtype=torch.float32, device=dev)
    peak_out = torch.empty((R, P, 4), dtype=torch.float32, device=dev)
    cfg = make_config(P, R, w["img_dim"], w["rings"], 256, 1.0, sr, sr)
    stream = torch.cuda.Stream(dev)
    from gpuisac.align import CONTRACTIONS
    L.gpuisac_set_contraction(CONTRACTIONS[args.contraction])

    def step():
        rc = L.gpuisac_multi_ref_align_device(ctypes.byref(cfg), parts_d.data_ptr(), refs_d.data_ptr(),
                                              base_d.data_ptr(), d_out.data_ptr(), peak_out.data_ptr(),
                                              stream.cuda_stream)
        if rc:
            _lib.check(L)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # tile shape of the CCF launches: the autotuner times the candidates on a
    # sample of this workload (setup, untimed)
    from gpuisac.align import autotune_ccf
    tune = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        tune_report = autotune_ccf(parts_d, refs_d, w["rings"], sr, sr, n_sample=2048, stream=stream)
        tune = {"seconds": time.perf_counter() - t0, "report": tune_report}

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
    split_ms = {}
    for kname in ("ccf_mma", "zfft_peak"):
        L.gpuisac_kernel_time(kname.encode(), ctypes.byref(n_l), ctypes.byref(t_l))
        split_ms[kname] = {"launches": n_l.value, "ms_per_step": t_l.value / args.steps}
    L.gpuisac_profile(0)
    if world > 1:
        from gpuisac import replicas
        ms_total = replicas.max_over_ranks(ms_total, device=dev)
    ms_step = ms_total / args.steps
    alignments = P * R
    value = world * alignments / (ms_step / 1000.0)

    # ---- roofline of the CCF / IFFT / peak kernel ----
    hbm_peak, bf16_peak, peak_kind = peaks()
    S = w["n_shifts"]
    flops_per_alignment = 8.0 * S * (w["ring_len"] // 2 + 1) * w["rings"]
    if args.contraction == "bf16x3":
        roofline = split_roofline(L, w, P, R, args.steps, split_ms, spec_ms, spec_launches, hbm_peak, bf16_peak,
                                  peak_kind)
    else:
        roofline = fp32_roofline(dev, w, P, R, args.steps, ccf_ms, ccf_launches, spec_ms, spec_launches, hbm_peak,
                                 bf16_peak, peak_kind)

    # ---- the plain FP32 form on the same resident stacks, timed the same way ----
    plain = None
    if args.contraction != "fp32" and args.plain_steps > 0:
        L.gpuisac_set_contraction(CONTRACTIONS["fp32"])
        step()
        torch.cuda.synchronize()
        L.gpuisac_profile(1)
        barrier()
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.plain_steps):
            step()
        p1.record(stream)
        torch.cuda.synchronize()
        barrier()
        pms = p0.elapsed_time(p1)
        if world > 1:
            from gpuisac import replicas
            pms = replicas.max_over_ranks(pms, device=dev)
        L.gpuisac_kernel_time(b"ccf_peak", ctypes.byref(n_l), ctypes.byref(t_l))
        p_ccf_launches, p_ccf_ms = n_l.value, t_l.value
        L.gpuisac_kernel_time(b"polar_spectra", ctypes.byref(n_l), ctypes.byref(t_l))
        p_spec_launches, p_spec_ms = n_l.value, t_l.value
        L.gpuisac_profile(0)
        L.gpuisac_set_contraction(CONTRACTIONS[args.contraction])
        pms /= args.plain_steps
        plain = {"value": world * alignments / (pms / 1000.0), "unit": UNIT, "ms_per_step": pms,
                 "steps": args.plain_steps, "warmup": 1,
                 "roofline": fp32_roofline(dev, w, P, R, args.plain_steps, p_ccf_ms, p_ccf_launches, p_spec_ms,
                                           p_spec_launches, hbm_peak, bf16_peak, peak_kind)}


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
            from gpuisac import replicas
            e2e_s = replicas.max_over_ranks(e2e_s, device=dev)
        h2d = (P + R) * w["img_dim"] ** 2 * 4 + P * 8
        d2h = R * P * 4 + R * P * 16
        e2e = {"value": world * alignments / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * e2e_s, "steps": args.e2e_steps,
               "host_to_device": "the caller's images copied through pinned staging buffers filled by host "
                                 "threads (DMA of one buffer overlapping the fill of the next); results copied "
                                 "back per chunk while the next chunk computes"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, n, t, thr = cpu_oracle_rate(st.particles, st.refs, target_s=args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{n} particles x {R} refs of the same workload, {t:.1f} s (FP32 oracle, OpenMP)"}

    # ---- the chosen form: the learned proposal in front of the exhaustive
    # search, on the same particles, against the plain FP32 full search ----
    chosen = None
    if rank == 0 and world == 1 and not args.no_learned and WORKLOAD["workload"].startswith("mref"):
        blk = bench_learned(args, dev, L, LEARNED_MREF, resident=(st, parts_d, refs_d))
        chosen = {"form": f"learned reference proposal (network inference on the tensor cores, top-{LEARNED_MREF['k']} "
                          "references) + exhaustive shift x angle x mirror search of every proposal, full search of "
                          "every reference below the calibrated margin",
                  "value": blk["value"], "unit": UNIT, "ms_per_step": blk["ms_per_step"],
                  "ratio_vs_plain_fp32": blk["ratio_vs_plain_fp32"], "plain_fp32": blk["plain_fp32"],
                  "vs_fp64_oracle": blk["vs_fp64_oracle"],
                  "same_best_ref_vs_plain_fp32": blk["same_best_ref"],
                  "same_ref_angle_shift_mirror_vs_plain_fp32": blk["same_ref_angle_shift_mirror"],
                  "fallback_rate": blk["fallback_rate"], "alignments_run_fraction": blk["alignments_run_fraction"],
                  "detail": blk}

    prec = learned_blk = grouped_blk = assign_blk = None
    learned_spec = LEARNED_LARGEBOX if WORKLOAD["workload"].startswith("largebox") else None
    if rank == 0 and world == 1 and not args.no_assign:
        assign_blk = {"on_alignment_peaks": bench_assign(args, dev, L, d_out, cpu=not args.no_cpu)}
        rng = torch.Generator(device=dev)
        rng.manual_seed(20261203 + 5)
        big = torch.rand((500, 100000), generator=rng, device=dev) * 0.1 + 0.5
        cls = torch.randint(0, 500, (100000,), generator=rng, device=dev)
        big[cls, torch.arange(100000, device=dev)] += 0.3 * torch.rand(100000, generator=rng, device=dev)
        assign_blk["synthetic_100000x500"] = bench_assign(args, dev, L, big, cpu=False)
        del big
    averages_blk = None
    if rank == 0 and world == 1 and not args.no_averages:
        averages_blk = bench_averages(args, dev, L, parts_d, d_out, peak_out, cpu=not args.no_cpu)
    multigroup_blk = prealign_blk = None
    if rank == 0 and world == 1 and not args.no_multigroup and WORKLOAD["workload"].startswith("mref"):
        multigroup_blk = bench_multigroup(args, dev, L, st)
    if rank == 0 and world == 1 and not args.no_prealign and WORKLOAD["workload"].startswith("mref"):
        prealign_blk = bench_prealign(args, dev, L, st)
    if rank == 0 and world == 1 and not args.no_grouped:
        del d_out, peak_out
        torch.cuda.empty_cache()
        grouped_blk = bench_grouped(args, dev, L, parts_d, refs_d)
    if rank == 0 and world == 1 and not args.no_cpu:
        prec = precision_vs_fp64(dev, n=256 if WORKLOAD["workload"].startswith("mref") else 32)
    if rank == 0 and world == 1 and WORKLOAD["workload"].startswith("largebox") and not args.no_grouped_largebox:
        grouped_blk = bench_grouped_largebox(args, dev, L, parts_d, refs_d)
    if rank == 0 and world == 1 and not args.no_learned:
        if learned_spec is None:
            del parts_d
            torch.cuda.empty_cache()
            learned_blk = bench_learned(args, dev, L, learned_spec)
        else:
            learned_blk = bench_learned(args, dev, L, learned_spec, resident=(st, parts_d, refs_d))
        if learned_spec is None and not args.no_learned_as_written:
            torch.cuda.empty_cache()
            aw = bench_learned(args, dev, L, LEARNED_AS_WRITTEN)
            aw["coarse_angles"] = ("not proposed: one inverse FFT gives every one of the 256 angles of a "
                                   "(shift, reference) pair, so the search of each proposed reference covers "
                                   "the top-16 coarse angles and their neighbourhoods at no extra cost")
            learned_blk = {"chosen_16harm_top32": learned_blk, "as_written_64harm_top8": aw}

    if rank == 0:
        dtype = "bf16x3 (BF16 hi/lo split operands, FP32 accumulate)" if args.contraction == "bf16x3" else "f32"
        line = {"metric": metric(), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype, "data": f"synthetic (seeded phantoms, {P} particles/GPU)",
                "chosen": chosen, "plain_fp32": plain,
                "config": dict(WORKLOAD, particles=P, autotune=tune,
                               path="plain FP32 CUDA-core contraction" if args.contraction == "fp32" else
                               "BF16 hi/lo split contraction on the tensor cores (tcgen05), pair spectra through HBM",
                               l2=f"inputs ({P * w['img_dim'] ** 2 * 4 / 1e9:.2f} GB images, spectra or operand "
                                  "chunks of GBs) exceed the 129 MB L2"),
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
                "split_kernels": split_ms if args.contraction == "bf16x3" else None,
                "precision_vs_fp64": prec, "grouped": grouped_blk, "learned": learned_blk,
                "assign_groups": assign_blk, "averages": averages_blk, "multigroup": multigroup_blk,
                "prealign": prealign_blk}
        print(json.dumps(line), flush=True)
        if prec is not None and not prec["meets_bar"]:
            sys.stderr.write("precision_vs_fp64: the parity bar is not met\n")
            sys.exit(3)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="mref",
                    help="mref: 50,000 x 76^2 vs 200 refs (default); cpu2000: 2,000 x 64^2 vs 16; "
                         "largebox: 128^2 particles vs 500 refs, 61 rings, 81 shifts")
    ap.add_argument("--particles", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-particles", type=int, default=4000)
    ap.add_argument("--step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-search comparison")
    ap.add_argument("--no-grouped", action="store_true", help="skip the grouped-launch comparison")
    ap.add_argument("--no-grouped-largebox", action="store_true",
                    help="largebox: skip the batched uneven groups over the whole stack")
    ap.add_argument("--no-learned-as-written", action="store_true",
                    help="skip the learned proposal as the workload writes it (64 harmonics, top-8)")
    ap.add_argument("--no-assign", action="store_true", help="skip the group-assignment block")
    ap.add_argument("--no-averages", action="store_true", help="skip the averaging-step block")
    ap.add_argument("--no-multigroup", action="store_true", help="skip the multigroup (stability test) block")
    ap.add_argument("--no-prealign", action="store_true", help="skip the pre-alignment block")
    ap.add_argument("--no-autotune", action="store_true", help="default tile shape (profiling runs)")
    ap.add_argument("--plain-steps", type=int, default=3,
                    help="timed steps of the plain FP32 form beside the headline (0: skip)")
    ap.add_argument("--fp64-sample", type=int, default=64,
                    help="particles of the chosen form checked against the FP64 oracle")
    ap.add_argument("--contraction", choices=["fp32", "bf16x3"], default="bf16x3",
                    help="ring-summed contraction of the timed search: fp32 (CUDA cores) or bf16x3 "
                         "(BF16 hi/lo split on the tensor cores)")
    ap.add_argument("--learned-particles", type=int, default=LEARNED["particles"])
    ap.add_argument("--learned-train", type=int, default=LEARNED["train_alignments"])
    ap.add_argument("--learned-train-largebox", type=int, default=None)
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = WORKLOADS[args.workload]
    if args.particles is None:
        args.particles = WORKLOAD["particles"]
    if args.workload != "mref":
        # the grouped and learned blocks are defined on the 76^2 workloads
        args.no_grouped = True
        args.no_learned = args.no_learned or args.workload == "cpu2000"
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
