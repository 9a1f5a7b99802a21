#!/usr/bin/env python3
"""Throughput of the GB300 pair-counting engine, one JSON line on stdout.

Default workload ("mocks256"): 256 periodic Neyman-Scott boxes (Poisson(100)
children per parent, Gaussian offsets sigma = 5 Mpc/h) with N log-uniform in
[1e4, 1e6] and box side (N / 2.5e-4)^(1/3); FCFC refuses the boxes with
s_max >= L / 2 (26 of them), the other 230 (5.5e7 points) are counted in
one persistent launch per step: unweighted DD in (s, mu), s in [0, 200)
Mpc/h in 40 bins, 100 mu bins.  The metric is unique in-range pairs per
second (pairs that land in a bin, i < j).

  value   -- FP32 + FP64-recheck path, catalogues already in HBM; a step is
             the batched count (rescale, cell sort, count, recheck), timed
             with CUDA events, the device idle on both sides; L2 is flushed
             between steps.
  e2e     -- the same step from pinned host arrays through the C ABI: the
             catalogues' transfer and the counts' read-back are inside.
  fp64    -- the all-FP64 GPU path on every accepted mock (one pass), with
             a check that its counts equal the FP32 path's.
  cpu_baseline -- the CPU restatement of FCFC's counter (oracle/: FCFC's FP64
             per-pair formula on a cell grid, OpenMP on every host core) on
             every 64th accepted mock; cpu_sample_on_gpu is the GPU on the
             same mocks.
--impl reference times that CPU restatement on the same sample mocks, each
step one pass over them.

Other workloads (--workload): ns_box_2e6 (one weighted 2e6-point box in
(s, mu) and (s_perp, pi)), survey (DD/DR/RR of 1e6 data and 1e7 randoms),
adjoint (dL/dw of a Landy-Szalay loss), cli (the command line drivers end
to end on an ASCII catalogue).
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "in-range pairs/s on 1 GB300: FP32+FP64-recheck vs all-FP64, exact counts"
UNIT = "pairs/s"
BOX = 2000.0
LOGBINS = np.geomspace(0.1, 100.0, 41)
FLOPS_PER_PAIR = {"smu": 10, "spi": 8}   # algorithmic FP32 flops per pair


def nvtx(name):
    """An NVTX range (profilers can restrict a capture to it: the timed
    steps are "timed", the all-FP64 passes "fp64")."""
    import contextlib
    try:
        import torch
        return torch.cuda.nvtx.range(name)
    except Exception:
        return contextlib.nullcontext()


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def workload(box=BOX, nparent=20000, seed=1):
    from fcfc_gb300 import synth
    x = synth.neyman_scott(nparent, box, 100.0, 5.0, seed=seed)
    w = synth.lognormal_weights(len(x), 0.3, seed=seed + 1)
    return x, w


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def fp32_peak_tflops(dev):
    """Measured FP32 (non-tensor) throughput: cuBLAS SGEMM with TF32 off."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev, dtype=torch.float32)
    b = torch.randn(n, n, device=dev, dtype=torch.float32)
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def profile_value(key, name="k_count32_box_smu_wt_ns_box.txt"):
    """A figure of a committed ncu summary (DRAM bytes per launch, warp
    instructions per in-range pair), if present; by default the summary of
    the box workload's dominant kernel."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def profile_traffic():
    return profile_value("traffic_bytes_per_launch_full_workload")


def issue_bound(pairs_per_s, clocks, name="k_count32_box_smu_wt_ns_box.txt"):
    """The bound the count kernel actually meets: instruction issue.  Warp
    instructions per in-range pair (ncu, committed summary) x pairs/s over
    the issue rate of the GPU (SMs x 4 schedulers x the SM clock sampled
    during the run)."""
    ipp = profile_value("warp_instructions_per_in_range_pair", name)
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    if ipp is None:
        return None
    peak = 152 * 4 * mhz * 1e6
    ach = pairs_per_s * ipp
    return {"achieved": ach, "peak": peak, "unit": "warp instructions/s",
            "frac": ach / peak, "warp_instructions_per_pair": ipp,
            "source": "ncu instruction count of the small case x measured "
                      "pairs/s; peak = 152 SMs x 4 issue slots x SM clock"}


def max_over_ranks(value, dist):
    """Step time of the slowest rank (replicas run independent jobs)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def run_reference_mocks(args, rank, world):
    """CPU restatement of FCFC's counter on the sample mocks of the batched
    workload (every 64th accepted mock), every host core."""
    from fcfc_gb300 import synth
    _, boxes = synth.mock_boxes(256, seed=7, sizes_only=True)
    acc = [j for j, L in enumerate(boxes) if 2 * MOCK_SMAX < L]
    subset = acc[::MOCK_CPU_STRIDE]
    cats = {j: synth.mock_boxes(j + 1, seed=7, first=j)[0][0] for j in subset}
    val, pairs, ms, desc = mocks_cpu_sample(cats, boxes, subset,
                                            steps=args.steps,
                                            warmup=args.warmup)
    out = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": mocks_config(256, boxes),
        "impl": "reference",
        "cpu_baseline": {"value": val, "unit": UNIT,
                         "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": desc},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def run_reference(args, rank, world):
    """CPU restatement of FCFC's counter on a bounded sample of the workload."""
    if rank != 0:
        return 0
    if args.workload == "mocks256":
        return run_reference_mocks(args, rank, world)
    from oracle import fcfc_oracle as fo
    box = 1200.0   # same density: 2e4 * (1200/2000)^3 parents
    x, w = workload(box=box, nparent=int(round(20000 * (box / BOX) ** 3)), seed=1)
    b1 = fo.Bins(False, 1, ns=40, smin=0, ds=5, nmu=100, box=box)
    b2 = fo.Bins(False, 2, ns=40, sedges=LOGBINS, np_=40, pmin=0, dpi=1, box=box)
    nthr = os.cpu_count() or 1

    def step():
        t0 = time.perf_counter()
        c1 = b1.count(x, wa=w, mode=3)
        c2 = b2.count(x, wa=w, mode=3)
        return time.perf_counter() - t0, c1, c2

    # unweighted in-range count once (weighted sums are not pair numbers)
    n_in = int(b1.count(x, mode=3).sum() + b2.count(x, mode=3).sum())
    for _ in range(args.warmup):
        step()
    tt = 0.0
    for _ in range(args.steps):
        dt, _, _ = step()
        tt += dt
    val = n_in * args.steps / tt
    sample = ("Neyman-Scott box L=%g Mpc/h, %d points (same density as the "
              "2e6-point workload), weighted DD (s,mu)+(s_perp,pi), %d pairs "
              "per step" % (box, len(x), n_in))
    out = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "ns_box_2e6 (bounded CPU sample)", "box": box,
                   "n_points": len(x), "bins": "smu 40x100 + spi 40x40"},
        "impl": "reference",
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": nthr,
                         "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def mocks_workload(nmock=256, seed=7):
    """Neyman-Scott boxes (the generator of the clustered-box workload:
    Poisson(100) children, sigma = 5 Mpc/h), N log-uniform in [1e4, 1e6],
    box side (N / 2.5e-4)^(1/3)."""
    from fcfc_gb300 import synth
    return synth.mock_boxes(nmock, seed=seed)


MOCK_SMAX = 200.0
MOCK_CPU_STRIDE = 64     # the CPU sample: every 64th accepted mock


def mocks_config(nmock, boxes):
    """The workload's configuration, the same dict in both arms."""
    acc = [j for j, L in enumerate(boxes) if 2 * MOCK_SMAX < L]
    return {"workload": "mocks%d" % nmock, "n_catalogues": nmock,
            "accepted": len(acc),
            "rejected_smax_ge_half_box": nmock - len(acc),
            "bins": "(s,mu) 40x100 s<200", "weighted": False,
            "density": 2.5e-4, "n_range": [1e4, 1e6], "seed": 7,
            "cpu_sample": "accepted mocks %s (one in %d)" % (
                acc[::MOCK_CPU_STRIDE], MOCK_CPU_STRIDE),
            "l2": "flushed between GPU steps (256 MiB write)"}


def mocks_cpu_sample(cats, boxes, subset, steps=1, warmup=0):
    """The CPU restatement of FCFC's counter (oracle/, cell grid, OpenMP on
    every host core) on the sample mocks: (pairs/s, in-range pairs, s per
    step, description)."""
    from oracle import fcfc_oracle as fo
    bins = [fo.Bins(False, 1, ns=40, smin=0, ds=5, nmu=100, box=boxes[j])
            for j in subset]
    pairs = 0
    tt = 0.0
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        tot = 0
        for b, j in zip(bins, subset):
            tot += int(b.count(cats[j], mode=3).sum())
        dt = time.perf_counter() - t0
        pairs = tot
        if it >= warmup:
            tt += dt
    ms = tt / steps
    desc = ("mocks %s of the 256 (%d catalogues, %d points, %d in-range "
            "pairs per step), unweighted DD (s,mu) 40x100, %.2f s per step" % (
                list(subset), len(subset), sum(len(cats[j]) for j in subset),
                pairs, ms))
    return pairs / ms, pairs, ms, desc


def kernel_source_sha256():
    """sha256 over the FP32 count kernel's sources (count32.cuh, then
    count_common.cuh): a committed ncu summary records the value it was
    captured on."""
    import hashlib
    h = hashlib.sha256()
    for f in ("count32.cuh", "count_common.cuh"):
        h.update(open(os.path.join(ROOT, "fcfc_gb300", "csrc", f), "rb").read())
    return h.hexdigest()


def profile_info(name):
    """Figures of a committed ncu summary (``key: value`` lines) and whether
    it was captured on the current count kernel source (its recorded
    kernel_source_sha256 against the files')."""
    info = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if ":" in line and not line.startswith((" ", "#")):
                k, v = line.split(":", 1)
                info[k.strip()] = v.strip()
    except OSError:
        return None
    info["source_matches"] = (info.get("kernel_source_sha256") ==
                              kernel_source_sha256())
    return info


def smem_atomic_peak(local):
    import ctypes as C
    import fcfc_gb300 as fg
    v = C.c_double()
    rc = fg.capi.load_library().fcfcg_probe_smem_atomics(int(local), C.byref(v))
    return v.value if rc == 0 else None


def run_mocks(args, rank, world, local, dist):
    """256 mock boxes, unweighted DD (s, mu) 40 x 100, one persistent launch
    per step (fcfcg_count_batch)."""
    import torch
    import fcfc_gb300 as fg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nmock = 32 if args.small else 256
    cats, boxes = mocks_workload(nmock=nmock, seed=7 + rank)
    ntot_pts = sum(len(c) for c in cats)
    tens = []
    dcats = []
    for x in cats:
        cols = [torch.from_numpy(np.ascontiguousarray(x[:, k])).to(dev)
                for k in range(3)]
        tens += cols
        dcats.append((cols[0].data_ptr(), cols[1].data_ptr(),
                      cols[2].data_ptr(), len(x)))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    pc = fg.PairCounter("box", fg.BIN_SMU, box=max(boxes), smin=0,
                        smax=MOCK_SMAX, ds=5, nmu=100, device=local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn, *a, **kw):
        """CUDA events on the current stream around a call that returns when
        its device work is done, the device idle on both sides."""
        torch.cuda.synchronize()
        e0.record()
        r = fn(*a, **kw)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), r

    def step(on_device=True, cat=None, sel=None, precision=fg.PREC_FP32_RECHECK):
        c = cat if cat is not None else dcats
        b = boxes
        if sel is not None:
            c = [c[j] for j in sel]
            b = [boxes[j] for j in sel]
        return pc.count_batch(c, b, on_device=on_device, precision=precision)

    counts, status, _ = step()
    accepted = [j for j in range(nmock) if status[j] == 0]
    pairs = int(sum(int(counts[j].sum()) for j in accepted))
    # fixed s_max / 3 cells against the autotuned refinement
    pc.set_cells_per_smax(3)
    step()
    ms_fixed3, _ = timed(step)
    pc.set_cells_per_smax(0)
    k_tuned, _ = pc.autotune_batch(dcats, boxes, on_device=True)
    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    launches0 = pc.stats()["launches"]
    tt, tk = 0.0, 0.0
    for _ in range(args.steps):
        flush.zero_()
        with nvtx("timed"):
            ms, _ = timed(step)
        tt += ms
        tk += pc.stats()["ms_count"]
    clocks = clk.stop()
    st = pc.stats()
    launches = pc.stats()["launches"] - launches0
    ms_step = max_over_ranks(tt / args.steps, dist)
    value = pairs * world / (ms_step * 1e-3)
    k_ms = tk / args.steps
    # the all-FP64 path on every accepted catalogue: same counts?
    with nvtx("fp64"):
        ms64, (c64, _, _) = timed(step, precision=fg.PREC_FP64)
    exact = all(np.array_equal(c64[j], counts[j]) for j in accepted)
    # the CPU sample mocks on the GPU (one launch of just those catalogues)
    subset = accepted[::MOCK_CPU_STRIDE]
    step(sel=subset)
    ms_sub = min(timed(step, sel=subset)[0] for _ in range(3))
    pairs_sub = int(sum(int(counts[j].sum()) for j in subset))
    # end to end from pinned host arrays (x, y, z columns per catalogue; the
    # copies to the device are inside the timed region)
    cols = [tuple(torch.from_numpy(np.ascontiguousarray(x[:, k])).pin_memory()
                  for k in range(3)) for x in cats]
    hcols = [tuple(t.numpy() for t in c) for c in cols]
    step(on_device=False, cat=hcols)
    te = 0.0
    for _ in range(args.steps):
        flush.zero_()
        ms, _ = timed(step, on_device=False, cat=hcols)
        te += ms
    e2e_ms = te / args.steps
    peak = fp32_peak_tflops(dev)
    apeak = smem_atomic_peak(local)
    achieved = pairs * FLOPS_PER_PAIR["smu"] / (k_ms * 1e-3) / 1e12
    prof = profile_info("k_count32_batch_mocks32.txt") or {}
    traffic = None
    if prof.get("traffic_bytes_per_launch_full_workload"):
        traffic = float(prof["traffic_bytes_per_launch_full_workload"])
    ipp = float(prof["warp_instructions_per_in_range_pair"]) \
        if prof.get("warp_instructions_per_in_range_pair") else None
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    cfg = mocks_config(nmock, boxes)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64-recheck", "data": "synthetic",
        "config": cfg,
        "workload_detail": {
            "n_points": ntot_pts, "pairs_per_step": pairs,
            "timing": "CUDA events on the current stream around each "
                      "batched count, device idle on both sides",
            "cells_per_smax_autotuned": k_tuned,
            "ms_per_step_fixed_smax_over_3": ms_fixed3,
            "parallelism": "replicas" if world > 1 else "1 GPU"},
        "fp64": {"value": pairs / (ms64 * 1e-3), "unit": UNIT,
                 "catalogues": len(accepted), "pairs": pairs, "ms": ms64,
                 "speedup_fp32_recheck_over_fp64": ms64 / ms_step,
                 "counts_identical": exact},
        "cpu_sample_on_gpu": {"value": pairs_sub / (ms_sub * 1e-3),
                              "unit": UNIT, "catalogues": subset,
                              "pairs": pairs_sub, "ms": ms_sub},
        "e2e": {"value": pairs / (e2e_ms * 1e-3), "unit": UNIT,
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": ntot_pts * 24,
                "d2h_bytes_per_step": len(accepted) * pc.ntot * 8},
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "kernel": "k_count32<box,smu,unweighted,batch>",
                     "kernel_ms": k_ms,
                     "peak_source": "measured cuBLAS SGEMM (TF32 off) on this GPU",
                     "flops_per_pair": FLOPS_PER_PAIR["smu"],
                     "smem_atomics": None if not apeak else {
                         "achieved": pairs / (k_ms * 1e-3), "peak": apeak,
                         "unit": "shared 32-bit atomic adds/s",
                         "frac": pairs / (k_ms * 1e-3) / apeak,
                         "per_pair": 1,
                         "peak_source": "fcfcg_probe_smem_atomics on this GPU "
                                        "(lane-distinct banks, every SM)"},
                     "issue": None if ipp is None else {
                         "achieved": pairs / (k_ms * 1e-3) * ipp,
                         "peak": 152 * 4 * mhz * 1e6,
                         "unit": "warp instructions/s",
                         "frac": pairs / (k_ms * 1e-3) * ipp / (152 * 4 * mhz * 1e6),
                         "warp_instructions_per_pair": ipp},
                     "from_profile": {
                         "file": "profiles/k_count32_batch_mocks32.txt",
                         "keys": ["traffic", "issue.warp_instructions_per_pair"],
                         "captured_on_current_source": prof.get("source_matches")}},
        "counters": {"candidates": st["candidates"], "rechecked": st["rechecked"],
                     "nchunks": st["nchunks"], "ms_grid": st["ms_grid"],
                     "ms_recheck": st["ms_recheck"]},
        "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu and not args.small:
        v, p_, ms_c, desc = mocks_cpu_sample(cats, boxes, subset)
        out["cpu_baseline"] = {"value": v, "unit": UNIT,
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": desc, "pairs_match_gpu": p_ == pairs_sub}
    if dist:
        dist.barrier()
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def survey_workload(nd, nr, seed=11):
    """RA uniform in [100, 260) deg, sin(Dec) uniform over [0, 60) deg,
    z ~ N(0.55, 0.10) truncated to [0.4, 0.7]; FKP weights 1 / (1 + n(z) P0),
    P0 = 1e4, n(z) from the data in dz = 0.01 shells (flat LCDM, Om = 0.31),
    applied to data and randoms alike."""
    from fcfc_gb300 import synth
    d = synth.survey_radecz(nd, seed=seed)
    r = synth.survey_radecz(nr, seed=seed + 1)
    wd = synth.fkp_weights(d)
    # the randoms carry the data's n(z) at their redshifts
    wr = synth.fkp_weights(d, at=r)
    return d, r, wd, wr


def _dev(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def run_survey(args, rank, world, local, dist):
    """Survey Landy-Szalay counts: DD, DR, RR weighted, in (s, mu) 40 x 100
    and (s_perp, pi) 40 log x 40, RA/Dec/z converted on the device."""
    import torch
    import fcfc_gb300 as fg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nd, nr = (100000, 1000000) if args.small else (1000000, 10000000)
    d, r, wd, wr = survey_workload(nd, nr, seed=11 + rank)
    D = [_dev(d[:, k], dev) for k in range(3)] + [_dev(wd, dev)]
    R = [_dev(r[:, k], dev) for k in range(3)] + [_dev(wr, dev)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    p1 = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=200, ds=5, nmu=100,
                        device=local)
    p2 = fg.PairCounter("survey", fg.BIN_SPI, sedges=LOGBINS, pmin=0, pmax=40,
                        dpi=1, device=local)

    def load(pc):
        pc.load_radecz_device(0, D[0].data_ptr(), D[1].data_ptr(),
                              D[2].data_ptr(), nd, D[3].data_ptr())
        pc.load_radecz_device(1, R[0].data_ptr(), R[1].data_ptr(),
                              R[2].data_ptr(), nr, R[3].data_ptr())

    def step(weighted=True, prec=fg.PREC_FP32_RECHECK, pairs=("DD", "DR", "RR")):
        res = {}
        kms = {}
        for name, pc in (("smu", p1), ("spi", p2)):
            load(pc)
            for pr in pairs:
                a, b = (0, None) if pr == "DD" else ((0, 1) if pr == "DR" else (1, None))
                res[(name, pr)] = pc.count_pairs(a, b, weighted=weighted,
                                                 precision=prec)
                kms[(name, pr)] = pc.stats()["ms_count"]
        return res, kms

    cnt, _ = step(weighted=False)
    pairs = {k: int(v.sum()) for k, v in cnt.items()}
    pairs_step = sum(pairs.values())
    # per-count kernel times from one plain step (outside the timed region)
    plain, kt = step()
    # the timed step: per binning, the catalogues converted and loaded, then
    # DD, DR and RR replayed from one CUDA graph
    LS = [(0, None, True), (0, 1, True), (1, None, True)]
    graphs = ((p1, p1.count_graph(LS)), (p2, p2.count_graph(LS)))

    def gstep():
        out = []
        for pc, g in graphs:
            load(pc)
            out += g.run()
        return out
    for _ in range(max(args.warmup, 0)):
        got = gstep()
    # the replays give exactly the plain counts
    want = [plain[(n, pr)] for n in ("smu", "spi") for pr in ("DD", "DR", "RR")]
    graph_equal = all(np.array_equal(a, b) for a, b in zip(got, want))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    l0 = p1.stats()["launches"] + p2.stats()["launches"]
    tt = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gstep()
        tt += time.perf_counter() - t0
    clocks = clk.stop()
    launches = p1.stats()["launches"] + p2.stats()["launches"] - l0
    ms_step = max_over_ranks(tt / args.steps * 1e3, dist)
    value = pairs_step * world / (ms_step * 1e-3)
    # all-FP64 path on DD (both binnings), against FP32 + recheck
    t0 = time.perf_counter()
    c64, k64 = step(prec=fg.PREC_FP64, pairs=("DD",))
    ms64 = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    c32, _ = step(pairs=("DD",))
    ms32 = (time.perf_counter() - t0) * 1e3
    rel = max(float(np.max(np.abs(c32[k] - c64[k]) /
                           np.maximum(np.abs(c64[k]), 1e-300))) for k in c64)
    dd_pairs = pairs[("smu", "DD")] + pairs[("spi", "DD")]
    # end to end from host arrays (conversion included)
    # host columns (RA, Dec, z), prepared outside the timed region
    dcols = tuple(np.ascontiguousarray(d[:, k]) for k in range(3))
    rcols = tuple(np.ascontiguousarray(r[:, k]) for k in range(3))

    def e2e():
        for pc, g in graphs:
            pc.load_radecz(0, dcols, wd)
            pc.load_radecz(1, rcols, wr)
            g.run()
    e2e()
    t0 = time.perf_counter()
    e2e()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    peak = fp32_peak_tflops(dev)
    k_rr = kt[("smu", "RR")]
    achieved = pairs[("smu", "RR")] * FLOPS_PER_PAIR["smu"] / (k_rr * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64-recheck", "data": "synthetic",
        "config": {"workload": "survey_ls_%dx%d" % (nd, nr), "n_data": nd,
                   "n_random": nr, "weights": "FKP, P0 = 1e4",
                   "coordinates": "RA/Dec/z converted on the device (Om = 0.31)",
                   "bins": "(s,mu) 40x100 s<200 + (s_perp,pi) 40 log [0.1,100) x 40 lin [0,40)",
                   "pairs": {"%s_%s" % k: v for k, v in pairs.items()},
                   "pairs_per_step": pairs_step,
                   "counts": "per binning: load + DD, DR, RR replayed from one CUDA graph",
                   "graph_equals_plain_counts": graph_equal,
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "fp64": {"value": dd_pairs / (ms64 * 1e-3), "unit": UNIT,
                 "counts": "DD (s,mu) + DD (s_perp,pi)", "ms": ms64,
                 "fp32_recheck_ms_same_counts": ms32,
                 "speedup_fp32_recheck_over_fp64": ms64 / ms32,
                 "max_rel_diff_weighted": rel},
        "e2e": {"value": pairs_step / (e2e_ms * 1e-3), "unit": UNIT,
                "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 2 * (nd + nr) * 32,
                "d2h_bytes_per_step": 3 * (p1.ntot + p2.ntot) * 8},
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "kernel": "k_count32<survey,smu,weighted> (RR)",
                     "kernel_ms": k_rr,
                     "peak_source": "measured cuBLAS SGEMM (TF32 off) on this GPU",
                     "flops_per_pair": FLOPS_PER_PAIR["smu"],
                     "issue": issue_bound(
                         pairs[("smu", "RR")] / (k_rr * 1e-3), clocks,
                         "k_count32_survey_smu_wt_rr.txt"),
                     "from_profile": {
                         "file": "profiles/k_count32_survey_smu_wt_rr.txt",
                         "keys": ["issue.warp_instructions_per_pair"],
                         "captured_on_current_source": (profile_info(
                             "k_count32_survey_smu_wt_rr.txt") or {}).get(
                                 "source_matches")}},
        "counters": {"kernel_ms_%s_%s" % k: v for k, v in kt.items()},
        "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if dist:
        dist.barrier()
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def run_adjoint(args, rank, world, local, dist):
    """dL/dw for every data weight, L = sum_b g_b xi_LS(b) over (s, mu)
    40 x 100, data 5e5 (lognormal weights) and randoms 5e6 of the survey
    generator: forward DD, DR, RR and the adjoint of DD and DR."""
    import torch
    import fcfc_gb300 as fg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fcfc_gb300 import synth
    nd, nr = (50000, 500000) if args.small else (500000, 5000000)
    d = synth.radecz_to_xyz(synth.survey_radecz(nd, seed=31 + rank))
    r = synth.radecz_to_xyz(synth.survey_radecz(nr, seed=32 + rank))
    wd = synth.lognormal_weights(nd, 0.3, seed=33 + rank)
    pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=200, ds=5, nmu=100,
                        device=local)
    g = np.random.default_rng(34).normal(size=pc.ntot)
    pc.load(0, d, wd)
    pc.load(1, r)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def forward():
        dd = pc.count_pairs(0, weighted=True)
        dr = pc.count_pairs(0, 1, weighted=True)
        rr = pc.count_pairs(1, weighted=True)
        return dd, dr, rr

    def backward(dd, dr, rr):
        W, Wr = float(np.sum(wd)), float(nr)
        nDD, nDR, nRR = W * (W - 1), W * Wr, Wr * (Wr - 1)
        rrn = 2 * rr / nRR
        ok = rrn > 0
        gdd = np.where(ok, g * 2 / nDD / np.where(ok, rrn, 1), 0.0)
        gdr = np.where(ok, -g * 2 / nDR / np.where(ok, rrn, 1), 0.0)
        a1, _ = pc.adjoint(0, None, gdd)
        ms1 = pc.stats()["ms_total"]
        a2, _ = pc.adjoint(0, 1, gdr)
        ms2 = pc.stats()["ms_total"]
        # the normalisations W (W - 1) and W Wr depend on every data weight
        gr = np.where(ok, g / np.where(ok, rrn, 1), 0.0)
        dW = (-(gr * 2 * dd).sum() * (2 * W - 1) / nDD ** 2 +
              (gr * 2 * dr).sum() * Wr / nDR ** 2)
        return a1 + a2 + dW, ms1 + ms2

    un = [int(pc.count_pairs(0).sum()), int(pc.count_pairs(0, 1).sum())]
    pairs_grad = sum(un)
    for _ in range(max(args.warmup, 0)):
        backward(*forward())
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    tf = tb = 0.0
    kb = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c = forward()
        t1 = time.perf_counter()
        grad, msb = backward(*c)
        t2 = time.perf_counter()
        tf += t1 - t0
        tb += t2 - t1
        kb += msb
    clocks = clk.stop()
    ms_b = max_over_ranks(tb / args.steps * 1e3, dist)
    out = {
        "metric": "adjoint: DD + DR pairs differentiated per second (dL/dw for "
                  "all data weights)",
        "value": pairs_grad * world / (ms_b * 1e-3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64-recheck bins, f64-rounded products summed as int64",
        "data": "synthetic",
        "config": {"workload": "adjoint_ls_%dx%d" % (nd, nr), "n_data": nd,
                   "n_random": nr, "bins": "(s,mu) 40x100 s<200",
                   "loss": "sum_b g_b xi_LS(b), g ~ N(0,1)",
                   "pairs_dd_dr": pairs_grad,
                   "forward_ms_dd_dr_rr": tf / args.steps * 1e3,
                   "backward_device_ms": kb / args.steps,
                   "grad_norm": float(np.linalg.norm(grad)),
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def cpu_baseline_sample(x, w, box):
    """The CPU restatement of FCFC's counter (oracle/, OpenMP on every host
    core) on the whole workload, one weighted step: 10-30 s of CPU work."""
    from oracle import fcfc_oracle as fo
    b1 = fo.Bins(False, 1, ns=40, smin=0, ds=5, nmu=100, box=box)
    b2 = fo.Bins(False, 2, ns=40, sedges=LOGBINS, np_=40, pmin=0, dpi=1, box=box)
    n_in = int(b1.count(x, mode=3).sum() + b2.count(x, mode=3).sum())
    t0 = time.perf_counter()
    b1.count(x, wa=w, mode=3)
    b2.count(x, wa=w, mode=3)
    dt = time.perf_counter() - t0
    return {"value": n_in / dt, "unit": UNIT, "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": "the full workload (%d points, L=%g Mpc/h), one weighted "
                      "DD (s,mu)+(s_perp,pi) step, %d in-range pairs, %.2f s" %
                      (len(x), box, n_in, dt)}


def run_cli(args, rank, world, local, dist):
    """FCFC's command line flow end to end: the 2e6-object Neyman-Scott box
    written as an ASCII catalogue (x y z w, %.17g), then FCFC_2PT_BOX_GPU run
    on it twice per step -- weighted DD in (s, mu) with xi and multipoles,
    and in (s_perp, pi) with w_p -- each a fresh process that reads the file,
    counts and writes FCFC's files.  Wall time per step, process start-up
    and device initialisation included."""
    import re
    import subprocess
    import tempfile
    box = BOX / 2 if args.small else BOX
    npar = 20000 // 8 if args.small else 20000
    x, w = workload(box=box, nparent=npar, seed=1 + rank)
    n = len(x)
    d = tempfile.mkdtemp(prefix="fcfcg_cli_")
    cat = os.path.join(d, "ns.txt")
    np.savetxt(cat, np.column_stack([x, w]), fmt="%.17g")
    np.savetxt(os.path.join(d, "sbin.txt"),
               np.column_stack([LOGBINS[:-1], LOGBINS[1:]]), fmt="%.17g")
    common = ["CATALOG = [%s]" % cat, "CATALOG_LABEL = [D]",
              'ASCII_FORMATTER = ["%lf %lf %lf %lf"]',
              "POSITION = [$1, $2, $3]", "WEIGHT = [$4]",
              "BOX_SIZE = %.17g" % box, "DATA_STRUCT = 0", "OVERWRITE = 2",
              "PAIR_COUNT = [DD]", 'CF_ESTIMATOR = ["DD / @@ - 1"]']
    confs = {
        "smu": common + ["BINNING_SCHEME = 1", "SEP_BIN_MIN = 0",
                         "SEP_BIN_MAX = 200", "SEP_BIN_SIZE = 5",
                         "MU_BIN_NUM = 100",
                         "PAIR_COUNT_FILE = [%s]" % os.path.join(d, "dd_smu.bin"),
                         "CF_OUTPUT_FILE = [%s]" % os.path.join(d, "xi_smu.txt"),
                         "MULTIPOLE = [0, 2, 4]",
                         "MULTIPOLE_FILE = [%s]" % os.path.join(d, "mp.txt")],
        "spi": common + ["BINNING_SCHEME = 2",
                         "SEP_BIN_FILE = %s" % os.path.join(d, "sbin.txt"),
                         "PI_BIN_MIN = 0", "PI_BIN_MAX = 40", "PI_BIN_SIZE = 1",
                         "PAIR_COUNT_FILE = [%s]" % os.path.join(d, "dd_spi.bin"),
                         "CF_OUTPUT_FILE = [%s]" % os.path.join(d, "xi_spi.txt"),
                         "PROJECTED_CF = T",
                         "PROJECTED_FILE = [%s]" % os.path.join(d, "wp.txt")],
    }
    for k, lines in confs.items():
        open(os.path.join(d, k + ".conf"), "w").write("\n".join(lines) + "\n")
    exe = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fcfc_gb300",
                       "bin", "FCFC_2PT_BOX_GPU")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES=str(local))

    def step():
        reads = []
        for k in ("smu", "spi"):
            r = subprocess.run([exe, "-c", os.path.join(d, k + ".conf"), "-v"],
                               capture_output=True, text=True, env=env)
            if r.returncode:
                raise RuntimeError(r.stdout + r.stderr)
            reads += [float(v) for v in re.findall(r"read ([0-9.]+) s", r.stdout)]
        return reads
    # in-range pairs of the two runs (unweighted counts through the library)
    import fcfc_gb300 as fg
    pairs = 0
    for kw in (dict(bintype=fg.BIN_SMU, smin=0, smax=200, ds=5, nmu=100),
               dict(bintype=fg.BIN_SPI, sedges=LOGBINS, pmin=0, pmax=40, dpi=1)):
        pc = fg.PairCounter("box", box=box, device=local, **kw)
        pc.load(0, x)
        pairs += int(pc.count_pairs(0).sum())
        pc.close()
    for _ in range(max(args.warmup, 1)):
        step()
    t0 = time.perf_counter()
    reads = []
    for _ in range(args.steps):
        reads += step()
    wall = (time.perf_counter() - t0) / args.steps
    ms_step = max_over_ranks(wall * 1e3, dist)
    out = {"metric": METRIC + " (command line, end to end)",
           "value": pairs * world / (ms_step * 1e-3), "unit": UNIT,
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64-recheck", "data": "synthetic",
           "config": {"workload": "cli_ns_box_%d" % n, "n_points": n,
                      "catalogue_bytes": os.path.getsize(cat),
                      "runs_per_step": "FCFC_2PT_BOX_GPU (s,mu) + (s_perp,pi)",
                      "pairs_per_step": pairs,
                      "ascii_read_s_mean": float(np.mean(reads)),
                      "parallelism": "replicas" if world > 1 else "1 GPU"},
           "e2e": {"value": pairs * world / (ms_step * 1e-3), "unit": UNIT,
                   "ms_per_step": ms_step,
                   "h2d_bytes_per_step": 2 * n * 32, "d2h_bytes_per_step": 0}}
    if dist:
        dist.barrier()
    if rank == 0:
        print(json.dumps(out), flush=True)
    shutil.rmtree(d, ignore_errors=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--small", action="store_true",
                    help="quarter-size box (for profiler captures)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="mocks256",
                    choices=["ns_box_2e6", "mocks256", "survey", "adjoint",
                             "cli"],
                    help="mocks256: 256 mock boxes in one persistent launch; "
                         "survey: DD/DR/RR of 1e6 data and 1e7 randoms; "
                         "adjoint: dL/dw of a Landy-Szalay loss; "
                         "cli: FCFC_2PT_BOX_GPU end to end on an ASCII file")
    args = ap.parse_args()
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.barrier()
        return rc

    if args.workload == "mocks256":
        return run_mocks(args, rank, world, local, dist)
    if args.workload == "survey":
        return run_survey(args, rank, world, local, dist)
    if args.workload == "adjoint":
        return run_adjoint(args, rank, world, local, dist)
    if args.workload == "cli":
        return run_cli(args, rank, world, local, dist)
    import torch
    import fcfc_gb300 as fg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    box = BOX / 2 if args.small else BOX
    npar = 20000 // 8 if args.small else 20000
    x, w = workload(box=box, nparent=npar, seed=1 + rank)
    n = len(x)
    # device-resident raw catalogue (FP64, as read)
    xd = [torch.from_numpy(np.ascontiguousarray(x[:, k])).to(dev) for k in range(3)]
    wd = torch.from_numpy(w).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    p1 = fg.PairCounter("box", fg.BIN_SMU, box=box, smin=0, smax=200, ds=5,
                        nmu=100, device=local)
    p2 = fg.PairCounter("box", fg.BIN_SPI, box=box, sedges=LOGBINS, pmin=0,
                        pmax=40, dpi=1, device=local)

    def step(prec=fg.PREC_FP32_RECHECK):
        ms = 0.0
        res = []
        for pc in (p1, p2):
            pc.load_device(0, xd[0].data_ptr(), xd[1].data_ptr(),
                           xd[2].data_ptr(), n, wd.data_ptr())
            c = pc.count_pairs(0, weighted=True, precision=prec)
            st = pc.stats()
            ms += st["ms_total"]
            res.append((c, st))
        return ms, res

    # exact in-range pair numbers of this workload (unweighted counts)
    n_in = []
    tuned = []
    for pc in (p1, p2):
        pc.load_device(0, xd[0].data_ptr(), xd[1].data_ptr(), xd[2].data_ptr(),
                       n, wd.data_ptr())
        n_in.append(int(pc.count_pairs(0, weighted=False).sum()))
        # grid refinement for this density, timed once before the run
        tuned.append(pc.autotune(0, weighted=True)[0])
    pairs_per_step = sum(n_in)
    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    # A step is timed whole: CUDA events on the current stream around it,
    # with the device idle on both sides.  The engine works on its own
    # streams and returns only when its work is done, so the interval holds
    # the preparation, both counts and every host round trip between them.
    ms_tot, ms_dev, ms_k1, ms_k2 = 0.0, 0.0, 0.0, 0.0
    launches0 = p1.stats()["launches"] + p2.stats()["launches"]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        with nvtx("timed"):
            e0.record()
            ms, res = step()
            e1.record()
        torch.cuda.synchronize()
        ms_tot += e0.elapsed_time(e1)
        ms_dev += ms
        ms_k1 += res[0][1]["ms_count"]
        ms_k2 += res[1][1]["ms_count"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clocks = clk.stop()
    launches_total = p1.stats()["launches"] + p2.stats()["launches"] - launches0
    st1 = res[0][1]
    st2 = res[1][1]
    # max over ranks
    ms_step = max_over_ranks(ms_tot / args.steps, dist)
    value = pairs_per_step * world / (ms_step * 1e-3)

    # all-FP64 GPU path, one step, timed the same way
    torch.cuda.synchronize()
    with nvtx("fp64"):
        e0.record()
        step(prec=fg.PREC_FP64)
        e1.record()
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1)
    fp64_value = pairs_per_step / (ms64 * 1e-3)

    # end to end through the C ABI from pinned host memory
    xh = [torch.from_numpy(np.ascontiguousarray(x[:, k])).pin_memory() for k in range(3)]
    wh = torch.from_numpy(w).pin_memory()
    import ctypes as C
    lib = fg.capi.load_library()
    e2e_res = []

    def e2e_step():
        for pc in (p1, p2):
            rc = lib.fcfcg_load_catalog(pc.h, 0, n, C.c_void_p(xh[0].data_ptr()),
                                        C.c_void_p(xh[1].data_ptr()),
                                        C.c_void_p(xh[2].data_ptr()),
                                        C.c_void_p(wh.data_ptr()))
            if rc:
                raise fg.FCFCGError(rc)
            e2e_res.append(pc.count_pairs(0, weighted=True))

    e2e_step()
    torch.cuda.synchronize()
    te = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        te += time.perf_counter() - t0
    e2e_ms = te / args.steps * 1e3
    h2d = 2 * n * 4 * 8
    d2h = (p1.ntot + p2.ntot) * 16

    # roofline of the dominant kernel: (s, mu) count, FP32 pipe
    peak = fp32_peak_tflops(dev)
    k1_ms = ms_k1 / args.steps
    achieved = n_in[0] * FLOPS_PER_PAIR["smu"] / (k1_ms * 1e-3) / 1e12
    traffic = profile_traffic()
    if traffic is not None and args.small:
        traffic = None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64-recheck", "data": "synthetic",
        "config": {"workload": "ns_box_2e6" if not args.small else "ns_box_2.5e5",
                   "n_points": n, "box": box,
                   "bins": "(s,mu) 40x100 s<200 + (s_perp,pi) 40 log [0.1,100) x 40 lin [0,40)",
                   "weighted": True, "pairs_per_step": pairs_per_step,
                   "pairs_smu": n_in[0], "pairs_spi": n_in[1],
                   "l2": "flushed between steps (256 MiB write)",
                   "cells_per_smax": [st1["cells_per_smax"], st2["cells_per_smax"]],
                   "cells_per_smax_autotuned": tuned,
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": ms64,
                 "speedup_fp32_recheck_over_fp64": value / world / fp64_value},
        "e2e": {"value": pairs_per_step / (e2e_ms * 1e-3), "unit": UNIT,
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "kernel": "k_count32<box,smu,weighted>",
                     "kernel_ms": k1_ms,
                     "peak_source": "measured cuBLAS SGEMM (TF32 off) on this GPU",
                     "flops_per_pair": FLOPS_PER_PAIR["smu"],
                     "issue": issue_bound(n_in[0] / (k1_ms * 1e-3), clocks),
                     "from_profile": {
                         "file": "profiles/k_count32_box_smu_wt_ns_box.txt",
                         "keys": ["traffic", "issue.warp_instructions_per_pair"],
                         "captured_on_current_source": (profile_info(
                             "k_count32_box_smu_wt_ns_box.txt") or {}).get(
                                 "source_matches")}},
        "counters": {"candidates_smu": st1["candidates"],
                     "rechecked_smu": st1["rechecked"],
                     "candidates_spi": st2["candidates"],
                     "rechecked_spi": st2["rechecked"],
                     "wall_ms_per_step": wall / args.steps * 1e3,
                     "engine_device_ms_per_step": ms_dev / args.steps,
                     "kernel_ms_smu": ms_k1 / args.steps,
                     "kernel_ms_spi": ms_k2 / args.steps},
        "clocks": clocks,
        "gpu_launches": int(launches_total),
    }
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_sample(x, w, box)
    if dist:
        dist.barrier()
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
