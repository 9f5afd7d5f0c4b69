"""Benchmark: NUFFT forward+adjoint coil-pairs/s on one GB300 (or N replicas).

Workload (one "step"): the 2-D multi-coil operator -- image 256x256,
oversampled grid 512x512, kernel 6x6, table oversampling 1024, golden-angle
radial trajectory of 402 spokes x 512 readout points (205,824 samples),
32 coils -- one batched forward and one batched adjoint over all coils.
Inputs are seeded synthetic data (complex N(0,1) image times smooth Gaussian
coil maps); no dataset is involved.

Reported (one JSON line on rank 0):
  value      batched coil-pairs/s with inputs resident in HBM (CUDA events,
             L2 flushed between steps by a 256 MB write)
  e2e        the same metric through the public drop-in API with host numpy
             buffers (H2D and D2H inside the timed region)
  per_call   coil-pairs/s of the plain per-coil transform on the same GPU
  roofline   the dominant kernel's algorithmic bytes / CUDA-event time vs the
             measured HBM copy bandwidth
  cpu_baseline  the oracle's CPU restatement of the reference table path on
             the host cores (bounded sample)
``--impl reference`` times the reference's CPU implementation instead (the
reference itself where it is importable, else the oracle restatement).
``--profile`` runs the same workload's kernels only (warm-up pairs, then
``--steps`` batched pairs and one table gather and spread) without timing,
parity or baselines: the command the kernel profiles are captured from.

Multi-GPU: the coil batches are independent, so N GPUs run N replicas
(weak scaling, no collective on the data path).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "NUFFT fwd+adj pairs/s, batched vs plain per-call, at rel err ≤1e-4 vs FP64 NUDFT"
UNIT = "coil-pairs/s"
WORKLOAD = dict(name="2d-multicoil-radial", Nd=(256, 256), Kd=(512, 512), Jd=(6, 6), L=1024,
                spokes=402, readout=512, coils=32)


def build_inputs():
    from mrrt.nufft_gb300.trajectories import complex_image, gaussian_coil_maps, radial_2d

    w = WORKLOAD
    omega = radial_2d(w["spokes"], w["readout"], golden=True)
    img = complex_image(w["Nd"], seed=0).astype(np.complex128)
    maps = gaussian_coil_maps(w["Nd"], w["coils"])
    x = (maps * img[None]).astype(np.complex64)           # [C, N0, N1]
    x_f = np.asfortranarray(np.moveaxis(x, 0, -1))        # [N0, N1, C] Fortran order
    return omega, x_f


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def clock_sampler_start(path):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-lms", "200"]
    try:
        return subprocess.Popen(cmd, stdout=open(path, "w"), stderr=subprocess.DEVNULL)
    except (OSError, FileNotFoundError):
        return None


def clock_sampler_stop(proc, path, device_index):
    if proc is None:
        return None
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        f = [v.strip() for v in line.split(",")]
        if len(f) < 9 or not f[0].isdigit() or int(f[0]) != device_index:
            continue
        try:
            sm.append(float(f[1]))
            smax.append(float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
            "samples": len(sm)}


def time_events(fn, steps, flush=None):
    """Per-step CUDA-event timing on the current stream; returns total ms."""
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        if flush is not None:
            flush()
        starts[i].record()
        fn()
        ends[i].record()
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends))


def cpu_baseline(omega, x_f, min_seconds=10.0, max_reps=50):
    """Time the CPU table path (reference via its package where importable,
    else the oracle restatement) on the full batched workload."""
    w = WORKLOAD
    kw = dict(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single")
    kind = "port"
    op = None
    try:
        from oracle.ref_shim import load_reference, reference_available

        if reference_available():
            op = load_reference().NufftBase(mode="table", **kw)
            kind = "reference"
    except Exception:
        op = None
    if op is None:
        from oracle import oracle

        op = oracle.OracleNufft(mode="table", **kw)
    y = op.fft(x_f)
    op.adj(y)
    t0 = time.perf_counter()
    reps = 0
    while True:
        y = op.fft(x_f)
        op.adj(y)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            break
    per = el / reps
    return {
        "value": w["coils"] / per,
        "unit": UNIT,
        "cores": os.cpu_count(),
        "kind": kind,
        "sample": "%d x batched fwd+adj of the full %d-coil workload (%.2f s each)" % (reps, w["coils"], per),
        "seconds_per_pair_batch": per,
    }


def run_reference(args, rank):
    if rank != 0:
        return
    omega, x_f = build_inputs()
    w = WORKLOAD
    kw = dict(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single", mode="table")
    kind = "port"
    try:
        from oracle.ref_shim import load_reference, reference_available

        if reference_available():
            op = load_reference().NufftBase(**kw)
            kind = "reference"
        else:
            raise RuntimeError
    except Exception:
        from oracle import oracle

        op = oracle.OracleNufft(**kw)
    for _ in range(args.warmup):
        op.adj(op.fft(x_f))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        op.adj(op.fft(x_f))
    el = time.perf_counter() - t0
    value = w["coils"] * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
        "data": "synthetic", "config": config_dict(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": kind,
                         "sample": "each step: batched fwd+adj of the full %d-coil workload" % w["coils"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(t, world, device):
    """The job's time for replicas: barrier, then the slowest rank's time
    (all-reduce MAX), identical on every rank."""
    if world <= 1:
        return float(t)
    import torch
    import torch.distributed as dist

    dist.barrier()
    v = torch.tensor([float(t)], device=device, dtype=torch.float64)
    dist.all_reduce(v, op=dist.ReduceOp.MAX)
    return float(v.item())


def job_value(units_per_rank, world, ms_per_step):
    """Whole-job throughput: the units all ranks processed per second."""
    return world * units_per_rank / (ms_per_step * 1e-3)


def config_dict():
    w = WORKLOAD
    return {"workload": w["name"], "Nd": list(w["Nd"]), "Kd": list(w["Kd"]), "Jd": list(w["Jd"]),
            "L": w["L"], "trajectory": "golden-angle radial %dx%d" % (w["spokes"], w["readout"]),
            "samples": w["spokes"] * w["readout"], "coils": w["coils"], "precision": "single",
            "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas"}


def run_ours(args, rank, world):
    import torch

    from mrrt.nufft_gb300 import NufftBase, dtft
    from oracle import oracle

    dev = torch.device("cuda", torch.cuda.current_device())
    w = WORKLOAD
    C = w["coils"]
    omega, x_f = build_inputs()
    kw = dict(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single")
    A = NufftBase(on_gpu=True, max_coils=C, **kw)
    A1 = NufftBase(on_gpu=True, max_coils=1, **kw)
    P, P1 = A.plan, A1.plan
    M = A.M
    N0, N1 = w["Nd"]
    # device-resident inputs in the plan layout [coil][N1][N0]
    x_dev = torch.from_numpy(np.ascontiguousarray(np.moveaxis(x_f, -1, 0).transpose(0, 2, 1))).to(dev)
    y_dev = torch.empty((C, M), dtype=torch.complex64, device=dev)
    xa_dev = torch.empty_like(x_dev)
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush():
        flush_buf.fill_(1.0)

    def pair():
        P.forward(x_dev, y_dev, C)
        P.adjoint(y_dev, xa_dev, C)

    # ---- parity (untimed): coil 0 vs the oracle; error vs the exact NUDFT ----
    pair()
    torch.cuda.synchronize()
    parity = {}
    if rank == 0:
        B = oracle.OracleNufft(**kw)
        x0 = x_f[..., :2]
        y_or = B.fft(x0)
        y_gpu = y_dev[:2].cpu().numpy().T
        parity["fwd_rel_err_vs_oracle"] = oracle.rel_l2(y_gpu, y_or)
        xa_or = B.adj(y_gpu)
        xa_gpu = xa_dev[:2].cpu().numpy().transpose(2, 1, 0)
        parity["adj_rel_err_vs_oracle"] = oracle.rel_l2(xa_gpu, xa_or)
        rows = np.random.default_rng(0).choice(M, 4096, replace=False)
        y_ex = dtft(x_f[..., 0].astype(np.complex128), omega[rows], shape=w["Nd"])
        parity["fwd_rel_err_vs_fp64_nudft"] = oracle.rel_l2(y_gpu[rows, 0], y_ex)
        parity["oracle_fwd_rel_err_vs_fp64_nudft"] = oracle.rel_l2(y_or[rows, 0], y_ex)

    stats = P.stats()
    launches_per_step = 2 + 2 + (1 if stats["split_tiles"] > 0 else 0)

    # ---- batched, device resident ------------------------------------------
    for _ in range(args.warmup):
        pair()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk_path = os.path.join(HERE, "gpurun_out" if os.path.isdir(os.path.join(HERE, "gpurun_out")) else ".",
                            "clocks_rank%d.csv" % rank)
    sampler = clock_sampler_start(clk_path) if rank == 0 else None
    t_batched = time_events(pair, args.steps, flush)
    torch.cuda.synchronize()
    t_batched = max_over_ranks(t_batched, world, dev)

    # ---- per-kernel timing for the roofline (same kernels, alone) -----------
    grid = torch.empty((C, w["Kd"][0] * w["Kd"][1]), dtype=torch.complex64, device=dev)

    def spread():
        P.interp_adjoint(y_dev, grid, C)

    def gather():
        P.interp_forward(grid, y_dev, C)

    for _ in range(2):
        spread()
        gather()
    t_spread = time_events(spread, args.steps, flush) / args.steps
    t_gather = time_events(gather, args.steps, flush) / args.steps
    clocks = clock_sampler_stop(sampler, clk_path, dev.index) if rank == 0 else None

    # ---- plain per-call loop on the same GPU --------------------------------
    x1 = [x_dev[c:c + 1].contiguous() for c in range(C)]
    y1 = [torch.empty((1, M), dtype=torch.complex64, device=dev) for _ in range(C)]
    xa1 = [torch.empty_like(x1[0]) for _ in range(C)]

    def per_call():
        for c in range(C):
            P1.forward(x1[c], y1[c], 1)
            P1.adjoint(y1[c], xa1[c], 1)

    for _ in range(max(1, args.warmup // 2)):
        per_call()
    per_steps = max(2, args.steps // 4)
    t_percall = time_events(per_call, per_steps, flush) / per_steps

    # ---- end to end through the public API with host buffers ----------------
    Ah = NufftBase(on_gpu=False, max_coils=C, **kw)
    for _ in range(2):
        Ah.adj(Ah.fft(x_f))
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        yh = Ah.fft(x_f)
        xh = Ah.adj(yh)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    h2d = x_f.nbytes + yh.nbytes
    d2h = yh.nbytes + xh.nbytes

    if rank != 0:
        return
    ms_per_step = t_batched / args.steps
    value = job_value(C, world, ms_per_step)
    hbm, peak_kind = peaks()
    Kp = w["Kd"][0] * w["Kd"][1]
    B_alg = C * M * 8 + M * 2 * 4 + C * Kp * 8
    dominant = "spread" if t_spread >= t_gather else "gather"
    t_dom = max(t_spread, t_gather)
    achieved = B_alg / (t_dom * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(dominant)
    cpu = cpu_baseline(omega, x_f)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex64", "data": "synthetic",
        "config": config_dict(),
        "per_call": {"value": C / (t_percall * 1e-3), "unit": UNIT, "ms_per_32_coil_pairs": t_percall,
                     "batched_over_per_call": (C / (ms_per_step * 1e-3)) / (C / (t_percall * 1e-3))},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "algorithmic_bytes": B_alg,
                     "kernel_ms": {"spread": t_spread, "gather": t_gather}},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": C / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds_per_step": t_e2e},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "parity": parity,
        "plan": stats,
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    """The workload's launches alone, for a profiler to capture."""
    import torch

    from mrrt.nufft_gb300 import NufftBase

    w = WORKLOAD
    C = w["coils"]
    omega, x_f = build_inputs()
    A = NufftBase(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single",
                  on_gpu=True, max_coils=C)
    P = A.plan
    dev = torch.device("cuda", torch.cuda.current_device())
    x_dev = torch.from_numpy(np.ascontiguousarray(np.moveaxis(x_f, -1, 0).transpose(0, 2, 1))).to(dev)
    y_dev = torch.empty((C, A.M), dtype=torch.complex64, device=dev)
    xa_dev = torch.empty_like(x_dev)
    grid = torch.empty((C, w["Kd"][0] * w["Kd"][1]), dtype=torch.complex64, device=dev)
    for _ in range(args.warmup + args.steps):
        P.forward(x_dev, y_dev, C)
        P.adjoint(y_dev, xa_dev, C)
    grid.copy_(torch.randn_like(grid))
    P.interp_forward(grid, y_dev, C)
    P.interp_adjoint(y_dev, grid, C)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": w["name"], "coils": C, "samples": A.M, "stats": P.stats()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", action="store_true", help="launch the workload's kernels only (no timing)")
    args = ap.parse_args()
    if args.profile:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        run_profile(args)
        return
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    try:
        run_ours(args, rank, world)
    finally:
        if world > 1:
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
