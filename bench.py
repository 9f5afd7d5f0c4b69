"""Benchmark: NUFFT forward+adjoint coil-pairs/s on one GB300 (or N replicas).

Workload (one "step"): the 2-D multi-coil operator -- image 256x256,
oversampled grid 512x512, kernel 6x6, table oversampling 1024, golden-angle
radial trajectory of 402 spokes x 512 readout points (205,824 samples),
32 coils -- one batched forward and one batched adjoint over all coils.
Inputs are seeded synthetic data (complex N(0,1) image times smooth Gaussian
coil maps); no dataset is involved.

Reported (one JSON line on rank 0):
  value      batched coil-pairs/s with inputs resident in HBM, the step
             (batched forward + adjoint) replayed from a CUDA graph (CUDA
             events, L2 flushed between steps by a 256 MB write); "eager"
             holds the same step launched call by call
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
WORKLOADS = {
    # the headline: one batched 32-coil operator vs 32 plain single-coil calls
    "2d-multicoil-radial": dict(name="2d-multicoil-radial", kind="radial2d", Nd=(256, 256),
                                Kd=(512, 512), Jd=(6, 6), L=1024, spokes=402, readout=512, coils=32),
    # 3-D kooshball: interp3 gather and 3-D tiled spread
    # the reference's CPU-runnable case: 128^2 image, 128 uniformly spaced spokes x 256, one coil
    "2d-radial-128": dict(name="2d-radial-128", kind="radial2d", Nd=(128, 128), Kd=(256, 256), Jd=(6, 6),
                          L=1024, spokes=128, readout=256, coils=1, golden=False),
    "3d-kooshball": dict(name="3d-kooshball", kind="koosh3d", Nd=(128, 128, 128), Kd=(256, 256, 256),
                         Jd=(6, 6, 6), L=1024, spokes=12000, readout=256, coils=8),
    # the 3-D kernels on a smaller volume (inputs still larger than L2), for profiler captures
    "3d-kooshball-96": dict(name="3d-kooshball-96", kind="koosh3d", Nd=(96, 96, 96), Kd=(192, 192, 192),
                            Jd=(6, 6, 6), L=1024, spokes=6000, readout=192, coils=8),
    # differentiable NUFFT: loss ||A(x; omega) - y||^2, gradients in x and omega, the trajectory
    # moved every step (device re-binning)
    "2d-spiral-grad": dict(name="2d-spiral-grad", kind="grad2d", Nd=(256, 256), Kd=(512, 512), Jd=(6, 6),
                           L=1024, interleaves=16, samples=4096, coils=1),
    # uneven dynamic series: every frame and coil in one launch per stage, CUDA graph, autotuned tiles
    "series-2d": dict(name="series-2d", kind="series", Nd=(192, 192), Kd=(384, 384), Jd=(6, 6),
                      L=1024, frames=64, readout=384, min_spokes=13, max_spokes=89, seed=4, coils=8),
}
WORKLOAD = WORKLOADS["2d-multicoil-radial"]


def build_inputs():
    """(omega [M, d], x_f [*Nd, C] Fortran order) of a single-operator workload."""
    from mrrt.nufft_gb300.trajectories import complex_image, gaussian_coil_maps, kooshball_3d, radial_2d

    w = WORKLOAD
    if w["kind"] == "koosh3d":
        omega = kooshball_3d(w["spokes"], w["readout"])
    else:
        omega = radial_2d(w["spokes"], w["readout"], golden=w.get("golden", True))
    img = complex_image(w["Nd"], seed=0).astype(np.complex128)
    maps = gaussian_coil_maps(w["Nd"], w["coils"])
    x = (maps * img[None]).astype(np.complex64)           # [C, *Nd]
    x_f = np.asfortranarray(np.moveaxis(x, 0, -1))        # [*Nd, C] Fortran order
    return omega, x_f


def plan_layout(x_f):
    """[*Nd, C] Fortran order -> contiguous [C, N_{d-1}, ..., N_0] (the plan's layout)."""
    nd = x_f.ndim - 1
    return np.ascontiguousarray(np.moveaxis(x_f, -1, 0).transpose((0,) + tuple(range(nd, 0, -1))))


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def clock_sampler_start(path):
    """Start nvidia-smi sampling every 50 ms and return once it has written
    its first line (at most 3 s), so that it is live when timing starts."""
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-lms", "50"]
    try:
        proc = subprocess.Popen(cmd, stdout=open(path, "w"), stderr=subprocess.DEVNULL)
    except (OSError, FileNotFoundError):
        return None
    t_end = time.time() + 3.0
    while time.time() < t_end and proc.poll() is None:
        if os.path.exists(path) and os.path.getsize(path) > 0:
            break
        time.sleep(0.02)
    return proc


def load_tail(fn, seconds=0.3):
    """Keep the timed workload running, untimed, while the clock sampler
    takes a few more samples under the same load."""
    import torch

    t_end = time.time() + seconds
    while time.time() < t_end:
        fn()
        torch.cuda.synchronize()


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


# What each cpu_baseline kind runs.
CPU_KIND_NOTE = {
    "reference": "the reference's own table interpolation C (mrrt/nufft/_extensions/c/nufft_table.c, "
                 "compiled on this host with its flags, -O2 -ffast-math -fopenmp)",
    "port": "the oracle's C restatement of the reference table path",
}


def _cpu_operator(omega, w):
    """The CPU table operator timed as the reference: the reference package
    itself where it imports (its sources present); else the reference's own
    compiled interpolation kernels (oracle/_ref, rebuilt on this host from the
    preprocessed unit) inside the oracle's restated pad / FFT / crop, which
    is where the reference spends its time; else the oracle restatement.
    Returns (op, kind)."""
    kw = dict(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single",
              mode="table")
    try:
        from oracle.ref_shim import load_reference, reference_available

        if reference_available():
            return load_reference().NufftBase(**kw), "reference"
    except Exception:
        pass
    from oracle import oracle, refc

    if refc.available():
        return oracle.OracleNufft(interp=refc, **kw), "reference"
    return oracle.OracleNufft(**kw), "port"


def cpu_baseline(omega, x_f, min_seconds=10.0, max_reps=50):
    """Time the CPU table path on the host cores: batched fwd+adj of the
    coils in ``x_f`` (the full workload, or a bounded sample of its coils),
    repeated for about ``min_seconds``."""
    w = WORKLOAD
    op, kind = _cpu_operator(omega, w)
    coils = x_f.shape[-1]
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
        "value": coils / per,
        "unit": UNIT,
        "cores": os.cpu_count(),
        "kind": kind,
        "sample": "%d x batched fwd+adj of %d of the workload's %d coils (%.2f s each); %s"
                  % (reps, coils, w["coils"], per, CPU_KIND_NOTE[kind]),
        "seconds_per_pair_batch": per,
    }


def _cpu_sample_coils(w):
    """Coils per CPU step: the full batch in 2-D; one coil of the 3-D volume
    (a full 8-coil 3-D pair takes the CPU tens of seconds)."""
    return 1 if len(w["Nd"]) == 3 else w["coils"]


# A throughput measured on wrong results is not a measurement: the parity
# step runs before any timing and stops the benchmark when the transform is
# off by more than the metric's own accuracy bar (relative L2 1e-4).  The
# oracle comparisons pass at 1e-7..1e-6 in 2-D; the 3-D adjoint differs from
# the serial float32 oracle by 7e-5 through summation order alone.
PARITY_BAR = 1e-4


def parity_gate(parity):
    bad = {k: v for k, v in parity.items()
           if not k.startswith("oracle_") and not (float(v) <= PARITY_BAR)}
    if bad:
        print("bench.py: parity failure, no timing taken: %s" % json.dumps(bad), file=sys.stderr, flush=True)
        raise SystemExit(1)


def run_reference(args, rank):
    """The reference's CPU table path (or the oracle restatement of it where
    the reference cannot be imported) on all host cores, same metric."""
    if rank != 0:
        return
    w = WORKLOAD
    if w["kind"] == "grad2d":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no autograd: no gradient "
                          "with respect to the image or the trajectory to time"}), flush=True)
        return
    if w["kind"] == "series":
        frames = _series_frames(w)[:4]
        ops, kind = [], "port"
        for om in frames:
            op, kind = _cpu_operator(om, w)
            ops.append(op)
        xs = [np.asfortranarray(np.moveaxis(_series_images_host(w, f), 0, -1)) for f in range(len(frames))]

        def step():
            for op, x in zip(ops, xs):
                op.adj(op.fft(x))

        units = len(frames) * w["coils"]
        sample = "each step: fwd+adj of frames 0-3 of the series, %d coils each, one operator per frame" % w["coils"]
    else:
        omega, x_f = build_inputs()
        op, kind = _cpu_operator(omega, w)
        xs = x_f[..., :_cpu_sample_coils(w)]

        def step():
            op.adj(op.fft(xs))

        units = xs.shape[-1]
        sample = "each step: batched fwd+adj of %d of the workload's %d coils" % (units, w["coils"])
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    value = units * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
        "data": "synthetic", "config": config_dict(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": kind,
                         "sample": sample + "; " + CPU_KIND_NOTE[kind]},
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


def config_dict(extra=None):
    w = WORKLOAD
    cfg = {"workload": w["name"], "Nd": list(w["Nd"]), "Kd": list(w["Kd"]), "Jd": list(w["Jd"]),
           "L": w["L"], "coils": w["coils"], "precision": "single",
           "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas"}
    if w["kind"] == "radial2d":
        cfg["trajectory"] = "%s radial %dx%d" % ("golden-angle" if w.get("golden", True) else "uniform-angle",
                                                  w["spokes"], w["readout"])
        cfg["samples"] = w["spokes"] * w["readout"]
    elif w["kind"] == "koosh3d":
        cfg["trajectory"] = "kooshball %d spokes x %d on a Fibonacci sphere" % (w["spokes"], w["readout"])
        cfg["samples"] = w["spokes"] * w["readout"]
    elif w["kind"] == "grad2d":
        cfg["trajectory"] = "variable-density spiral %d x %d" % (w["interleaves"], w["samples"])
        cfg["samples"] = w["interleaves"] * w["samples"]
    else:
        cfg["trajectory"] = ("%d frames, U{%d..%d} golden-angle spokes (seed %d) x %d"
                             % (w["frames"], w["min_spokes"], w["max_spokes"], w["seed"], w["readout"]))
        cfg["frames"] = w["frames"]
    if extra:
        cfg.update(extra)
    return cfg


# FFT lengths the library transforms with its own passes (gbn_colfft.cu,
# gbn_rowfft.cu); the other lengths use cuFFT (whose launches are not ours)
OWN_FFT_LENGTHS = (64, 96, 128, 192, 256, 384, 512, 768)


def our_launches_per_step(Kd, split_tiles):
    """Launches of this library's kernels in one forward + adjoint pair of a
    single-precision plan: with every axis length supported, the row pass
    (pad or crop folded in), the strided-axis passes and the interpolation
    kernel each way; else pad / crop and the interpolation kernel, plus the
    last-axis pass when its length is supported; the reduce of split tiles."""
    nd = len(Kd)
    if nd >= 2 and all(k in OWN_FFT_LENGTHS for k in Kd):
        per_dir = nd + 1
    elif nd >= 2 and Kd[-1] in OWN_FFT_LENGTHS:
        per_dir = 3
    else:
        per_dir = 2
    return 2 * per_dir + (1 if split_tiles > 0 else 0)


def _clock_path(rank):
    """Where the clock sampler writes: $GBN_BENCH_OUT, else the working directory."""
    out = os.environ.get("GBN_BENCH_OUT", ".")
    return os.path.join(out if os.path.isdir(out) else ".", "clocks_rank%d.csv" % rank)


def _traffic(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary of the
    default workload (read + write), or None."""
    tp = os.path.join(HERE, "profiles", "traffic.json")
    if WORKLOAD["name"] != "2d-multicoil-radial" or not os.path.exists(tp):
        return None
    return json.load(open(tp)).get(kernel)


def run_ours(args, rank, world):
    import torch

    from mrrt.nufft_gb300 import NufftBase, dtft
    from oracle import oracle

    if WORKLOAD["kind"] == "series":
        return run_series(args, rank, world)
    if WORKLOAD["kind"] == "grad2d":
        return run_grad(args, rank, world)
    dev = torch.device("cuda", torch.cuda.current_device())
    w = WORKLOAD
    C = w["coils"]
    nd = len(w["Nd"])
    omega, x_f = build_inputs()
    kw = dict(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single")
    A = NufftBase(on_gpu=True, max_coils=C, **kw)
    A1 = NufftBase(on_gpu=True, max_coils=1, **kw)
    P, P1 = A.plan, A1.plan
    M = A.M
    Kp = int(np.prod(w["Kd"]))
    # device-resident inputs in the plan layout [coil][N_{d-1}]...[N_0]
    x_dev = torch.from_numpy(plan_layout(x_f)).to(dev)
    y_dev = torch.empty((C, M), dtype=torch.complex64, device=dev)
    xa_dev = torch.empty_like(x_dev)
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush():
        flush_buf.fill_(1.0)

    def pair():
        P.forward(x_dev, y_dev, C)
        P.adjoint(y_dev, xa_dev, C)

    # ---- parity (untimed): first coils vs the oracle; error vs the exact NUDFT
    pair()
    torch.cuda.synchronize()
    parity = {}
    if rank == 0:
        B = oracle.OracleNufft(**kw)
        npar = 2 if nd < 3 else 1
        y_or = B.fft(x_f[..., :npar])
        y_gpu = y_dev[:npar].cpu().numpy().T
        parity["fwd_rel_err_vs_oracle"] = oracle.rel_l2(y_gpu.reshape(y_or.shape), y_or)
        xa_or = B.adj(y_gpu.reshape(y_or.shape))
        xa_gpu = xa_dev[:npar].cpu().numpy().transpose(tuple(range(nd, -1, -1)))
        parity["adj_rel_err_vs_oracle"] = oracle.rel_l2(xa_gpu.reshape(xa_or.shape), xa_or)
        # both single-precision adjoints against the oracle in double precision:
        # dense trajectory centres make float32 sums order-dependent
        B64 = oracle.OracleNufft(**dict(kw, precision="double"))
        xa_64 = B64.adj(y_gpu.reshape(y_or.shape).astype(np.complex128))
        parity["adj_rel_err_vs_fp64_oracle"] = oracle.rel_l2(xa_gpu.reshape(xa_64.shape), xa_64)
        parity["oracle_adj_rel_err_vs_fp64_oracle"] = oracle.rel_l2(xa_or.reshape(xa_64.shape), xa_64)
        rows = np.random.default_rng(0).choice(M, 4096 if nd < 3 else 1024, replace=False)
        y_ex = dtft(x_f[..., 0].astype(np.complex128), omega[rows], shape=w["Nd"])
        y_or0 = y_or.reshape(M, -1)[:, 0]
        parity["fwd_rel_err_vs_fp64_nudft"] = oracle.rel_l2(y_gpu[rows, 0], y_ex)
        parity["oracle_fwd_rel_err_vs_fp64_nudft"] = oracle.rel_l2(y_or0[rows], y_ex)
        parity_gate(parity)

    stats = P.stats()
    launches_per_step = our_launches_per_step(w["Kd"], stats["split_tiles"])

    # ---- batched, device resident: the step replayed from a CUDA graph -----
    for _ in range(args.warmup):
        pair()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        pair()

    def pair_graph():
        graph.replay()

    for _ in range(args.warmup):
        pair_graph()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = clock_sampler_start(_clock_path(rank)) if rank == 0 else None
    t_batched = time_events(pair_graph, args.steps, flush)
    torch.cuda.synchronize()
    t_batched = max_over_ranks(t_batched, world, dev)
    t_eager = time_events(pair, args.steps, flush) / args.steps

    # ---- per-kernel timing for the roofline (same kernels, alone) -----------
    grid = torch.empty((C, Kp), dtype=torch.complex64, device=dev)

    def spread():
        P.interp_adjoint(y_dev, grid, C)

    def gather():
        P.interp_forward(grid, y_dev, C)

    for _ in range(2):
        spread()
        gather()
    t_spread = time_events(spread, args.steps, flush) / args.steps
    t_gather = time_events(gather, args.steps, flush) / args.steps
    if rank == 0:
        load_tail(pair_graph)
    clocks = clock_sampler_stop(sampler, _clock_path(rank), dev.index) if rank == 0 else None

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
    del x1, y1, xa1, grid
    Ah = NufftBase(on_gpu=False, max_coils=C, **kw)
    # warm-up also grows torch's pinned host-memory pool to its working size:
    # it holds each step's results while the next step allocates, as the
    # timed loop does
    yh = xh = None
    for _ in range(max(6, args.warmup)):
        yh = Ah.fft(x_f)
        xh = Ah.adj(yh)
    torch.cuda.synchronize()
    e2e_steps = max(10, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        yh = Ah.fft(x_f)
        xh = Ah.adj(yh)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    h2d = x_f.nbytes + yh.nbytes
    d2h = yh.nbytes + xh.nbytes
    # the host path's results against the device path on the same images
    # (the pipelined chunks run their FFTs 16 planes at a time)
    P.forward(x_dev, y_dev, C)
    P.adjoint(y_dev, xa_dev, C)
    e_f = oracle.rel_l2(np.asarray(yh).T.reshape(-1), y_dev.reshape(-1).cpu().numpy())
    e_a = oracle.rel_l2(np.asarray(Ah.adj(np.asarray(y_dev.cpu().numpy().T))).ravel(order="F"),
                        xa_dev.cpu().numpy().transpose(tuple(range(nd, -1, -1))).ravel(order="F"))
    if not (e_f < 1e-6 and e_a < 1e-6):
        print("bench.py: end-to-end results differ from the device path: %.3g %.3g" % (e_f, e_a),
              file=sys.stderr, flush=True)
        raise SystemExit(1)

    if rank != 0:
        return
    ms_per_step = t_batched / args.steps
    value = job_value(C, world, ms_per_step)
    hbm, peak_kind = peaks()
    B_alg = C * M * 8 + M * nd * 4 + C * Kp * 8
    dominant = "spread" if t_spread >= t_gather else "gather"
    t_dom = max(t_spread, t_gather)
    achieved = B_alg / (t_dom * 1e-3) / 1e9
    cpu = cpu_baseline(omega, x_f[..., :_cpu_sample_coils(w)])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex64", "data": "synthetic",
        "config": config_dict(),
        # how this arm runs the workload (kept out of `config`, which names the
        # workload and matches the reference arm's)
        "execution": {"graph": True},
        "eager": {"ms_per_step": t_eager, "value": C / (t_eager * 1e-3)},
        "per_call": {"value": C / (t_percall * 1e-3), "unit": UNIT, "ms_per_step": t_percall,
                     "calls_per_step": 2 * C,
                     "batched_over_per_call": (C / (ms_per_step * 1e-3)) / (C / (t_percall * 1e-3))},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": _traffic(dominant), "algorithmic_bytes": B_alg,
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


def run_grad(args, rank, world):
    """Differentiable NUFFT step: y_hat = A(x; omega), loss = ||y_hat - y||^2,
    backward to x (the adjoint transform) and to omega (the derivative-table
    gather K5), with the trajectory moved every step (as an optimiser of the
    trajectory would) and its samples re-binned on the device.  Timed: the
    whole step, the re-bin alone, and K5 alone (CUDA events)."""
    import torch

    from mrrt.nufft_gb300.autograd import NufftOperator
    from mrrt.nufft_gb300.trajectories import complex_image, spiral_2d

    w = WORKLOAD
    dev = torch.device("cuda", torch.cuda.current_device())
    C, Nd, Kd = w["coils"], w["Nd"], w["Kd"]
    om0 = spiral_2d(w["interleaves"], w["samples"])
    M = om0.shape[0]
    op = NufftOperator(Nd, om0, Jd=w["Jd"], Kd=Kd, Ld=w["L"], max_coils=C)
    x_true = torch.from_numpy(np.stack([complex_image(Nd, seed=1 + c) for c in range(C)])).to(dev)
    g = torch.Generator(device="cpu").manual_seed(0)
    with torch.no_grad():
        y0 = op.forward(x_true)
        noise = torch.randn(y0.shape, dtype=torch.complex64, generator=g).to(dev)
        y = y0 + 0.01 * y0.abs().pow(2).mean().sqrt() * noise
    y64 = y.to(torch.complex128)
    x = torch.randn((C,) + Nd, dtype=torch.complex64, generator=g).to(dev).requires_grad_(True)
    om_base = torch.from_numpy(om0.astype(np.float32)).to(dev)
    # two trajectories alternate, so every step re-bins
    oms = [om_base, om_base + 1e-3]

    def step(k):
        om = oms[k % 2].clone().requires_grad_(True)
        loss = (op.forward(x, om).to(torch.complex128) - y64).abs().pow(2).sum()
        loss.backward()
        return loss, om.grad

    # parity (untimed): the omega gradient along a random +-1 direction
    # against central differences of the loss (steps 1e-3 and 5e-4 rad,
    # Richardson-extrapolated: the 1e-3 difference alone carries an O(eps^2)
    # truncation of about 1%)
    loss0, gom = step(0)
    v = torch.from_numpy(np.random.default_rng(9).choice([-1.0, 1.0], (M, 2))).to(dev, torch.float32)

    def loss_at(o):
        with torch.no_grad():
            return float((op.forward(x, o).to(torch.complex128) - y64).abs().pow(2).sum())

    def central(h):
        return (loss_at(oms[0] + h * v) - loss_at(oms[0] - h * v)) / (2 * h)

    fd1, fd2 = central(1e-3), central(5e-4)
    rich = (4 * fd2 - fd1) / 3
    an = float((gom.double() * v.double()).sum())
    parity = {"omega_grad_rel_err_vs_richardson_central_difference": abs(rich - an) / abs(an),
              "omega_grad_rel_err_vs_central_difference_1e-3": abs(fd1 - an) / abs(an)}
    if parity["omega_grad_rel_err_vs_richardson_central_difference"] > 2e-3:
        print("bench.py: omega gradient off: %s" % json.dumps(parity), file=sys.stderr, flush=True)
        raise SystemExit(1)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    sampler = clock_sampler_start(_clock_path(rank)) if rank == 0 else None
    t_steps = []
    for k in range(args.steps):
        flush_buf.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(k)
        torch.cuda.synchronize()
        t_steps.append(time.perf_counter() - t0)
    # re-bin alone (device binning of a changed trajectory)
    t_bin = []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.set_omega(oms[(k + 1) % 2])
        torch.cuda.synchronize()
        t_bin.append(time.perf_counter() - t0)
    # K5 alone: the derivative-table gather on the forward grid
    op.set_omega(oms[0])
    xp = op._image_to_plan(x.detach())
    scratch = torch.empty((C, M), dtype=torch.complex64, device=dev)
    op.plan.forward(xp, scratch, C)
    gy = torch.randn((C, M), dtype=torch.complex64, generator=g).to(dev)
    gtm = torch.empty((M, 2), dtype=torch.float32, device=dev)
    grid_ptr = op.plan.forward_grid(C)

    def k5():
        op.plan.grad_tm(grid_ptr, gy, op.phase_shift, gtm, C)

    for _ in range(3):
        k5()
    t_k5 = time_events(k5, args.steps) / args.steps
    clocks = clock_sampler_stop(sampler, _clock_path(rank), dev.index) if rank == 0 else None
    if rank != 0:
        return
    t_step = float(np.median(t_steps))
    Kp = int(np.prod(Kd))
    B_k5 = C * Kp * 8 + C * M * 8 + M * 2 * 4 + M * 2 * 4
    hbm, peak_kind = peaks()
    achieved = B_k5 / (t_k5 * 1e-3) / 1e9
    line = {
        "metric": "differentiable NUFFT steps/s (forward, image and omega gradients, device re-bin)",
        "value": 1.0 / t_step, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "complex64", "data": "synthetic", "config": config_dict(),
        "rebin_ms": 1e3 * float(np.median(t_bin)),
        "k5": {"kernel_ms": t_k5, "algorithmic_bytes": B_k5,
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "peak_kind": peak_kind,
                            "unit": "GB/s", "frac": achieved / hbm}},
        "loss": float(loss0.item()), "parity": parity, "clocks": clocks,
        "timing": "host clock around each step with torch.cuda.synchronize (the step is a chain of "
                  "launches with two small device-to-host reads in the re-bin); K5 by CUDA events",
    }
    print(json.dumps(line), flush=True)



def _series_frames(w):
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    return uneven_series_2d(w["frames"], w["readout"], min_spokes=w["min_spokes"],
                            max_spokes=w["max_spokes"], seed=w["seed"])


def _series_images_host(w, f):
    """Frame f's coil images [C, *Nd] (complex64): a seeded N(0,1) image per
    frame times the Gaussian coil maps."""
    from mrrt.nufft_gb300.trajectories import complex_image, gaussian_coil_maps

    img = complex_image(w["Nd"], seed=100 + f).astype(np.complex128)
    return (gaussian_coil_maps(w["Nd"], w["coils"]) * img[None]).astype(np.complex64)


def run_series(args, rank, world):
    """The uneven dynamic series: all frames and coils in one plan (one launch
    per stage), tiles from the autotuner, steps replayed from CUDA graphs;
    against one plain single-coil call per frame and coil."""
    import torch

    from mrrt.nufft_gb300 import NufftBase, dtft
    from mrrt.nufft_gb300.autotune import tune_series
    from mrrt.nufft_gb300.series import NufftSeries
    from oracle import oracle

    dev = torch.device("cuda", torch.cuda.current_device())
    w = WORKLOAD
    C, F = w["coils"], w["frames"]
    oms = _series_frames(w)
    tile, stile, report = tune_series(w["Nd"], oms, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], coils=C, reps=3)
    S = NufftSeries(w["Nd"], oms, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], coils=C, tile=tile, stile=stile)
    x_host = np.stack([plan_layout(np.asfortranarray(np.moveaxis(_series_images_host(w, f), 0, -1)))
                       for f in range(F)])                     # [F, C, N1, N0]
    x_dev = torch.from_numpy(x_host).to(dev)
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush():
        flush_buf.fill_(1.0)

    S.capture()
    S.x_static.copy_(x_dev)

    def pair_graph():
        S.replay_forward()
        S.replay_adjoint()

    y_eager = S.forward(x_dev)
    xa_eager = S.adjoint(y_eager)
    torch.cuda.synchronize()

    # ---- parity (untimed): frames vs the oracle, one frame vs the FP64 NUDFT
    parity = {}
    if rank == 0:
        ys = S.split_samples(y_eager)
        errs_f, errs_a = [], []
        for f in (0, F // 2, F - 1):
            B = oracle.OracleNufft(Nd=w["Nd"], omega=oms[f], Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"],
                                   precision="single")
            xf = np.asfortranarray(np.moveaxis(_series_images_host(w, f), 0, -1)[..., :2])
            y_or = B.fft(xf)
            y_gpu = ys[f][:2].cpu().numpy().T
            errs_f.append(oracle.rel_l2(y_gpu, y_or))
            xa_or = B.adj(y_gpu)
            errs_a.append(oracle.rel_l2(xa_eager[f, :2].cpu().numpy().transpose(2, 1, 0), xa_or))
        parity["fwd_rel_err_vs_oracle_max_of_3_frames"] = max(errs_f)
        parity["adj_rel_err_vs_oracle_max_of_3_frames"] = max(errs_a)
        f = 17
        rows = np.random.default_rng(0).choice(oms[f].shape[0], 2048, replace=False)
        x17 = _series_images_host(w, f)[0].astype(np.complex128)
        y_ex = dtft(x17, oms[f][rows], shape=w["Nd"])
        parity["fwd_rel_err_vs_fp64_nudft_frame17"] = oracle.rel_l2(ys[f][0].cpu().numpy()[rows], y_ex)
        parity_gate(parity)

    stats = S.plan.stats()
    launches_per_step = our_launches_per_step(w["Kd"], stats["split_tiles"])

    # ---- batched series from CUDA graphs, device resident -------------------
    for _ in range(args.warmup):
        pair_graph()
    torch.cuda.synchronize()
    sampler = clock_sampler_start(_clock_path(rank)) if rank == 0 else None
    t_graph = max_over_ranks(time_events(pair_graph, args.steps, flush), world, dev)

    def pair_eager():
        S.forward(x_dev, y_eager)
        S.adjoint(y_eager, xa_eager)

    for _ in range(2):
        pair_eager()
    t_eager = time_events(pair_eager, args.steps, flush) / args.steps

    Kp = int(np.prod(w["Kd"]))
    grid = torch.empty((F * C * Kp,), dtype=torch.complex64, device=dev)

    def spread():
        S.plan.interp_adjoint(y_eager, grid, C)

    def gather():
        S.plan.interp_forward(grid, y_eager, C)

    for _ in range(2):
        spread()
        gather()
    t_spread = time_events(spread, args.steps, flush) / args.steps
    t_gather = time_events(gather, args.steps, flush) / args.steps
    if rank == 0:
        load_tail(pair_graph)
    clocks = clock_sampler_stop(sampler, _clock_path(rank), dev.index) if rank == 0 else None
    del grid

    # ---- plain per-call: one single-coil operator per frame ------------------
    ops = [NufftBase(w["Nd"], oms[f], Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], on_gpu=True, max_coils=1).plan
           for f in range(F)]
    x1 = [[x_dev[f, c:c + 1].contiguous() for c in range(C)] for f in range(F)]
    y1 = [torch.empty((1, oms[f].shape[0]), dtype=torch.complex64, device=dev) for f in range(F)]
    xa1 = torch.empty_like(x1[0][0])

    def per_call():
        for f in range(F):
            for c in range(C):
                ops[f].forward(x1[f][c], y1[f], 1)
                ops[f].adjoint(y1[f], xa1, 1)

    per_call()
    per_steps = max(2, args.steps // 4)
    t_percall = time_events(per_call, per_steps, flush) / per_steps
    del ops, x1, y1

    # ---- end to end: host images in, host samples and images out -----------
    x_pin = torch.from_numpy(x_host).pin_memory()
    y_pin = torch.empty((C * S.M_total,), dtype=torch.complex64).pin_memory()
    xa_pin = torch.empty_like(x_pin).pin_memory()

    # A stream of independent series: every step copies its images in from
    # pinned host memory and reads its samples and adjoint images back.  The
    # copies run on two copy streams beside the graphs: step k + 1's images
    # come in and step k's samples go out while step k's adjoint runs; step
    # k's images go out while step k + 1's forward runs.  The timed region
    # ends when the last step's results are in host memory.
    h2d = torch.cuda.Stream(device=dev)
    d2h = torch.cuda.Stream(device=dev)
    ev_in, ev_fwd, ev_adj, ev_y, ev_xa = (torch.cuda.Event() for _ in range(5))

    def e2e_run(steps):
        main = torch.cuda.current_stream()
        h2d.wait_stream(main)
        d2h.wait_stream(main)
        with torch.cuda.stream(h2d):
            S.x_static.copy_(x_pin, non_blocking=True)
            ev_in.record(h2d)
        for k in range(steps):
            main.wait_event(ev_in)              # this step's images are in
            if k > 0:
                main.wait_event(ev_y)           # previous samples read out
            S.replay_forward()
            ev_fwd.record(main)
            if k + 1 < steps:                   # next step's images
                h2d.wait_event(ev_fwd)
                with torch.cuda.stream(h2d):
                    S.x_static.copy_(x_pin, non_blocking=True)
                    ev_in.record(h2d)
            d2h.wait_event(ev_fwd)
            with torch.cuda.stream(d2h):
                y_pin.copy_(S.y_static, non_blocking=True)
                ev_y.record(d2h)
            if k > 0:
                main.wait_event(ev_xa)          # previous images read out
            S.replay_adjoint()
            ev_adj.record(main)
            d2h.wait_event(ev_adj)
            with torch.cuda.stream(d2h):
                xa_pin.copy_(S.xa_static, non_blocking=True)
                ev_xa.record(d2h)
        d2h.synchronize()
        main.synchronize()

    e2e_run(3)
    e2e_steps = max(10, args.steps)
    t0 = time.perf_counter()
    e2e_run(e2e_steps)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    # the overlapped copies must deliver exactly the eager transforms' results
    y_ref = S.forward(x_dev)
    xa_ref = S.adjoint(y_ref)
    if not (torch.equal(y_pin, y_ref.reshape(-1).cpu()) and torch.equal(xa_pin, xa_ref.cpu())):
        print("bench.py: end-to-end results differ from the eager transform", file=sys.stderr, flush=True)
        raise SystemExit(1)

    if rank != 0:
        return
    units = F * C
    ms_per_step = t_graph / args.steps
    hbm, peak_kind = peaks()
    M = S.M_total
    B_alg = C * M * 8 + M * 2 * 4 + F * C * Kp * 8
    dominant = "spread" if t_spread >= t_gather else "gather"
    achieved = B_alg / (max(t_spread, t_gather) * 1e-3) / 1e9
    # CPU baseline: frames 0-3 with one oracle operator per frame
    cpu_ops = [(_cpu_operator(oms[f], w), np.asfortranarray(np.moveaxis(_series_images_host(w, f), 0, -1)))
               for f in range(4)]
    for (op, _), x in cpu_ops:
        op.adj(op.fft(x))
    t0 = time.perf_counter()
    reps = 0
    while True:
        for (op, _), x in cpu_ops:
            op.adj(op.fft(x))
        reps += 1
        if time.perf_counter() - t0 > 10.0 or reps >= 20:
            break
    cpu_per = (time.perf_counter() - t0) / reps
    line = {
        "metric": METRIC, "value": job_value(units, world, ms_per_step), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
        "data": "synthetic",
        "config": config_dict(),
        "execution": {"graph": True, "samples": int(M), "tile": list(tile), "stile": list(stile)},
        "eager": {"ms_per_step": t_eager, "value": units / (t_eager * 1e-3)},
        "per_call": {"value": units / (t_percall * 1e-3), "unit": UNIT, "ms_per_step": t_percall,
                     "calls_per_step": 2 * units,
                     "batched_over_per_call": t_percall / ms_per_step},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "algorithmic_bytes": B_alg,
                     "kernel_ms": {"spread": t_spread, "gather": t_gather}},
        "cpu_baseline": {"value": 4 * C / cpu_per, "unit": UNIT, "cores": os.cpu_count(),
                         "kind": cpu_ops[0][0][1],
                         "sample": "%d x fwd+adj of frames 0-3 (%d coils each), %.2f s each" % (reps, C, cpu_per)},
        "e2e": {"value": units / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(x_pin.numel() * 8),
                "d2h_bytes_per_step": int((y_pin.numel() + xa_pin.numel()) * 8), "seconds_per_step": t_e2e},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "parity": parity,
        "autotune": report,
        "plan": stats,
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    """The workload's launches alone, for a profiler to capture."""
    import torch

    from mrrt.nufft_gb300 import NufftBase

    w = WORKLOAD
    C = w["coils"]
    if w["kind"] == "series":
        # the tile shapes the autotuner picks for this series (fixed here, so
        # that no tuning launches enter a capture)
        from mrrt.nufft_gb300.series import NufftSeries

        S = NufftSeries(w["Nd"], _series_frames(w), Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], coils=C,
                        tile=(32, 16), stile=(8, 8))
        g = torch.Generator(device="cpu").manual_seed(0)
        x_dev = torch.randn(S.image_shape, dtype=torch.complex64, generator=g).to(S.device)
        for _ in range(args.warmup + args.steps):
            S.adjoint(S.forward(x_dev))
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": w["name"], "coils": C, "samples": S.M_total,
                          "stats": S.plan.stats()}))
        return
    if w["kind"] == "grad2d":
        # one differentiable step: forward, backward (image and omega
        # gradients), then a moved trajectory re-binned on the device
        from mrrt.nufft_gb300.autograd import NufftOperator
        from mrrt.nufft_gb300.trajectories import spiral_2d

        om0 = spiral_2d(w["interleaves"], w["samples"])
        op = NufftOperator(w["Nd"], om0, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], max_coils=C)
        dev = op.device
        om = torch.from_numpy(om0.astype(np.float32)).to(dev)
        x = torch.randn((C,) + tuple(w["Nd"]), dtype=torch.complex64, device=dev).requires_grad_(True)
        for k in range(args.warmup + args.steps):
            o = (om + 1e-3 * (k % 2)).requires_grad_(True)
            op.forward(x, o).abs().pow(2).sum().backward()
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": w["name"], "coils": C, "samples": op.M, "stats": op.plan.stats()}))
        return
    omega, x_f = build_inputs()
    A = NufftBase(Nd=w["Nd"], omega=omega, Jd=w["Jd"], Kd=w["Kd"], Ld=w["L"], precision="single",
                  on_gpu=True, max_coils=C)
    P = A.plan
    dev = torch.device("cuda", torch.cuda.current_device())
    x_dev = torch.from_numpy(plan_layout(x_f)).to(dev)
    y_dev = torch.empty((C, A.M), dtype=torch.complex64, device=dev)
    xa_dev = torch.empty_like(x_dev)
    grid = torch.empty((C, int(np.prod(w["Kd"]))), dtype=torch.complex64, device=dev)
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
    ap.add_argument("--workload", default="2d-multicoil-radial", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = WORKLOADS[args.workload]
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
