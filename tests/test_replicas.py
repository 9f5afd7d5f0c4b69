"""Replicas path of bench.py on CPU: world-size-2 gloo ranks agree on the
job time (the slowest rank's) and the whole-job throughput.  Coils and
frames shard with no exchange step, so this host logic is all that N>1 adds."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, world, torch.device("cpu"))
        out[rank] = (t, bench.job_value(32, world, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_job_time():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]
    t, v = res[0]
    assert t == pytest.approx(2.5)
    assert v == pytest.approx(2 * 32 / 2.5e-3)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(3.0, 1, None) == 3.0
    assert bench.job_value(32, 1, 4.0) == pytest.approx(8000.0)


def test_bench_parity_gate():
    """bench.py stops before timing when the transform misses the metric's
    accuracy bar; the oracle's own error figures are reported, not gated."""
    import bench

    bench.parity_gate({"fwd_rel_err_vs_oracle": 2.9e-7, "adj_rel_err_vs_fp64_oracle": 3.7e-5,
                       "oracle_adj_rel_err_vs_fp64_oracle": 0.5})
    for bad in (0.93, 2e-4, float("nan")):
        with pytest.raises(SystemExit):
            bench.parity_gate({"fwd_rel_err_vs_oracle": bad})


def test_own_kernel_launch_count_follows_the_fft_path():
    """gpu_launches: per pair, the row pass, the strided passes and the
    interpolation kernel each way when every axis length has an own FFT pass;
    pad / crop around the interpolation kernels (plus the last-axis pass when
    only its length is supported) otherwise; one reduce when tiles split."""
    import bench

    assert bench.our_launches_per_step((512, 512), 1) == 7
    assert bench.our_launches_per_step((256, 256, 256), 1) == 9
    assert bench.our_launches_per_step((384, 384), 0) == 6
    assert bench.our_launches_per_step((40, 512), 0) == 6
    assert bench.our_launches_per_step((512, 1024), 1) == 5
    assert bench.our_launches_per_step((1024,), 0) == 4
