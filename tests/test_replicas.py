"""Host logic of the multi-GPU path (replicas only: one independent system
per GPU, no data-path collective) on CPU: two gloo ranks aggregate their
per-rank results the way bench.py does (sums of work, max of time), each
rank integrates a different seed, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    acc, rhs, ms = bench.aggregate_over_ranks(100.0 + rank, 1000.0 * (rank + 1), 5.0 + 3.0 * rank,
                                              device="cpu")
    q.put((rank, acc, rhs, ms, bench.replica_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seeds = set()
    for rank, acc, rhs, ms, seed in out:
        assert acc == 201.0 and rhs == 3000.0 and ms == 8.0  # sum, sum, max over ranks
        seeds.add(seed)
    assert len(seeds) == world  # an independent system per rank


def test_single_process_aggregation_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_over_ranks(7.0, 8.0, 9.0, device="cpu") == (7.0, 8.0, 9.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    args = argparse.Namespace(gpus=2, steps=1, warmup=0)
    assert bench.run_reference(args, world=2, rank=1) is None  # returns without work
    assert capsys.readouterr().out == ""


def test_stage_kernel_naming():
    """The bench names the integrator's stage kernel from the geometry it
    reports: one-lane packed mixed stages run as partner chunks
    (fused_split_kernel), every other geometry as clusters."""
    import bench
    split = {"j_split": 16, "lanes": 1, "mixed_variant": 3}
    assert bench.stage_kernel_name("mixed", split).startswith("fused_split_kernel")
    assert "16 partner chunks" in bench.stage_kernel_name("mixed", split)
    for geo in ({"j_split": 8, "lanes": 2, "mixed_variant": 3},   # clusters, lanes
                {"j_split": 1, "lanes": 1, "mixed_variant": 3},   # one CTA per tile
                {"j_split": 8, "lanes": 1, "mixed_variant": 1}):  # scalar loop
        assert bench.stage_kernel_name("mixed", geo).startswith("fused_stage_kernel")
    assert bench.stage_kernel_name("f64", split).startswith("fused_stage_kernel")


def test_conservation_drift():
    import numpy as np
    import bench
    e0 = {"e": -0.25, "p": np.zeros(3), "l": np.array([0.0, 0.0, 1.0])}
    e1 = {"e": -0.25 * (1 + 2e-9), "p": np.array([3e-12, 0.0, 4e-12]),
          "l": np.array([0.0, 0.0, 1.0 + 1e-11])}
    d = bench.drift(e0, e1)
    assert abs(d["energy_rel_err"] - 2e-9) < 1e-15
    assert abs(d["momentum_drift"] - 5e-12) < 1e-20
    assert abs(d["angular_momentum_drift"] - 1e-11) < 1e-16


def test_pipe_probe_compiles(tmp_path):
    """The throughput probe behind `bench.py --workload pipes` builds for
    sm_103a (nvcc cross-compiles without a GPU); running it needs one."""
    import shutil
    import subprocess
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") \
        else shutil.which("nvcc")
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = os.path.join(ROOT, "ode_prototyping_gb300", "csrc", "probe", "pipes.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-c", src, "-o", str(tmp_path / "pipes.o")], check=True)
