"""Multi-GPU layout (replicas only) on CPU: two gloo ranks run the bench's
whole-job aggregation; the reference arm prints from rank 0 only."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [100.0, 250.0][rank]
    value, t_max = bench.aggregate_over_ranks(local_ms, 3, world, dist, "cpu")
    out[rank] = (value, t_max)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_takes_the_slowest_rank():
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        value, t_max = out[rank]
        assert t_max == 250.0
        assert value == pytest.approx(2 * 3 / 0.25)


def test_single_rank_aggregation():
    import bench
    value, t_max = bench.aggregate_over_ranks(500.0, 4, 1)
    assert t_max == 500.0 and value == pytest.approx(8.0)


def test_reference_arm_only_rank0_reports():
    import argparse
    import bench
    args = argparse.Namespace(warmup=0, steps=1, chi=8, arm=2, dt=0.01, tol=1e-10)
    assert bench.run_reference(args, rank=1, world=2) is None


def test_reference_arm_line_states_its_timing():
    """Rank 0's line: value and ms_per_step describe the same modelled sweep,
    the wall time actually sampled is reported beside it, and the recorded
    full-sweep check is attached only at the size it was measured at."""
    import argparse
    import bench
    args = argparse.Namespace(warmup=1, steps=2, chi=8, arm=2, dt=0.01, tol=1e-10, precision="mixed")
    line = bench.run_reference(args, rank=0, world=1)
    assert line["impl"] == "reference"
    assert line["ms_per_step"] == pytest.approx(1000.0 / line["value"])
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["value"] == line["value"]
    assert line["timing"]["sampled_wall_seconds"] > 0.0
    assert line["timing"]["model_check"] is None
    assert bench.MODEL_CHECK["full_sweep_seconds"] > 0.0
