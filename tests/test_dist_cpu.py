"""The bench's host-side contract on CPU.

Multi-process path, with two gloo ranks on 127.0.0.1. ``bench.py`` under
torchrun runs one replica per rank. ``dist_setup`` reads the rank from the
environment, ``barrier`` brackets the timed region, and ``max_over_ranks``
reduces each timing to the slowest rank. The reference arm runs on rank 0
only; the other ranks return without work.

Also checked: the JSON line of the reference arm (the CPU port), which needs
no GPU.
"""

import argparse
import contextlib
import io
import json
import os
import socket
import sys
import time

import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    got = {}
    got["setup"] = list(bench.dist_setup())
    bench.barrier(world)
    got["max"] = bench.max_over_ranks(float(10 * (rank + 1)), world, torch.device("cpu"))
    if rank == 1:
        args = argparse.Namespace(gpus=world, steps=3, warmup=3, ref_coils=4)
        buf = io.StringIO()
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(buf):
            bench.run_reference(args)
        got["ref_seconds"] = time.perf_counter() - t0
        got["ref_output"] = buf.getvalue()
    bench.barrier(world)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(got, f)


def test_two_gloo_ranks(tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    for r, got in enumerate(res):
        assert got["setup"] == [world, r, r]
        assert got["max"] == 10.0 * world  # the slowest rank's time on every rank
    assert res[1]["ref_output"] == ""  # the reference arm prints on rank 0 only
    assert res[1]["ref_seconds"] < 5.0  # and does no work elsewhere


def test_reference_arm_line():
    """``bench.py --impl reference`` (the CPU port on the host cores) prints one
    JSON line with the headline metric, a cpu_baseline describing the run and
    an e2e block with the line's own value and no copies."""
    import subprocess

    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench

    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0 and line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_algorithmic_bytes_of_the_headline_workload():
    """The roofline's byte counts at the headline workload: forward and adjoint
    NUFFT as the per-unit formulas give them (8 B per complex64, 4 B per
    coordinate), and the interpolation kernels' own inputs and outputs."""
    sys.path.insert(0, ROOT)
    import bench

    M = 404 * 640
    b = bench.algorithmic_bytes(M)
    assert b["forward"] == 1_029_017_600 and b["adjoint"] == 871_731_200
    # gather: grid read + kdata write + sorted coordinates, phase and index
    assert b["gather"] == 8 * 4 * 16 * 640 * 640 + 8 * 4 * 16 * M + 12 * M == 345_200_640
