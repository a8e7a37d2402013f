"""The bench's host logic on CPU.  The multi-rank path (gloo, world size 2):
the slowest rank's time is the job's, the throughput counts every rank's box,
and under torchrun the reference arm runs on rank 0 alone while the other
ranks exit cleanly (the GPU arm's ranks are independent replicas with no
collective on the data path).  Also the roofline's algorithmic bytes and the
seeded batch of boxes."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    slowest = bench.max_over_ranks(2.0 + 3.0 * rank, world, device="cpu")
    value = bench.job_throughput(1000, world, slowest)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"slowest": slowest, "value": value}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo(tmp_path):
    import torch.multiprocessing as mp
    world, port = 2, free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    for r in range(world):
        d = json.loads((tmp_path / f"r{r}.json").read_text())
        assert d["slowest"] == 5.0                      # rank 1's 5 ms
        assert d["value"] == pytest.approx(2 * 1000 / 5e-3)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(10, 1, 2.0) == pytest.approx(5000.0)


def test_reference_arm_under_torchrun_two_ranks(tmp_path):
    """`--impl reference` launched as the multi-GPU bench is: rank 0 prints one
    JSON line, the other rank exits 0 without output."""
    env = dict(os.environ, OMP_NUM_THREADS="2", CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}",
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--nside", "32", "--grid", "32",
           "--box", "1000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(tmp_path),
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "particles/s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    # measured on the whole workload every step, not extrapolated from a sample
    assert "whole workload" in d["cpu_baseline"]["sample"]
    assert d["ms_per_step"] == pytest.approx(1e3 * sum(d["stages_s"].values()), rel=0.05)


def test_algorithmic_bytes_match_the_stated_figures():
    """The roofline's numerators: deposit = particles read once + FP32 padded
    grid written once; binning = the half-complex spectrum read once.  512^3:
    1.61 GB + 0.539 GB and 0.539 GB; 1024^3: 12.88 GB + 4.30 GB and 4.30 GB."""
    sys.path.insert(0, ROOT)
    import bench
    dep, binb = bench.algorithmic_bytes(512 ** 3, 512)
    assert dep == 512 ** 3 * 12 + 4 * 512 * 512 * 2 * 257
    assert round(dep / 1e9, 2) == round(1.611 + 0.539, 2) and round(binb / 1e9, 3) == 0.539
    dep, binb = bench.algorithmic_bytes(1024 ** 3, 1024)
    assert round((dep - 1024 ** 3 * 12) / 1e9, 2) == 4.30 and round(binb / 1e9, 2) == 4.30
    dep_m, _ = bench.algorithmic_bytes(1000, 64, var_masses=True)
    assert dep_m - bench.algorithmic_bytes(1000, 64)[0] == 4000


def test_box_batch_is_seeded_and_in_range():
    sys.path.insert(0, ROOT)
    import bench
    a, box = bench.box_batch()
    b, _ = bench.box_batch()
    assert a == b and len(a) == 16 and box == 25000.0
    assert all(1e5 <= c <= 3e7 and g in (128, 256) for c, g, _ in a)


def test_particle_orders_are_permutations_of_the_lattice():
    """--order morton and --order random reorder the same particles: a Morton
    code sorts (x, y, z) with the bits interleaved, and both orders hold every
    lattice particle once (the deposit does not depend on the order)."""
    import argparse
    import numpy as np
    import torch
    sys.path.insert(0, ROOT)
    import bench
    perm = bench.morton_order(8, "cpu").numpy()
    assert np.array_equal(np.sort(perm), np.arange(8 ** 3))
    x, y, z = perm // 64, (perm // 8) % 8, perm % 8
    assert list(zip(x[:8], y[:8], z[:8])) == [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1),
                                              (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]
    base = dict(workload="zeldovich", nside=16, box=1000.0)
    lattice = bench.positions(argparse.Namespace(order="lattice", **base), seed=3)
    for order in ("morton", "random"):
        other = bench.positions(argparse.Namespace(order=order, **base), seed=3)
        assert other.shape == lattice.shape and not np.array_equal(other, lattice)
        key = lambda a: a[np.lexsort(a.T[::-1])]
        assert np.array_equal(key(other), key(lattice))
