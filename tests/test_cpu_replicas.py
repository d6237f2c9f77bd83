"""Multi-process replicas on CPU (gloo, world size 2).

Each rank renders its own range of sample passes of the same image (here
with the CPU oracle, the GPU path's checker) and the films are reduced to
rank 0, which must equal one render of all passes: counts exactly, sums to
FP32 rounding of the different addition order.
"""
import os
import socket

import numpy as np
import pytest

import helpers


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, scene_path, spp, out_path):
    import torch.distributed as dist

    from oracle import port as oport
    from orion_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = oport.Scene.load(scene_path)
        first, n = replicas.pass_range(rank, world, spp)
        film, _ = sc.render(spp=n, first_pass=first, threads=1)
        count = np.full(film.shape[:2], n, np.uint32)
        s, c = replicas.reduce_film(film, count)
        if rank == 0:
            np.savez(out_path, sum=s, count=c)
    finally:
        dist.destroy_process_group()


def test_pass_ranges_partition_the_passes():
    from orion_gb300 import replicas
    ranges = [replicas.pass_range(r, 4, 3, first_pass=5) for r in range(4)]
    passes = [p for f, n in ranges for p in range(f, f + n)]
    assert passes == list(range(5, 17))
    with pytest.raises(ValueError):
        replicas.pass_range(4, 4, 3)


def test_two_gloo_ranks_equal_one_render(built, tmp_path):
    import torch.multiprocessing as mp

    from oracle import port as oport
    path = helpers.write_scene("cornell", str(tmp_path / "c"), res=16, spp=2)
    out = str(tmp_path / "reduced.npz")
    world, spp = 2, 2
    mp.start_processes(_rank_main, args=(world, _free_port(), path, spp, out), nprocs=world, join=True,
                       start_method="spawn")
    got = np.load(out)
    ref, _ = oport.Scene.load(path).render(spp=world * spp, first_pass=0, threads=1)
    assert np.array_equal(got["count"], np.full(ref.shape[:2], world * spp, np.uint32))
    assert np.allclose(got["sum"], ref, rtol=1e-5, atol=1e-6)
