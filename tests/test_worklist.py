"""Multi-GPU work-list host logic (fftgal_gb300/worklist.py) with two gloo
ranks on the CPU: round-robin sharding covers every catalog once, the whole-job
time is the maximum over ranks, and the per-catalog bin tables gather on rank 0
in catalog order.  The GPU work is replaced by a stand-in grid whose result
names the catalog it was given."""
import os
import socket

import numpy as np
import pytest

from fftgal_gb300 import worklist


class FakeGrid:
    def power_batch_f32(self, cats, V, los, dK, Nmu=3):
        return [dict(first_x=float(c[0][0]), n=len(c[0]), V=float(v), Nmu=Nmu) for c, v in zip(cats, V)]


def _catalogs(n):
    return [(np.full(5 + i, float(i)), np.zeros(5 + i), np.zeros(5 + i)) for i in range(n)]


def test_shard_covers_every_catalog_once():
    for n in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in worklist.shard(n, r, world))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        worklist.shard(4, 2, 2)


def test_single_process():
    cats = _catalogs(5)
    res = worklist.power_worklist(FakeGrid(), cats, 1e9, (0, 0, 1), 0.1, Nmu=4)
    assert [r["first_x"] for r in res] == [0.0, 1.0, 2.0, 3.0, 4.0]
    assert worklist.max_over_ranks(2.5) == 2.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 9
        cats = _catalogs(n)
        Vs = [1e9 + i for i in range(n)]
        res = worklist.power_worklist(FakeGrid(), cats, Vs, (0, 0, 1), 0.1, Nmu=3, rank=rank, world=world)
        t = worklist.max_over_ranks(1.0 + rank)
        # a catalog claimed by two ranks is an error on rank 0
        dup = None
        try:
            worklist.gather_tables({0: "x"}, 1)
        except RuntimeError as e:
            dup = str(e)
        with open(os.path.join(outdir, f"rank{rank}.txt"), "w") as fh:
            if rank == 0:
                fh.write(repr([(r["first_x"], r["n"], r["V"]) for r in res]) + "\n")
                fh.write(repr(dup) + "\n")
            else:
                fh.write(repr(res) + "\n")
            fh.write(repr(t) + "\n")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r0 = (tmp_path / "rank0.txt").read_text().splitlines()
    r1 = (tmp_path / "rank1.txt").read_text().splitlines()
    got = eval(r0[0])
    assert got == [(float(i), 5 + i, 1e9 + i) for i in range(9)]
    assert "measured twice" in eval(r0[1])
    assert r1[0] == "None"
    assert eval(r0[2]) == 2.0 and eval(r1[1]) == 2.0
