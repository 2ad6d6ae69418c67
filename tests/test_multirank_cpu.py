"""bench.py's multi-GPU host logic on two gloo ranks (CPU): rendezvous, one
independent synthetic sequence per rank (seed + rank, no data exchange), the
barrier, the max-over-ranks step time and the whole-job value."""
from __future__ import annotations

import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import hashlib

    import torch.distributed as dist

    import bench

    bench.set_config("1")
    w, r = bench.dist_init(torch)
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    frames, flows = bench.make_workload(r)
    digest = hashlib.sha1(b"".join(f.tobytes() for f in frames)).hexdigest()
    digests = [None] * w
    dist.all_gather_object(digests, digest)
    bench.barrier(torch, w)
    local_ms = 10.0 + 5.0 * r
    slowest = bench.max_over_ranks(torch, w, local_ms)
    px = bench.PAIRS * bench.W * bench.H
    out[r] = (digests, slowest, bench.aggregate_value(w, px, slowest), px)
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    digests, slowest, value, px = res[0]
    assert len(set(digests)) == world, "each rank must draw its own sequence"
    assert res[1][0] == digests
    assert slowest == res[1][1] == 15.0
    assert value == pytest.approx(world * px / 15e-3 / 1e6)
