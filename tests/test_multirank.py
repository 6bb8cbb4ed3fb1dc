"""The multi-rank bench path on CPU: two `gloo` ranks run the host logic that
`bench.py --gpus 2` runs over NCCL (one process per GPU, replicas of the
ensemble with no exchange step).

Checked: the timed region's time is the slowest rank's on every rank; the
whole-job rate counts every rank's units over that time (weak scaling);
each rank steps its own members (distinct seeds, reproducible per rank);
the reference arm's non-zero ranks exit 0 without work."""
import os
import socket
import types

import pytest

WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    import hashlib

    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        t = 1.25 + rank  # rank 1 is the slowest
        t_max = bench.rank_max(t, dist, "cpu")
        rate = bench.job_rate(1000, 5, t_max, WORLD)
        specs = bench.ensemble_specs(2, rank=rank)
        again = bench.ensemble_specs(2, rank=rank)
        digest = hashlib.sha1(b"".join(sp["z"].tobytes() for sp in specs)).hexdigest()
        same = all((a["z"] == b["z"]).all() for a, b in zip(specs, again))
        digests = [None] * WORLD
        dist.all_gather_object(digests, digest)
        ref_rc = None
        if rank != 0:
            args = types.SimpleNamespace(members=256, warmup=3, steps=5, gpus=WORLD, cpu_sample=4096)
            ref_rc = (bench.ensemble_reference(args, rank, WORLD), bench.routing_reference(args, rank, WORLD))
        dist.barrier()
        q.put(dict(rank=rank, t_max=t_max, rate=rate, same=same, digests=digests, ref_rc=ref_rc))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_rate_and_members():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(WORLD)]
    for p in procs:
        p.start()
    try:
        out = {}
        for _ in range(WORLD):
            o = q.get(timeout=120)
            out[o["rank"]] = o
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    for r in range(WORLD):
        o = out[r]
        assert o["t_max"] == 2.25
        assert o["rate"] == pytest.approx(WORLD * 1000 * 5 / 2.25, rel=1e-15)
        assert o["same"]
        assert len(set(o["digests"])) == WORLD  # each rank its own members
    assert out[1]["ref_rc"] == (0, 0)
