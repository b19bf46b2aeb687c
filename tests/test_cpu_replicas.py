"""Multi-rank replica logic (axgb.replicas) on CPU with the gloo backend,
world size 2: the max-over-ranks step time, the whole-job rate and the
sharding of independent work units."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from axgb import replicas
    replicas.init("gloo")
    try:
        r, w, local = replicas.world_info()
        replicas.barrier()
        t = replicas.max_over_ranks(1.5 + r)  # per-rank "step time"
        rate = replicas.aggregate_rate(100.0, t, w)
        q.put((r, w, local, t, rate, replicas.shard(10, r, w)))
    finally:
        replicas.finalize()


def test_replicas_gloo_world2():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 2.5 for o in out)  # max over ranks
    assert all(abs(o[4] - 2 * 100.0 / 2.5) < 1e-12 for o in out)
    assert out[0][5] == (0, 5) and out[1][5] == (5, 10)


def test_shard_covers_units():
    from axgb import replicas
    for n in (0, 1, 7, 16, 17):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
