"""The N>1 path on CPU: two gloo ranks shard the pages, encode their share
(with the oracle, as there is no GPU here) and combine only the timing.
Together the ranks cover every page exactly once, each page's bytes are the
same as in a single-process run, and the job time is the slowest rank's."""
import hashlib
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from jp2lam_gb300 import replicas

PAGES = [(97, 61, 1, 85), (64, 64, 3, 100), (130, 77, 1, 50), (33, 120, 3, 75), (200, 150, 1, 99)]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _page(i):
    from jp2lam_gb300._native import synth_page
    w, h, c, q = PAGES[i]
    return synth_page(w, h, c, 4000 + i, photo_w=w // 3, photo_h=h // 3), w, h, c, q


def _rank(rank, world, port, out):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from tests import oracle_lib
        orc = oracle_lib.load()
        mine = replicas.shard(list(range(len(PAGES))), rank, world)
        digests = {}
        for i in mine:
            px, w, h, c, q = _page(i)
            digests[i] = hashlib.sha256(orc.encode(px, w, h, c, q, 1)).hexdigest()
        gathered = [None] * world
        td.all_gather_object(gathered, digests)
        # each rank reports a different "time"; the job time is the largest
        job = replicas.max_over_ranks(1.0 + rank)
        out[rank] = (gathered, job)
    finally:
        td.destroy_process_group()


def test_shard_covers_pages_once():
    for world in (1, 2, 3, 7):
        seen = sorted(i for r in range(world) for i in replicas.shard(list(range(10)), r, world))
        assert seen == list(range(10))
    with pytest.raises(ValueError):
        replicas.shard([1, 2], 2, 2)
    assert replicas.whole_job_rate(8.4, 2, 0.5) == pytest.approx(33.6)
    assert replicas.max_over_ranks(3.5) == 3.5  # no process group


def test_two_gloo_ranks(orc):
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=180)
            assert p.exitcode == 0
        res = dict(out)
    assert set(res) == {0, 1}
    gathered, job0 = res[0]
    _, job1 = res[1]
    assert job0 == job1 == 2.0
    merged = {}
    for d in gathered:
        assert not set(d) & set(merged)
        merged.update(d)
    assert sorted(merged) == list(range(len(PAGES)))
    for i, dig in merged.items():
        px, w, h, c, q = _page(i)
        assert dig == hashlib.sha256(orc.encode(px, w, h, c, q, 1)).hexdigest()
