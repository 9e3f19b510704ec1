"""Multi-rank host logic of replica execution (one process per GPU, no
collective on the data path), run as two gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import replicas


def test_shard_covers_every_item_once():
    for n in (0, 1, 5, 64, 4096, 4097):
        for world in (1, 2, 3, 8):
            got = [list(replicas.shard(n, r, world)) for r in range(world)]
            flat = [i for g in got for i in g]
            assert flat == list(range(n))
            sizes = [len(g) for g in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)
    with pytest.raises(ValueError):
        replicas.shard(4, 0, 0)


def test_single_rank_reductions_are_identity():
    assert replicas.max_over_ranks(2.5, 1) == 2.5
    assert replicas.sum_over_ranks(3, 1) == 3.0
    assert replicas.job_rate(10, 2.0, 1) == 5.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    r, w, local = replicas.dist_info()
    replicas.init(w)
    try:
        # each rank owns a shard of the job; its "time" depends on its shard
        items = replicas.shard(10, r, w)
        units = len(items)
        seconds = 1.0 + r  # rank 1 is the slowest
        replicas.barrier(w)
        rate = replicas.job_rate(units, seconds, w)
        tmax = replicas.max_over_ranks(seconds, w)
        total = replicas.sum_over_ranks(units, w)
        np.save(os.path.join(out, f"rank{r}.npy"), np.array([rate, tmax, total, items.start, items.stop, local]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f"rank{r}.npy") for r in range(world)]
    for r, x in enumerate(res):
        rate, tmax, total, lo, hi, local = x
        assert tmax == 2.0 and total == 10.0
        assert rate == pytest.approx(10.0 / 2.0)  # all ranks' units over the slowest rank's time
        assert local == r
    # the shards are disjoint and cover the job
    assert [(int(x[3]), int(x[4])) for x in res] == [(0, 5), (5, 10)]


def test_sweep_shards_are_slices_of_one_sweep(lib):
    """Rank r's sweep sets are sets r*k .. (r+1)*k-1 of the same seeded sweep."""
    from pyblastafterglowmag_gb300 import histories as H
    kw = dict(seed=3, min_steps=8, max_steps=12, max_layers=2)
    recs2, off2, prm2, _ = H.sweep_batch(lib, 2, **kw)
    recs1, off1, prm1, _ = H.sweep_batch(lib, 1, first=1, **kw)
    nb = len(prm1)
    assert nb >= 2 and len(prm2) > nb
    # the second set of the two-set sweep is the one-set shard starting at 1
    tail = slice(len(prm2) - nb, len(prm2))
    assert prm2[tail].tobytes() == prm1.tobytes()
    assert recs2[off2[len(prm2) - nb]:].tobytes() == recs1.tobytes()
