"""Multi-process (gloo, world size 2) check of the replica sharding on the CPU: each
rank computes its curve shard with the oracle and rank 0 gathers the per-curve
results, which must equal the single-process result."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from gtrap_gb300.shard import gather_rows, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 64, 1025):
        for w in (1, 2, 3, 8):
            rs = [shard_range(n, r, w) for r in range(w)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, result_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from gtrap_gb300 import synth
        wl = synth.plain_bls(nq=6, n=512, nf=24, nb=128, seed=3, n_transit=3)
        a, b = shard_range(wl.lc.shape[1], rank, world)
        sr = oracle.bls(wl.lc[:, a:b], wl.tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin,
                        wl.df, nthreads=1)[0]
        full = gather_rows(sr, rank, world, wl.lc.shape[1])
        if rank == 0:
            np.save(result_path, full)
    finally:
        dist.destroy_process_group()


def test_two_rank_gather_equals_single(tmp_path):
    import oracle
    from gtrap_gb300 import synth
    oracle.build()
    path = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(2, _free_port(), path), nprocs=2, start_method="spawn")
    wl = synth.plain_bls(nq=6, n=512, nf=24, nb=128, seed=3, n_transit=3)
    ref = oracle.bls(wl.lc, wl.tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df, nthreads=1)[0]
    np.testing.assert_array_equal(np.load(path), ref)
