"""Host side of the row-shard protocol (cuscan_gb300.shards) with gloo ranks on the CPU: the
row partition, the key encoding, the all-gather of unequal row blocks and the all-reduce MIN of
the per-row Borůvka keys. Each rank's keys for its own rows come from the oracle here (the
device path is covered by tests/test_gpu_shards.py); the reduced keys must equal the keys of
all rows computed at once."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from cuscan_gb300 import shards


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_rows_partition_every_row_once():
    for n in (1, 2, 7, 100, 1001):
        for world in (1, 2, 3, 8):
            blocks = [shards.shard_rows(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
    with pytest.raises(ValueError):
        shards.shard_rows(10, 2, 2)


def test_candidate_keys_order_like_the_device_keys():
    w = np.array([1.5, -0.0, 0.0, np.inf, np.nan, 2.0], np.float32)
    dst = np.array([3, 4, 2, 1, 0, -1], np.int32)
    k = shards.candidate_keys(w, dst)
    assert k[1] == np.uint64(4) and k[2] == np.uint64(2)       # -0 folds onto +0
    assert k[4] == shards.KEY_NONE and k[5] == shards.KEY_NONE  # NaN, no candidate
    assert k[2] < k[1] < k[0] < k[3]
    assert np.all(k[k != shards.KEY_NONE] < np.uint64(1) << np.uint64(63))


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(3)
        n, d = 517, 9
        x = rng.integers(-4, 5, size=(n, d)).astype(np.float32)  # many exact ties
        core = rng.integers(0, 3, size=n).astype(np.float32)
        comps = rng.integers(0, 7, size=n).astype(np.int32)
        begin, end = shards.shard_rows(n, rank, world)
        keys = np.full(n, shards.KEY_NONE, np.uint64)
        w, j = O.boruvka_candidate_rows(x, core, comps, begin, end)
        keys[begin:end] = shards.candidate_keys(w, np.where(j >= n, -1, j))
        reduced = shards.reduce_row_keys(keys)
        block = np.arange(begin, end, dtype=np.int64)[:, None] * np.array([[1, -1, 7]])
        gathered = shards.gather_rows(block, n)
        if rank == 0:
            wa, ja = O.boruvka_candidates(x, core, comps)
            np.savez(out, reduced=reduced, gathered=gathered,
                     expected=shards.candidate_keys(wa, np.where(ja >= n, -1, ja)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_keys_reduced_over_ranks_equal_all_rows(tmp_path, world):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    port = _free_port()
    out = str(tmp_path / "keys.npz")
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = np.load(out)
    np.testing.assert_array_equal(res["reduced"], res["expected"])
    n = res["gathered"].shape[0]
    np.testing.assert_array_equal(res["gathered"],
                                  np.arange(n)[:, None] * np.array([[1, -1, 7]]))
