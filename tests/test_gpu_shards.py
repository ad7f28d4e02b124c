"""Row shards on the device: two or three processes (gloo ranks) on GPU 0 each run the kNN rows
and the Borůvka candidates of their share of the rows through the C ABI (cuscan_exact_knn over
the shard's rows, cuscan_shard_seed, cuscan_shard_round_keys, cuscan_shard_round_merge),
exchange them on the host, and must end with the single-process fit core bit for bit: kNN rows,
core distances, MST edges in merge order and the f64 total weight. The ranks' kernels never
wait on one another; they meet only in the host collectives."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from cuscan_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, x, ms, out):
    import torch.distributed as dist

    import cuscan_gb300 as cg
    from cuscan_gb300 import shards
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ctx = cg.context(0)
        res = shards.fit_core_sharded(ctx, x, ms)
        np.savez(f"{out}_{rank}.npz", **{k: np.asarray(v) for k, v in res.items()})
    finally:
        dist.destroy_process_group()


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name,world", [("blobs", 2), ("aniso", 2), ("blobs", 3)])
def test_row_shards_equal_the_single_process_fit(gpu_ctx, tmp_path, name, world):
    import multiprocessing as mp

    if name == "blobs":
        x, ms = synthetic.blobs_with_noise(n=6001, d=16, centers=10, seed=17), 10
    else:
        x, ms = synthetic.anisotropic_mixture(n=9000, d=64, components=12, seed=19), 10
    ctx = mp.get_context("spawn")
    port = _free_port()
    out = str(tmp_path / "shard")
    procs = [ctx.Process(target=_rank, args=(r, world, port, x, ms, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    one = gpu_ctx.fit_core(x, ms, _lib.PRECISION_PLAIN)
    for r in range(world):
        got = np.load(f"{out}_{r}.npz")
        np.testing.assert_array_equal(got["knn_ids"], one["knn_ids"])
        np.testing.assert_array_equal(_bits(got["knn_sq"]), _bits(one["knn_sq"]))
        np.testing.assert_array_equal(_bits(got["core_sq"]), _bits(one["core_sq"]))
        np.testing.assert_array_equal(got["src"], one["src"])
        np.testing.assert_array_equal(got["dst"], one["dst"])
        np.testing.assert_array_equal(_bits(got["wsq"]), _bits(one["wsq"]))
        assert int(got["rounds"]) == one["stats"]["rounds"]
        assert float(got["mst_weight"]) == one["stats"]["mst_weight"]
        b, e = got["rows"]
        assert e - b in (x.shape[0] // world, x.shape[0] // world + 1)
