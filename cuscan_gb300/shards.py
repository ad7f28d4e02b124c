"""One fit split by query rows over the ranks of a torch.distributed group.

Every rank holds all n points. Rank r owns the rows [r n / w, (r + 1) n / w) and computes
their kNN rows and, each Borůvka round, their cheapest cross-component edges; the ranks exchange
these on the host and every rank merges the same rounds, so that all ranks end with the same
minimum spanning tree, bit for bit the tree of a single-device fit (the plain f32 form):

1. kNN rows of the shard (the exact f32 kernel, ``cuscan_exact_knn`` over the shard's query
   rows), then an all-gather of the rows;
2. core distances and the kNN seed forest on every rank (``cuscan_shard_seed``);
3. each round: per-row keys ``(canonical weight bits << 32) | destination`` of the shard's rows
   (``cuscan_shard_round_keys``, ~0 elsewhere), an all-reduce MIN of the keys over the ranks,
   and the same merge on every rank (``cuscan_shard_round_merge``), until one component
   remains.

The reference runs the same steps on one device (crates/hdbscan/src/estimator.rs:524-874); the
per-row rule is crates/hdbscan/src/kernels/boruvka.rs:68-140. The exchange is the only
collective: the kNN rows once, then 8 n bytes per round. Kernels of different ranks never wait
on one another; they meet only in the host collectives.
"""
from __future__ import annotations

import numpy as np

KEY_NONE = np.uint64(0xFFFFFFFFFFFFFFFF)
_SIGNED_NONE = np.int64(np.iinfo(np.int64).max)


def shard_rows(n: int, rank: int, world: int) -> tuple[int, int]:
    """The contiguous row block [begin, end) rank `rank` of `world` owns."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    return n * rank // world, n * (rank + 1) // world


def candidate_keys(weights: np.ndarray, destinations: np.ndarray) -> np.ndarray:
    """Host form of a row key: (canonical f32 bits of the weight << 32) | destination, with -0
    folded onto +0 and rows without a candidate (negative destination) or with a NaN weight set
    to KEY_NONE. Keys of non-negative weights stay below 2^63, so they order alike as signed
    integers."""
    w = np.ascontiguousarray(weights, np.float32)
    dst = np.asarray(destinations)
    bits = w.view(np.uint32).astype(np.uint64)
    bits[(bits & np.uint64(0x7FFFFFFF)) == 0] = 0
    keys = (bits << np.uint64(32)) | dst.astype(np.int64).astype(np.uint32).astype(np.uint64)
    keys[np.isnan(w) | (dst < 0)] = KEY_NONE
    return keys


def reduce_row_keys(keys: np.ndarray, group=None) -> np.ndarray:
    """All-reduce MIN of per-row keys (uint64, KEY_NONE = no candidate) over the group."""
    import torch
    import torch.distributed as dist

    k = np.ascontiguousarray(keys, np.uint64)
    if np.any((k >= np.uint64(1) << np.uint64(63)) & (k != KEY_NONE)):
        raise ValueError("row keys must be below 2^63 (non-negative weights)")
    signed = k.view(np.int64).copy()
    signed[k == KEY_NONE] = _SIGNED_NONE
    t = torch.from_numpy(signed)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    out = t.numpy().copy()
    none = out == _SIGNED_NONE
    out = out.view(np.uint64)
    out[none] = KEY_NONE
    return out


def gather_rows(local: np.ndarray, n: int, group=None) -> np.ndarray:
    """All-gather of every rank's row block (the blocks of shard_rows) into the full array,
    byte for byte."""
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    sizes = [shard_rows(n, r, world)[1] - shard_rows(n, r, world)[0] for r in range(world)]
    if local.shape[0] != sizes[rank]:
        raise ValueError("local block does not match this rank's shard")
    row_bytes = int(np.prod(local.shape[1:], dtype=np.int64)) * local.dtype.itemsize
    pad = np.zeros((max(sizes), row_bytes), np.uint8)
    pad[:local.shape[0]] = np.ascontiguousarray(local).reshape(local.shape[0], -1).view(
        np.uint8).reshape(local.shape[0], row_bytes)
    t = torch.from_numpy(pad)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    rows = np.concatenate([o.numpy()[:sizes[r]] for r, o in enumerate(outs)])
    return rows.view(local.dtype).reshape((n,) + local.shape[1:])


def fit_core_sharded(ctx, x: np.ndarray, min_samples: int, group=None) -> dict:
    """The exact fit core of `x` (every rank passes the same points) with the query rows split
    over the group's ranks. Returns the kNN rows, core distances and MST edges in merge order
    (the same on every rank), the f64 total weight and this rank's rows."""
    import torch
    import torch.distributed as dist

    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    if n < 2:
        raise ValueError("a fit needs at least two rows")
    k = min(int(min_samples), n - 1)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    begin, end = shard_rows(n, rank, world)
    dev = torch.device("cuda", ctx.device)
    stream = ctx.stream
    xd = torch.from_numpy(x).to(dev)
    # 1. kNN rows of the shard, then every rank's rows
    ids = torch.empty((max(end - begin, 1), k), dtype=torch.int32, device=dev)
    dsq = torch.empty((max(end - begin, 1), k), dtype=torch.float32, device=dev)
    if end > begin:
        ctx.exact_knn(xd.data_ptr() + begin * d * 4, end - begin, xd.data_ptr(), n, d, k, 1,
                      begin, 1, ids.data_ptr(), dsq.data_ptr(), stream)
    torch.cuda.synchronize(dev)
    knn_ids = gather_rows(ids.cpu().numpy()[:end - begin], n, group)
    knn_sq = gather_rows(dsq.cpu().numpy()[:end - begin], n, group)
    # 2. core distances and the seed forest, the same on every rank
    ids_all = torch.from_numpy(knn_ids).to(dev)
    dsq_all = torch.from_numpy(knn_sq).to(dev)
    core = torch.empty(n, dtype=torch.float32, device=dev)
    labels = torch.empty(n, dtype=torch.int32, device=dev)
    src = torch.empty(n, dtype=torch.int32, device=dev)
    dst = torch.empty(n, dtype=torch.int32, device=dev)
    wsq = torch.empty(n, dtype=torch.float32, device=dev)
    edges, comps = ctx.shard_seed(n, d, min_samples, ids_all.data_ptr(), dsq_all.data_ptr(),
                                  core.data_ptr(), labels.data_ptr(), src.data_ptr(),
                                  dst.data_ptr(), wsq.data_ptr(), stream)
    seed_edges = edges
    # 3. rounds: own rows' keys, all-reduce MIN, the same merge everywhere
    keys = torch.empty(n, dtype=torch.int64, device=dev)
    rounds, weight = 0, float("nan")
    while comps > 1:
        if rounds > 64:
            raise RuntimeError("Boruvka did not converge")
        ctx.shard_round_keys(xd.data_ptr(), core.data_ptr(), labels.data_ptr(), n, d, begin,
                             end, keys.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        reduced = reduce_row_keys(keys.cpu().numpy().view(np.uint64), group)
        keys.copy_(torch.from_numpy(reduced.view(np.int64)))
        torch.cuda.synchronize(dev)
        edges, comps, weight = ctx.shard_round_merge(
            xd.data_ptr(), core.data_ptr(), labels.data_ptr(), n, d, keys.data_ptr(),
            src.data_ptr(), dst.data_ptr(), wsq.data_ptr(), stream)
        rounds += 1
    if rounds == 0:  # the seed alone spans the points: only the total weight is left
        _, _, weight = ctx.shard_round_merge(
            xd.data_ptr(), core.data_ptr(), labels.data_ptr(), n, d, keys.data_ptr(),
            src.data_ptr(), dst.data_ptr(), wsq.data_ptr(), stream)
    torch.cuda.synchronize(dev)
    if edges != n - 1:
        raise RuntimeError("Boruvka produced an incomplete spanning tree")
    return {
        "knn_ids": knn_ids, "knn_sq": knn_sq, "core_sq": core.cpu().numpy(),
        "src": src.cpu().numpy()[:edges].astype(np.uint32),
        "dst": dst.cpu().numpy()[:edges].astype(np.uint32),
        "wsq": wsq.cpu().numpy()[:edges], "rounds": rounds, "seed_edges": seed_edges,
        "mst_weight": weight, "rows": (begin, end),
    }


__all__ = ["shard_rows", "candidate_keys", "reduce_row_keys", "gather_rows",
           "fit_core_sharded", "KEY_NONE"]
