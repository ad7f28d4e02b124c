"""The component reduction variant that allocates nothing (cuscan_component_reduce_noalloc).

It exists for callers that cannot allocate device memory when they need the reduction (their
device memory belongs to another framework's pool, or the implicit synchronisation of
cudaMalloc/cudaFree is not acceptable on their path). Its tile scratch is a static device array
shared by every call. The GPU test checks its results against the allocating entry point,
cuscan_component_reduce, bit for bit, on two calls in a row with different plans, so that what
the first call leaves in the shared array cannot leak into the second.
"""
from __future__ import annotations

import numpy as np
import pytest

from cuscan_gb300 import _lib
from oracle import oracle as O


def test_noalloc_rejects_plans_beyond_the_static_capacity():
    n = _lib.NOALLOC_MAX_TILES + 10
    with pytest.raises(OverflowError, match="at most"):
        _lib.component_reduce_noalloc(None, None, None, None, None, None, n,
                                      _lib.NOALLOC_MAX_TILES + 1, 1, None, None)


@pytest.mark.gpu
def test_noalloc_matches_allocating_reduce_on_two_calls(gpu_ctx):
    torch = pytest.importorskip("torch")

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def problem(seed, n, comps, tile):
        rng = np.random.default_rng(seed)
        labels = rng.integers(0, comps, size=n).astype(np.int32)
        plan = O.component_plan(labels, tile)
        w = rng.integers(0, 40, size=n).astype(np.float32)
        w[rng.random(n) < 0.05] = -0.0
        w[rng.random(n) < 0.05] = np.inf
        w[rng.random(n) < 0.01] = np.nan
        dst = rng.integers(0, n, size=n).astype(np.int32)
        dst[rng.random(n) < 0.05] = -1
        dst[rng.random(n) < 0.01] = n + 5
        return w, dst, plan

    stream = torch.cuda.current_stream().cuda_stream
    for seed, n, comps, tile in [(1, 20000, 300, 64), (2, 9000, 7, 512)]:
        w, dst, plan = problem(seed, n, comps, tile)
        c = plan.offsets.shape[0] - 1
        p = plan.tile_starts.shape[0]
        ins = [dev(a) for a in (w, dst, plan.members, plan.tile_starts, plan.tile_ends,
                                plan.partial_offsets)]
        ptrs = [t.data_ptr() for t in ins]
        ref_w = torch.empty(c, dtype=torch.float32, device="cuda")
        ref_m = torch.empty((c, 5), dtype=torch.int32, device="cuda")
        gpu_ctx.component_reduce(*ptrs, n, p, c, ref_w.data_ptr(), ref_m.data_ptr(), stream)
        got_w = torch.full((c,), 7.0, dtype=torch.float32, device="cuda")
        got_m = torch.full((c, 5), -7, dtype=torch.int32, device="cuda")
        _lib.component_reduce_noalloc(*ptrs, n, p, c, got_w.data_ptr(), got_m.data_ptr(), stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got_m.cpu().numpy(), ref_m.cpu().numpy())
        np.testing.assert_array_equal(got_w.cpu().numpy().view(np.uint32),
                                      ref_w.cpu().numpy().view(np.uint32))
        ew, em = O.component_reduce(w, dst, plan)
        np.testing.assert_array_equal(got_m.cpu().numpy(), em)
