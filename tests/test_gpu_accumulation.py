"""Adversarial checks of the tensor-core accumulation model and of the screens' lower bound.

The screens' lower bound of a squared distance assumes (refined.cu, error_coefficients) that the
tcgen05 f32 accumulation of the K 16-bit products of a tile entry (K = d_pad, or 3 d_pad for
split-bf16 operands) is off from the exact sum of those products by at most

    K * 2^-23 * sum |a_f b_f|                                  (the assumed model),

two f32 units in the last place per product. The first test drives the accumulator with
operands built to stress it and requires the observed worst case to stay within a quarter of
the model:

* mixed exponents across K (powers of two from 2^-30 to 2^30, random signs);
* heavy cancellation (rows [a, b] against [a, -b] with ||a|| close to ||b||);
* all-equal magnitudes (+-(1 + m 2^-7): 16-bit products, integer-like sums);
* one giant coordinate per row among small ones;
* magnitudes ramping up along K, so the largest products arrive last;

with bf16 and fp16 operands (the latter scaled by the fp16 screens' own power-of-two scale)
at K blocks of 64 and 128 (d = 64, 100, 128), and split-bf16 operands at d = 64 (the widest
rows a split tile serves).

The second test checks the bound itself: fmaf(-cm_r, m_c, fmaf(-2, acc, pb_c) + ps_r), the
epilogue's bound in screen units, must not exceed the reference's f32 squared distance
(sequential fused multiply-adds, the oracle's arithmetic) on general f32 data far from and near
the origin, in every operand format.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RATIO_MAX = 0.25
FORMATS = {"bf16": 0, "fp16": 1, "split": 2}


def _to16(x: np.ndarray, fp16: bool) -> np.ndarray:
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32))
    return t.to(torch.float16 if fp16 else torch.bfloat16).to(torch.float32).numpy()


def _operands(x: np.ndarray, fmt: str, scale: float):
    """The 16-bit values the tensor core multiplies, as float64 rows (a, b): entry (i, j) of
    the tile is sum_f a[i, f] b[j, f]."""
    if fmt == "split":
        hi = _to16(x, False)
        lo = _to16(x - hi, False)  # x - hi is exact in f32
        return (np.concatenate([hi, lo, hi], axis=1).astype(np.float64),
                np.concatenate([hi, hi, lo], axis=1).astype(np.float64))
    v = _to16(x * np.float32(scale), fmt == "fp16").astype(np.float64)
    return v, v


def _tile(ctx, x: np.ndarray, fmt: str):
    n, d = x.shape
    tx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    out = torch.zeros((128, 256), dtype=torch.float32, device="cuda")
    rows = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    scale = ctx.debug_screen_tile(tx.data_ptr(), n, d, out.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream,
                                  operands=FORMATS[fmt], rows_out=rows.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy(), rows.cpu().numpy(), scale


def _bf16_exact(rng, shape, lo_exp=0, hi_exp=3):
    """Random values with 8 significant bits (exact in bf16) and exponents in [lo, hi]."""
    mant = rng.integers(128, 256, size=shape) / 128.0
    ex = rng.integers(lo_exp, hi_exp + 1, size=shape)
    sign = rng.choice([-1.0, 1.0], size=shape)
    return (sign * mant * np.exp2(ex)).astype(np.float32)


def families(d: int):
    rng = np.random.default_rng(d)
    n = 256
    x = np.exp2(rng.integers(-30, 31, size=(n, d))) * rng.choice([-1.0, 1.0], size=(n, d))
    yield "mixed_exponents", x.astype(np.float32)
    h = d // 2
    a = _bf16_exact(rng, (128, h))
    b = a[:, rng.permutation(h)].copy()
    b[:, : h // 8] = _bf16_exact(rng, (128, h // 8))  # ||b|| close to, not equal to, ||a||
    top = np.concatenate([a, b, np.zeros((128, d - 2 * h), np.float32)], axis=1)
    bot = np.concatenate([a, -b, np.zeros((128, d - 2 * h), np.float32)], axis=1)
    yield "cancellation", np.concatenate([top, bot]).astype(np.float32)
    m = rng.integers(0, 128, size=(n, d))
    yield "equal_magnitudes", (rng.choice([-1.0, 1.0], size=(n, d)) *
                               (1 + m / 128.0)).astype(np.float32)
    g = _bf16_exact(rng, (n, d), -6, -3)
    g[:, rng.integers(0, d)] = np.float32(2.0 ** 20)
    yield "one_giant", g
    ramp = _bf16_exact(rng, (n, d), 0, 0) * np.exp2(np.arange(d) // 4)[None, :]
    yield "ramp", ramp.astype(np.float32)


CASES = ([(fmt, d, name) for fmt in ("bf16", "fp16") for d in (64, 100, 128)
          for name, _ in families(d)] + [("split", d, name) for d in (16, 64)
                                         for name, _ in families(d)])


@pytest.mark.parametrize("fmt,d,name", CASES)
def test_accumulation_within_a_quarter_of_the_model(gpu_ctx, fmt, d, name):
    x = dict(families(d))[name]
    if fmt == "fp16":
        # the fp16 screens scale x by 2^k with max |x| 2^k in [2^14, 2^15); keep every scaled
        # value in fp16's normal range so that the accumulation alone is measured
        amax = float(np.abs(x).max())
        nz = np.abs(x[x != 0])
        if nz.min() / amax < 2.0 ** -27:
            pytest.skip("dynamic range beyond fp16's normal range")
    got, _, scale = _tile(gpu_ctx, x, fmt)
    a, b = _operands(x, fmt, scale)
    exact = a[:128] @ b[:256].T
    absum = np.abs(a[:128]) @ np.abs(b[:256]).T
    k = (3 if fmt == "split" else 1) * (-(-d // 64) * 64)
    model = k * 2.0 ** -23 * absum
    err = np.abs(got.astype(np.float64) - exact)
    mask = model > 0
    ratio = float(np.max(err[mask] / model[mask])) if mask.any() else 0.0
    print(f"[accumulation] {fmt} d={d} {name}: observed / assumed = {ratio:.3e}")
    assert np.all(err[~mask] == 0)
    assert ratio <= RATIO_MAX, (fmt, d, name, ratio)


def _bound_data(d: int, offset: float, tiny: bool):
    rng = np.random.default_rng(int(d + offset))
    x = rng.normal(size=(256, d)) + offset * rng.uniform(-1, 1, size=(1, d))
    x[128:] = x[:128] + 0.01 * rng.normal(size=(128, d))  # near neighbours of the query rows
    if tiny:
        x *= 1e-18
    return x.astype(np.float32)


BOUND_CASES = ([(fmt, d) for fmt in ("bf16", "fp16") for d in (16, 64, 100, 128)] +
               [("split", d) for d in (16, 64)])


@pytest.mark.parametrize("offset,tiny", [(0.0, False), (10.0, False), (1000.0, False),
                                         (3.0, True)])
@pytest.mark.parametrize("fmt,d", BOUND_CASES)
def test_bound_never_exceeds_the_reference_distance(gpu_ctx, fmt, d, offset, tiny):
    if fmt == "fp16" and tiny:
        pytest.skip("no power-of-two scale keeps these values in the fp16 screens' range")
    x = _bound_data(d, offset, tiny)
    got, rows, scale = _tile(gpu_ctx, x, fmt)
    ps, pb, cm, m = (rows[:, i].astype(np.float64) for i in range(4))
    acc = got.astype(np.float64)
    # the epilogue's f32 steps, each rounded to f32 (the f64 sums of two f32 values are exact
    # except in rare far-apart cases, where the f32 rounding matches fmaf's closely enough to
    # sit inside the bound's margin)
    f = (pb[None, :256] - 2.0 * acc).astype(np.float32).astype(np.float64)
    t = (f + ps[:128, None]).astype(np.float32).astype(np.float64)
    lb = (t - cm[:128, None] * m[None, :256]).astype(np.float32).astype(np.float64)
    lb /= float(scale) ** 2
    qi, rj = np.meshgrid(np.arange(128), np.arange(256), indexing="ij")
    ref = O.pair_distances(x[qi.ravel()], x[rj.ravel()]).reshape(128, 256).astype(np.float64)
    worst = float(np.max(lb - ref))
    pos = ref > 0
    slack = float(np.median((ref - lb)[pos] / ref[pos])) if np.any(pos) else 0.0
    print(f"[bound] {fmt} d={d} offset={offset} tiny={tiny}: max(L - d2) = {worst:.3e}, "
          f"median relative slack {slack:.3e}")
    assert worst <= 0.0
