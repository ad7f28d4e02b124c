"""Adversarial check of the tensor-core accumulation model behind the screens' error bound.

The screens' lower bound of a squared distance assumes (refined.cu, error_coefficients) that the
tcgen05 f32 accumulation of K = d_pad 16-bit products is off from the exact sum of those
products by at most

    K * 2^-21 * sum_f |a_f b_f|                                  (the assumed model)

and that the whole dot product of the f32 inputs is off by at most
a1 * ||x|| * ||y||, a1 = (2u + u^2) + K 2^-21 (1 + u)^2 (u the operand unit roundoff).
These tests drive the accumulator with operands built to stress it and require the observed
worst case to stay within a quarter of the assumed model:

* mixed exponents across K (powers of two from 2^-30 to 2^30, random signs);
* heavy cancellation (rows [a, b] against [a, -b] with ||a|| close to ||b||);
* all-equal magnitudes (+-(1 + m 2^-7): 16-bit products, integer-like sums);
* one giant coordinate per row among small ones;
* magnitudes ramping up along K, so the largest products arrive last;
* fp16 operands scaled into [2^14, 2^15) by the fp16 screens' own power-of-two scale.

K = 64 and 128 (d = 64, 100 and 128). Operands are exact in the 16-bit format where the test
isolates the accumulation, and general f32 data checks the whole dot-product bound.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RATIO_MAX = 0.25
WORST: dict = {}


def _round(x: np.ndarray, fp16: bool, scale: float = 1.0) -> np.ndarray:
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32) * np.float32(scale))
    return t.to(torch.float16 if fp16 else torch.bfloat16).to(torch.float64).numpy()


def _tile(ctx, x: np.ndarray, operands: int):
    tx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    out = torch.zeros((128, 256), dtype=torch.float32, device="cuda")
    scale = ctx.debug_screen_tile(tx.data_ptr(), x.shape[0], x.shape[1], out.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream, operands=operands)
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64), scale


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


CASES = [(d, name) for d in (64, 100, 128) for name, _ in families(d)]


@pytest.mark.parametrize("d,name", CASES)
@pytest.mark.parametrize("operands", [0, 1], ids=["bf16", "fp16"])
def test_accumulation_within_a_quarter_of_the_model(gpu_ctx, d, name, operands):
    x = dict(families(d))[name]
    fp16 = operands == 1
    if fp16:
        # the fp16 screens scale x by 2^k with max |x| 2^k in [2^14, 2^15); keep every scaled
        # value in fp16's normal range so that the accumulation alone is measured
        amax = float(np.abs(x).max())
        nz = np.abs(x[x != 0])
        if nz.min() / amax < 2.0 ** -27:
            pytest.skip("dynamic range beyond fp16's normal range")
    got, scale = _tile(gpu_ctx, x, operands)
    xr = _round(x, fp16, scale)
    exact = xr[:128] @ xr[:256].T
    absum = np.abs(xr[:128]) @ np.abs(xr[:256]).T
    k = -(-d // 64) * 64
    model = k * 2.0 ** -21 * absum
    err = np.abs(got - exact)
    mask = model > 0
    ratio = float(np.max(err[mask] / model[mask])) if mask.any() else 0.0
    key = ("fp16" if fp16 else "bf16", d, name)
    WORST[key] = ratio
    print(f"[accumulation] {key}: observed / assumed = {ratio:.3e}")
    assert np.all(err[~mask] == 0)
    assert ratio <= RATIO_MAX, (key, ratio)


@pytest.mark.parametrize("d", [64, 100, 128])
@pytest.mark.parametrize("offset", [0.0, 10.0, 1000.0])
def test_whole_dot_product_bound_on_f32_data(gpu_ctx, d, offset):
    """General f32 data (bf16 rounding of both factors plus the accumulation): the observed
    error stays within half of a1 ||x|| ||y||."""
    rng = np.random.default_rng(int(d + offset))
    x = (rng.normal(size=(256, d)) + offset * rng.uniform(-1, 1, size=(1, d))).astype(np.float32)
    got, _ = _tile(gpu_ctx, x, 0)
    xf = x.astype(np.float64)
    exact = xf[:128] @ xf[:256].T
    u = 2.0 ** -8
    k = -(-d // 64) * 64
    a1 = (2 * u + u * u) + k * 2.0 ** -21 * (1 + u) ** 2
    nrm = np.linalg.norm(xf, axis=1)
    bound = a1 * np.outer(nrm[:128], nrm[:256])
    ratio = float(np.max(np.abs(got - exact) / bound))
    print(f"[dot bound] d={d} offset={offset}: observed / bound = {ratio:.3e}")
    assert ratio <= 0.5
