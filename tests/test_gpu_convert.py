"""Block conversions through the C ABI (`chefsi_convert_block`, DFT-FE's
copyValueType1ArrToValueType2Arr) against numpy, bit for bit.

A power-of-two scale is applied on the bit patterns and must equal the exactly scaled value
rounded once to the destination type (numpy: scale in float64, then cast). The inputs span
zeros of both signs, FP32 subnormals, values whose scaled FP32 image is subnormal or
overflows, and ordinary values over many decades; contiguous blocks (flat vectorised pass) and
strided blocks with odd widths (row pass) both run.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def values(rng, shape, lo_exp, hi_exp):
    mant = rng.uniform(1.0, 2.0, shape) * rng.choice([-1.0, 1.0], shape)
    x = mant * np.exp2(rng.integers(lo_exp, hi_exp, shape).astype(np.float64))
    flat = x.reshape(-1)
    flat[::17] = 0.0
    flat[5::23] = -0.0
    return x


def run(C, src_np, dst_dtype, scale, ld_pad):
    rows, n = src_np.shape
    src_t = torch.zeros((rows, n + ld_pad), dtype=torch.from_numpy(src_np).dtype, device="cuda")
    src_t[:, :n] = torch.from_numpy(src_np).cuda()
    dst_t = torch.full((rows, n + ld_pad), 7.0, dtype=dst_dtype, device="cuda")
    C.copyValueType1ArrToValueType2Arr(src_t[:, :n], dst_t[:, :n], scale)
    out = dst_t.cpu().numpy()
    # the padding columns are untouched
    assert np.all(out[:, n:] == 7.0)
    return out[:, :n]


def same_bits(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.dtype == b.dtype
    ia = a.view(np.uint64 if a.dtype == np.float64 else np.uint32)
    ib = b.view(np.uint64 if b.dtype == np.float64 else np.uint32)
    bad = np.flatnonzero(ia != ib)
    assert bad.size == 0, (bad[:5], a.reshape(-1)[bad[:5]], b.reshape(-1)[bad[:5]])


SHAPES = [(1000, 64, 0), (333, 7, 5), (64, 300, 12), (1, 4096, 0)]


@pytest.mark.parametrize("rows,n,pad", SHAPES)
@pytest.mark.parametrize("k", [0, 8, -20, 100, -140])
def test_f64_to_f32_pow2(C, rows, n, pad, k):
    rng = np.random.default_rng(abs(rows + n + k))
    x = values(rng, (rows, n), -160, 140)
    got = run(C, x, torch.float32, 2.0 ** k, pad)
    with np.errstate(over="ignore"):
        ref = (x * 2.0 ** k).astype(np.float32)
    same_bits(got, ref)


@pytest.mark.parametrize("rows,n,pad", SHAPES)
@pytest.mark.parametrize("k", [0, -8, 30, -300])
def test_f32_to_f64_pow2(C, rows, n, pad, k):
    rng = np.random.default_rng(abs(2 * rows + n + k))
    x = values(rng, (rows, n), -149, 127).astype(np.float32)
    got = run(C, x, torch.float64, 2.0 ** k, pad)
    same_bits(got, x.astype(np.float64) * 2.0 ** k)


@pytest.mark.parametrize("rows,n,pad", SHAPES)
@pytest.mark.parametrize("k", [0, 5, -30, 60])
def test_f32_to_f32_pow2(C, rows, n, pad, k):
    rng = np.random.default_rng(abs(3 * rows + n + k))
    x = values(rng, (rows, n), -149, 127).astype(np.float32)
    got = run(C, x, torch.float32, 2.0 ** k, pad)
    with np.errstate(over="ignore"):
        ref = (x.astype(np.float64) * 2.0 ** k).astype(np.float32)
    same_bits(got, ref)


@pytest.mark.parametrize("rows,n,pad", SHAPES)
@pytest.mark.parametrize("k", [0, -3, 700, -1060])
def test_f64_to_f64_pow2(C, rows, n, pad, k):
    rng = np.random.default_rng(abs(4 * rows + n + k))
    x = values(rng, (rows, n), -300, 300)
    got = run(C, x, torch.float64, 2.0 ** k if k > -1023 else np.ldexp(1.0, k), pad)
    with np.errstate(over="ignore", under="ignore"):
        ref = np.ldexp(x, k)
    same_bits(got, ref)


@pytest.mark.parametrize("rows,n,pad", SHAPES[:2])
def test_general_scale_multiplies_in_destination_precision(C, rows, n, pad):
    rng = np.random.default_rng(rows)
    s = 0.3711
    x64 = values(rng, (rows, n), -20, 20)
    x32 = x64.astype(np.float32)
    same_bits(run(C, x64, torch.float32, s, pad), (s * x64).astype(np.float32))
    same_bits(run(C, x32, torch.float32, s, pad), np.float32(s) * x32)
    same_bits(run(C, x32, torch.float64, s, pad), s * x32.astype(np.float64))
    same_bits(run(C, x64, torch.float64, s, pad), s * x64)
