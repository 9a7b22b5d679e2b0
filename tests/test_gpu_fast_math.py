"""Error bounds of the FAST-mode FP64 reciprocal, reciprocal square root and
square root (an FP32 hardware seed and one third-order Newton step on the
mantissa, the exponent handled on the integer bits), which replace CUDA's
correctly rounded divide and square root in the FAST kernels.

The device results (through weno_fast_math_eval) are compared with the same
functions evaluated in numpy's extended precision (at least 64 significant
bits): within 1 ulp for 1/x and 1/sqrt(x), 2 ulp for sqrt(x), and a relative
error below 2^-41 for the second-order reciprocal (the WENO weight
normalisations and the Euler-flux density pair), over mantissas and exponents
spread across the fast range [2^-1000, 2^1000] and the edges of the mantissa
interval.  Outside the fast range (zero, subnormals, huge values,
infinities, NaN) and for negative square-root arguments the functions take
CUDA's IEEE operations: 1/x and sqrt(x) then equal numpy's correctly rounded
results bit for bit.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RCP_ULP, RSQRT_ULP, SQRT_ULP = 1.0, 1.0, 2.0


def _eval(x):
    import torch
    from weno_ext import _lib
    L = _lib.load()
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    out = torch.empty(4 * x.size, dtype=torch.float64, device="cuda")
    _lib.check(L.weno_fast_math_eval(xd.data_ptr(), out.data_ptr(), x.size,
                                     torch.cuda.current_stream().cuda_stream), "fast_math_eval")
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    return o[:x.size], o[x.size:2 * x.size], o[2 * x.size:3 * x.size], o[3 * x.size:]


def _ulp_err(got, true_ld):
    ref = true_ld.astype(np.float64)
    ulp = np.spacing(np.abs(ref))
    return np.abs((got.astype(np.longdouble) - true_ld) / ulp.astype(np.longdouble)).astype(np.float64)


def _fast_range_sample(rng, n):
    mant = rng.uniform(1.0, 2.0, n)
    ex = rng.integers(-1000, 1000, n)  # 2^ex * [1, 2): biased exponent within [23, 2022]
    x = np.ldexp(mant, ex)
    one = np.float64(1.0)
    edges = []
    for e in (-1000, -999, -1, 0, 1, 2, 3, 511, 512, 999):
        b = np.ldexp(one, e)
        edges += [b, np.nextafter(b, np.inf), np.ldexp(2.0, e) * (1 - 2 ** -53), b * 1.5,
                  np.ldexp(np.float64(1.9999999), e), np.ldexp(np.float64(1 + 2 ** -23), e),
                  np.ldexp(np.float64(1 + 2 ** -23 - 2 ** -52), e)]
    # mantissas whose 23-bit truncation is furthest from the value
    edges += list(np.ldexp(np.float64(1.0) + (2.0 ** -23 - 2.0 ** -52) * np.arange(1, 9), 7))
    return np.concatenate([x, np.array(edges)])


def test_reciprocal_within_one_ulp():
    rng = np.random.default_rng(11)
    x = _fast_range_sample(rng, 60000)
    x = np.concatenate([x, -x[:20000]])
    r, _, _, _ = _eval(x)
    true = np.longdouble(1) / x.astype(np.longdouble)
    err = _ulp_err(r, true)
    assert err.max() <= RCP_ULP, (err.max(), x[err.argmax()])
    assert np.all(np.sign(r) == np.sign(x))
    # nearly always the correctly rounded quotient
    assert np.mean(r == 1.0 / x) > 0.98


def test_second_order_reciprocal_within_bound():
    rng = np.random.default_rng(13)
    x = _fast_range_sample(rng, 60000)
    x = np.concatenate([x, -x[:20000]])
    _, _, _, r2 = _eval(x)
    xl = x.astype(np.longdouble)
    rel = np.abs((r2.astype(np.longdouble) * xl - 1).astype(np.float64))
    assert rel.max() < 2.0 ** -41, (rel.max(), x[rel.argmax()])
    assert np.all(np.sign(r2) == np.sign(x))


def test_rsqrt_and_sqrt_within_bounds():
    rng = np.random.default_rng(12)
    x = _fast_range_sample(rng, 60000)
    _, rs, sq, _ = _eval(x)
    xl = x.astype(np.longdouble)
    true_sqrt = np.sqrt(xl)
    e_rs = _ulp_err(rs, np.longdouble(1) / true_sqrt)
    e_sq = _ulp_err(sq, true_sqrt)
    assert e_rs.max() <= RSQRT_ULP, (e_rs.max(), x[e_rs.argmax()])
    assert e_sq.max() <= SQRT_ULP, (e_sq.max(), x[e_sq.argmax()])


def test_outside_fast_range_takes_ieee():
    tiny = np.ldexp(1.0, -1001)
    huge = np.ldexp(1.0, 1001)
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1e-310, -1e-310, tiny, tiny * 1.7, huge, huge * 1.3,
                  1.7e308, -1.7e308, np.ldexp(1.0, -1022), np.ldexp(1.5, 1023)])
    r, rs, sq, r2 = _eval(x)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        want_r = 1.0 / x
        want_sq = np.sqrt(x)
    assert np.array_equal(r, want_r, equal_nan=True)
    assert np.array_equal(r2, want_r, equal_nan=True)
    assert np.array_equal(sq, want_sq, equal_nan=True)
    # CUDA's rsqrt: the limits exactly, finite values within 2 ulp
    assert np.isposinf(rs[0]) and np.isneginf(rs[1]) and rs[2] == 0.0 and np.isnan(rs[3]) and np.isnan(rs[4])
    assert np.all(np.isnan(rs[[7, 13]]))
    pos = np.array([5, 6, 8, 9, 10, 11, 12, 14, 15])
    true = np.longdouble(1) / np.sqrt(x[pos].astype(np.longdouble))
    assert _ulp_err(rs[pos], true).max() <= 2.0
    # negative arguments of the square roots: NaN
    _, rs_n, sq_n, _ = _eval(np.array([-1.0, -3.5e10, -1e-300]))
    assert np.all(np.isnan(rs_n)) and np.all(np.isnan(sq_n))
