"""The exact-rounding helpers of aces4_gb300/csrc/exact_fp.h as the kernels run
them on the GPU (a4g_selftest_round, a4g_selftest_div), bit for bit against
IEEE arithmetic formed on the host:

* the one rounding of an exact 64-bit integer sum scaled by a power of two,
  which produces every split-precision result (on the GPU: the hardware
  integer-to-FP64 conversion and an exponent addition where the result is
  normal, the integer construction elsewhere); the reference is Python's
  correctly rounded conversion of the exact rational value;
* the division of the orbital-energy denominators and of the (T) energy
  (integer arithmetic for normal operands and results, the FP64 divide
  otherwise); the reference is numpy's IEEE division.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def _round_ref(v: int, e2: int, neg: bool) -> float:
    try:
        x = float(Fraction(v) * Fraction(2) ** e2)  # one correct rounding (ties to even)
    except OverflowError:
        x = math.inf if v > 0 else -math.inf
    if v == 0:
        x = 0.0
    return -x if neg else x


def test_device_rounding_matches_ieee(a4):
    import torch

    rng = np.random.default_rng(20261204)
    n = 60000
    bits = rng.integers(1, 64, n)
    v = [int(rng.integers(0, 1 << 62, dtype=np.int64)) >> (62 - int(b)) if b < 63 else
         int(rng.integers(1 << 61, 1 << 62, dtype=np.int64)) * 2 + int(rng.integers(0, 2)) for b in bits]
    for i in range(0, n, 7):  # exactly halfway: 53 bits, a one, then zeros
        m = int(rng.integers(1 << 52, 1 << 53, dtype=np.int64))
        s = int(rng.integers(0, 9))
        v[i] = ((m << 1) | 1) << s
    for i in range(3, n, 11):  # one above and one below halfway
        v[i] = v[i - 3] + (1 if i % 2 else -1)
    v = [x if rng.random() < 0.5 else -x for x in v]
    v[0], v[1] = 0, 0
    e2 = rng.integers(-1000, 900, n)
    e2[::13] = rng.integers(-1140, -1040, len(e2[::13]))  # subnormal and underflowing results
    e2[5::17] = rng.integers(960, 1000, len(e2[5::17]))   # near and beyond the largest double
    neg = rng.integers(0, 2, n)
    dv = torch.tensor(np.array(v, dtype=np.int64), device="cuda")
    de = torch.tensor(e2.astype(np.int32), device="cuda")
    dn = torch.tensor(neg.astype(np.int32), device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    rc = a4.lib().a4g_selftest_round(n, dv.data_ptr(), de.data_ptr(), dn.data_ptr(), out.data_ptr(), None)
    assert rc == 0
    a4.device.sync()
    got = out.cpu().numpy()
    want = np.array([_round_ref(v[i], int(e2[i]), bool(neg[i])) for i in range(n)])
    bad = np.nonzero(got.view(np.int64) != want.view(np.int64))[0]
    assert bad.size == 0, [(v[i], int(e2[i]), int(neg[i]), got[i].hex(), want[i].hex()) for i in bad[:5]]
    assert np.sum(np.abs(want) < 2.2250738585072014e-308) > 100  # the subnormal path was exercised
    assert np.sum(np.isinf(want)) > 10


def test_device_division_matches_ieee(a4):
    import torch

    rng = np.random.default_rng(7)
    n = 1 << 20
    ua = rng.integers(0, 1 << 63, n, dtype=np.int64).astype(np.uint64)
    ub = rng.integers(0, 1 << 63, n, dtype=np.int64).astype(np.uint64)
    ea = rng.integers(900, 1150, n).astype(np.uint64)
    eb = rng.integers(900, 1150, n).astype(np.uint64)
    frac = np.uint64((1 << 52) - 1)
    a = ((ua & frac) | (ea << np.uint64(52)) | (ua & np.uint64(1 << 63))).view(np.float64)
    b = ((ub & frac) | (eb << np.uint64(52)) | (ub & np.uint64(1 << 63))).view(np.float64)
    # denominator-like operands: amplitudes over sums of orbital energies
    k = n // 4
    e = rng.uniform(-2.0, -0.5, (k, 3)).sum(1) - rng.uniform(0.2, 5.0, (k, 3)).sum(1)
    a[:k], b[:k] = rng.standard_normal(k) * 1e-3, e
    # edge significands, zeros, subnormals, infinities, results beyond the range
    a[k:k + 64] = np.ldexp(1.0 + np.arange(64) * 2.0 ** -52, 0)
    b[k:k + 64] = np.ldexp(2.0 - np.arange(64) * 2.0 ** -52, 0)
    a[k + 64:k + 72] = [0.0, -0.0, 5e-324, 1e-310, np.inf, -np.inf, 1e300, 1e-300]
    b[k + 64:k + 72] = [3.0, 3.0, 7.0, 3.0, 2.0, np.inf, 1e-300, 1e300]
    da, db = torch.tensor(a, device="cuda"), torch.tensor(b, device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    assert a4.lib().a4g_selftest_div(n, da.data_ptr(), db.data_ptr(), out.data_ptr(), None) == 0
    a4.device.sync()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        want = a / b
    same = (got.view(np.int64) == want.view(np.int64)) | (np.isnan(got) & np.isnan(want))
    bad = np.nonzero(~same)[0]
    assert bad.size == 0, [(a[i].hex(), b[i].hex(), got[i].hex(), want[i].hex()) for i in bad[:5]]
