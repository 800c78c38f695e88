"""The allocation-free add/subtract entry point (a4g_add_sub_noalloc) against
the allocating one (a4g_add_sub), through the C ABI, on two calls in a row.

Callers that cannot allocate device memory while they run (a fixed device
budget owned by the host program, or work issued inside CUDA stream capture)
use a4g_add_sub_noalloc; it must give exactly the same bits as a4g_add_sub,
including the aliased, permuted case `d[i,j,k] += d[k,i,j]` that stages the
permuted operand in the library's fixed device array.  Element-wise results
are compared bit for bit, the tolerance the other element-wise tests use.

Collected last (file name) so a run that stops at the first failure has run
every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A4G_ERR_RANGE = 7


def _iarr(seq):
    return (ctypes.c_int * max(1, len(seq)))(*[int(x) for x in seq])


def _call(fn, subtract, d_labels, r_labels, r_ext, d, l, r, stream):
    return fn(ctypes.c_int(int(subtract)), ctypes.c_int(len(r_ext)), _iarr(d_labels), _iarr(r_labels),
              _iarr(r_ext), ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(l.data_ptr()),
              ctypes.c_void_p(r.data_ptr()), ctypes.c_void_p(stream))


@pytest.fixture(scope="module")
def so():
    import aces4_gb300

    aces4_gb300.build()
    return aces4_gb300.lib()


@pytest.mark.parametrize("subtract", [False, True])
def test_noalloc_matches_allocating_entry_twice(so, subtract):
    import torch

    torch.cuda.init()
    stream = torch.cuda.current_stream().cuda_stream or 1  # 1 = cudaStreamLegacy
    rng = np.random.default_rng(123)
    e = 64  # 64^3 = 262144 doubles, within the 2^20-double fixed array
    for call in range(2):  # two calls in a row share (and reuse) the array
        x = torch.tensor(rng.standard_normal(e ** 3), device="cuda")
        a, b = x.clone(), x.clone()
        # a[i,j,k] (+|-)= a[k,i,j]: r aliases d in another index order
        rc0 = _call(so.a4g_add_sub, subtract, [1, 2, 3], [3, 1, 2], [e, e, e], a, a, a, stream)
        rc1 = _call(so.a4g_add_sub_noalloc, subtract, [1, 2, 3], [3, 1, 2], [e, e, e], b, b, b, stream)
        torch.cuda.synchronize()
        assert rc0 == 0 and rc1 == 0, so.a4g_last_error()
        assert torch.equal(a, b), f"call {call}"
        # non-aliased operands: d = l - r with r in permuted order
        l = torch.tensor(rng.standard_normal(e ** 3), device="cuda")
        r = torch.tensor(rng.standard_normal(e ** 3), device="cuda")
        d0, d1 = torch.empty_like(l), torch.empty_like(l)
        rc0 = _call(so.a4g_add_sub, subtract, [1, 2, 3], [2, 3, 1], [e, e, e], d0, l, r, stream)
        rc1 = _call(so.a4g_add_sub_noalloc, subtract, [1, 2, 3], [2, 3, 1], [e, e, e], d1, l, r, stream)
        torch.cuda.synchronize()
        assert rc0 == 0 and rc1 == 0
        assert torch.equal(d0, d1), f"call {call}"
    # reference check of the aliased form on the host
    y = rng.standard_normal(e ** 3)
    t = torch.tensor(y, device="cuda")
    assert _call(so.a4g_add_sub_noalloc, subtract, [1, 2, 3], [3, 1, 2], [e, e, e], t, t, t, stream) == 0
    torch.cuda.synchronize()
    yb = y.reshape((e, e, e), order="F")
    ref = yb - np.transpose(yb, (1, 2, 0)) if subtract else yb + np.transpose(yb, (1, 2, 0))
    np.testing.assert_array_equal(t.cpu().numpy(), ref.ravel(order="F"))


def test_noalloc_rejects_oversized_aliased_operand(so):
    import torch

    e = 128  # 2^21 doubles > the 2^20-double array
    x = torch.zeros(e ** 3, dtype=torch.float64, device="cuda")
    rc = _call(so.a4g_add_sub_noalloc, 0, [1, 2, 3], [3, 1, 2], [e, e, e], x, x, x, 1)
    assert rc == A4G_ERR_RANGE
    assert b"exceeds the fixed scratch" in ctypes.c_char_p(so.a4g_last_error()).value
