"""Failure detection without a GPU fault: a device-side wait that nothing
completes gives up after its limit, reports through the device error flag,
and leaves the CUDA context usable (the bounded-wait path of every pipeline
wait in the library)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

A4G_ERR_TIMEOUT = 5


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def test_bounded_wait_reports_timeout_and_context_survives(a4):
    import torch

    L = a4.lib()
    waited = ctypes.c_int(-1)
    rc = L.a4g_selftest_wait_timeout(ctypes.c_int(200), ctypes.byref(waited), ctypes.c_void_p(1))
    assert rc == A4G_ERR_TIMEOUT, rc
    assert 200 <= waited.value < 5000, waited.value
    assert b"iteration limit" in ctypes.c_char_p(L.a4g_last_error()).value
    # the flag was consumed: the next checked call is clean, and work still runs
    L.a4g_clear_error()
    rng = np.random.default_rng(3)
    le, re, de = [6, 7, 8], [8, 5], [6, 7, 5]
    x, y = rng.standard_normal(int(np.prod(le))), rng.standard_normal(int(np.prod(re)))
    d = torch.empty(int(np.prod(de)), dtype=torch.float64, device="cuda")
    a4.device.contract_labels([1, 2, 4], [1, 2, 3], [3, 4], torch.tensor(x, device="cuda"), le,
                              torch.tensor(y, device="cuda"), re, d, de)
    a4.device.sync()
    ierr, want = oracle.contract_labels([1, 2, 4], [1, 2, 3], [3, 4], x, le, y, re, de)
    assert ierr == 0
    np.testing.assert_allclose(d.cpu().numpy(), want, rtol=1e-13, atol=1e-13)
