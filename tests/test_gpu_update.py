"""Fused amplitude update (a4g_update_t2, procedure updatet2 of
rlccd_rhf.sialx:557-600) against the oracle's sequence of the reference's
block operations: DIIS error block and next amplitudes bit for bit, the
error's squared norm to 1e-13 (summation order)."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def _case(seed, iv, segs, rank1, diagonal):
    rng = np.random.default_rng(seed)
    o = segs[0]
    norb = sum(segs)
    e = np.concatenate([rng.uniform(-2.0, -0.5, o), rng.uniform(0.2, 5.0, norb - o)])
    f1 = np.diag(e).ravel(order="F").copy() if rank1 == 2 else e.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    ext = [segs[v - 1] for v in iv]
    n = int(np.prod(ext))
    xn, xo = rng.standard_normal(n) * 0.1, rng.standard_normal(n) * 0.1
    xnp = xn if diagonal else rng.standard_normal(n) * 0.1
    xop = xo if diagonal else rng.standard_normal(n) * 0.1
    return ext, ext1, f1, xn, xnp, xo, xop


@pytest.mark.parametrize("iv,segs,rank1,diagonal", [
    ([2, 1, 3, 1], [16, 32, 40], 2, False),      # a, b in different virtual segments
    ([2, 1, 2, 1], [16, 32, 40], 2, True),       # diagonal block: its own pair
    ([3, 1, 2, 1], [12, 33, 37], 1, False),      # odd extents, 1-D energies
    ([2, 1, 3, 1], [64, 96, 80], 2, False),      # several 32x32 tiles per (i, j)
])
def test_update_t2_matches_oracle(a4, iv, segs, rank1, diagonal):
    import torch

    ext, ext1, f1, xn, xnp, xo, xop = _case(7 + len(segs) + rank1 + diagonal, iv, segs, rank1, diagonal)
    want_err, want_next, want_nrm = oracle.update_t2(iv, ext, xn, xnp, xo, xop, ext1, f1, segs)
    d = lambda x: torch.tensor(x, device="cuda")
    txn, txo = d(xn), d(xo)
    txnp = txn if diagonal else d(xnp)
    txop = txo if diagonal else d(xop)
    err = torch.full_like(txn, float("nan"))
    nxt = torch.full_like(txn, float("nan"))
    nrm = torch.full((1,), 1.5, dtype=torch.float64, device="cuda")
    a4.device.update_t2(iv, ext, txn, txnp, txo, txop, err, nxt, ext1, d(f1), segs, nrm)
    a4.device.sync()
    np.testing.assert_array_equal(err.cpu().numpy(), want_err)
    np.testing.assert_array_equal(nxt.cpu().numpy(), want_next)
    assert abs(float(nrm.item()) - 1.5 - want_nrm) <= 1e-13 * want_nrm
    # the error block is optional
    nxt2 = torch.full_like(txn, float("nan"))
    a4.device.update_t2(iv, ext, txn, txnp, txo, txop, None, nxt2, ext1, d(f1), segs)
    a4.device.sync()
    assert torch.equal(nxt, nxt2)


def test_update_t2_rejects_in_place_output(a4):
    import torch

    ext, ext1, f1, xn, xnp, xo, xop = _case(3, [2, 1, 3, 1], [8, 8, 8], 2, False)
    t = torch.tensor(xo, device="cuda")
    other = torch.tensor(xn, device="cuda")
    with pytest.raises(a4.device.A4GError):
        a4.device.update_t2([2, 1, 3, 1], ext, other, other, t, t, None, t, ext1, torch.tensor(f1, device="cuda"),
                            [8, 8, 8])
