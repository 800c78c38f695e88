"""Accuracy of the split-precision contraction, measured and certified.

Measured: the relative Frobenius error of every destination block against the
plain FP64 GPU form (and one block against the CPU oracle's BLAS path) on the
full o=64/v=512 ladder slab (V ~ U[-1,1]/512, T ~ N(0,1e-2) with 1 % of its
entries x 1e3) at 4, 5 and 6 slices: 4 slices 1e-7, 5 slices 1e-10 (the
stated bound of the default), 6 slices 1e-12.

Certified: a4g_batch_error_bound's worst-case bound must lie above the
measured error for every slice count (3..7), fall as slices are added, and
flag (A4G_ERR_PRECISION) data whose rows span a wide range, on which 5 slices
really do miss 1e-10.
"""
import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu

A4G_ERR_PRECISION = 8


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def _ptrn():
    from aces4_gb300.blocks import LADDER_LABELS

    d, l, r = LADDER_LABELS
    return oracle.get_contraction_ptrn(4, 4, 4, d + l + r)[1]


def _errors(R, ref):
    out = []
    for k in R.keys():
        o, n = R.offsets[k], R.size(k)
        out.append(float(torch.linalg.norm(R.buf[o:o + n] - ref[o:o + n]) / torch.linalg.norm(ref[o:o + n])))
    return out


def _ladder(vs, os_, seed, wide=False):
    from aces4_gb300.blocks import BlockArray, ladder_triples

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    v = sum(vs)
    V = BlockArray([vs] * 4)
    T = BlockArray([vs, vs, os_, os_])
    R = BlockArray([vs, vs, os_, os_])
    V.buf.uniform_(-1.0 / v, 1.0 / v, generator=g)
    T.buf.normal_(0.0, 0.1, generator=g)
    T.buf[torch.rand(T.buf.shape, device="cuda", generator=g) < 0.01] *= 1e3
    if wide:
        # every V row gets one element 1e6 x larger, in the k column where the
        # matching T row is zero: the product is unchanged, but the row's
        # scale (and so the digits' grid) follows the large element
        for (a, b, c, d) in V.keys():
            if (c, d) != (0, 0):
                continue
            blk = V.block((a, b, c, d)).view(vs[d], vs[c], vs[b], vs[a])  # [d][c][b][a]: rows (a,b) fastest
            blk[0, 0] *= 1e6
            for i in range(len(os_)):
                for j in range(len(os_)):
                    T.block((c, d, i, j)).view(os_[j], os_[i], vs[d], vs[c])[:, :, 0, 0] = 0.0
    return V, T, R, ladder_triples(R, V, T)


def test_bound_holds_and_falls_with_slices(a4):
    V, T, R, trip = _ladder([32] * 2, [16, 16], 5)
    ptrn = _ptrn()
    f = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=0)
    f.run()
    a4.device.sync()
    ref = R.buf.clone()
    f.close()
    prev = None
    for S in range(3, 8):
        b = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=1, slices=S)
        b.run()
        bound = b.error_bound()
        err = max(_errors(R, ref))
        b.close()
        assert err <= bound, (S, err, bound)
        assert prev is None or bound < prev / 100, (S, bound, prev)
        prev = bound


def test_bound_flags_wide_range_rows(a4):
    V, T, R, trip = _ladder([32] * 2, [16, 16], 6, wide=True)
    ptrn = _ptrn()
    f = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=0)
    f.run()
    a4.device.sync()
    ref = R.buf.clone()
    f.close()
    b = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=1, slices=5)
    b.run()
    with pytest.raises(a4.device.A4GError) as e:
        b.error_bound(target=1e-10)
    assert e.value.rc == A4G_ERR_PRECISION and e.value.bound > 1e-10
    err = max(_errors(R, ref))
    b.close()
    assert 1e-10 < err <= e.value.bound  # the flagged miss is real


def test_full_slab_slices_4_5_6(a4):
    """The full o=64/v=512 ladder slab (4096 block pairs of 1024x256x1024)."""
    from aces4_gb300.blocks import BlockArray, ladder_slab_array

    vs, os_ = [32] * 16, [16] * 4
    g = torch.Generator(device="cuda")
    g.manual_seed(99)
    T = BlockArray([vs, vs, os_, os_])
    R = BlockArray([[32], [32], os_, os_])
    V = BlockArray([[32], [32], vs, vs])
    V.buf.uniform_(-1.0 / 512, 1.0 / 512, generator=g)
    step = 1 << 27
    for s0 in range(0, T.buf.numel(), step):
        t = T.buf[s0:s0 + step]
        t.normal_(0.0, 0.1, generator=g)
        t[torch.rand(t.shape, device="cuda", generator=g) < 0.01] *= 1e3
    ptrn = _ptrn()
    arr = ladder_slab_array(R, V, T, 0, 0)
    f = a4.device.Batch(ptrn, 4, 4, 4, arr, precision=0)
    f.run()
    a4.device.sync()
    ref = R.buf.clone()
    f.close()
    # the FP64 GPU form against the CPU oracle on one block (all 256 pairs)
    acc = np.zeros(R.size((0, 0, 0, 0)))
    for c in range(16):
        for d in range(16):
            acc += oracle.contract_blas(ptrn, V.block((0, 0, c, d)).cpu().numpy(), [32] * 4,
                                        T.block((c, d, 0, 0)).cpu().numpy(), [32, 32, 16, 16], [32, 32, 16, 16])
    o, n = R.offsets[(0, 0, 0, 0)], R.size((0, 0, 0, 0))
    assert np.linalg.norm(ref[o:o + n].cpu().numpy() - acc) <= 1e-12 * np.linalg.norm(acc)
    tol = {4: 1e-7, 5: 1e-10, 6: 1e-12}
    for S in (4, 5, 6):
        b = a4.device.Batch(ptrn, 4, 4, 4, arr, precision=1, slices=S)
        b.run()
        bound = b.error_bound()
        errs = _errors(R, ref)
        got = R.buf[o:o + n].cpu().numpy()
        b.close()
        assert max(errs) <= tol[S], (S, max(errs))
        assert max(errs) <= bound
        assert np.linalg.norm(got - acc) <= tol[S] * np.linalg.norm(acc)
