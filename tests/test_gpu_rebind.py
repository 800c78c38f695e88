"""One batch serving a whole pardo loop: a4g_batch_rebind (the same planned
step pointed at the next iteration's blocks), a4g_batch_hold (an operand's
split digits reused across runs) and the tuning cache (a batch of a known
structure skips the autotuner), through the C ABI.

A rebound batch must give the same bits as a batch created fresh on the new
blocks (both precisions, eager runs and graph replays); a held operand must
give the same bits as slicing it every run; a batch tuned from the cache must
give the same bits as the autotuned one.  Against the CPU oracle the usual
tolerances hold (split 1e-10, FP64 1e-12 relative Frobenius per block).
"""
import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-10
TOL_FP64 = 1e-12
A4G_ERR_ARG = 1


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def _ladder(seed, vsegs, osegs, nslab_v=1, outliers=True):
    """V (every slab, or a one-slab buffer), T and R of a small ladder."""
    from aces4_gb300.blocks import BlockArray

    rng = np.random.default_rng(seed)
    v = sum(vsegs)
    V = BlockArray([vsegs] * 4)
    T = BlockArray([vsegs, vsegs, osegs, osegs])
    R = BlockArray([vsegs, vsegs, osegs, osegs])
    V.fill_from(lambda k, e: rng.uniform(-1, 1, int(np.prod(e))) / v)

    def tfill(k, e):
        x = rng.normal(0.0, 0.1, int(np.prod(e)))
        if outliers:
            x[rng.random(x.size) < 0.01] *= 1e3
        return x

    T.fill_from(tfill)
    return V, T, R


def _ptrn():
    from aces4_gb300.blocks import LADDER_LABELS

    d, l, r = LADDER_LABELS
    return oracle.get_contraction_ptrn(4, 4, 4, d + l + r)[1]


def _slab_blocks(R, a, b):
    return [R.block(k) for k in R.keys() if k[0] == a and k[1] == b]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("graph", [False, True])
def test_rebind_matches_fresh_batch(a4, prec, graph):
    """One batch rebound over every (a,b) slab == a fresh batch per slab, bit
    for bit; the operand T is held (sliced once) in the split form."""
    from aces4_gb300.blocks import ladder_slab_triples

    vs, os_ = [12, 16, 12], [5, 6]
    V, T, R = _ladder(1, vs, os_)
    R2 = type(R)([vs, vs, os_, os_])
    ptrn = _ptrn()
    st = torch.cuda.Stream()
    slabs = [(0, 0), (0, 2), (2, 0), (2, 2)]  # the slabs of one shape (12 x 12 rows; uneven c, d inside)
    b = a4.device.Batch(ptrn, 4, 4, 4, ladder_slab_triples(R, V, T, 0, 0), precision=prec, slices=5)
    b.hold(1, True, stream=st)
    for (sa, sb) in slabs:
        b.rebind(ladder_slab_triples(R, V, T, sa, sb), stream=st)
        (b.run_graph if graph else b.run)(st)
    st.synchronize()
    for (sa, sb) in slabs:
        f = a4.device.Batch(ptrn, 4, 4, 4, ladder_slab_triples(R2, V, T, sa, sb), precision=prec, slices=5)
        f.run(st)
        st.synchronize()
        f.close()
    b.close()
    assert torch.equal(R.buf, R2.buf)
    # and against the oracle on one block of the last slab
    key = (2, 2, 1, 1)
    want = np.zeros(R.size(key))
    for c in range(3):
        for d in range(3):
            want += oracle.contract_blas(ptrn, V.block((2, 2, c, d)).cpu().numpy(), V.ext((2, 2, c, d)),
                                         T.block((c, d, 1, 1)).cpu().numpy(), T.ext((c, d, 1, 1)), R.ext(key))
    got = R.block(key).cpu().numpy()
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err <= (TOL_SPLIT if prec else TOL_FP64), err


def test_rebind_slab_buffer_and_held_operand(a4):
    """The whole-contraction pattern: V slabs written one after another into
    one buffer, R slabs into a resident array, T held; equals fresh batches."""
    from aces4_gb300.blocks import BlockArray, ladder_slab_triples

    vs, os_ = [16] * 4, [8, 8]
    V, T, R = _ladder(2, vs, os_)
    Vbuf = [BlockArray([[16], [16], vs, vs]) for _ in range(2)]
    R2 = BlockArray([vs, vs, os_, os_])
    ptrn = _ptrn()
    st = torch.cuda.Stream()

    def load(buf, a, b):
        for c in range(4):
            for d in range(4):
                buf.block((0, 0, c, d)).copy_(V.block((a, b, c, d)))

    load(Vbuf[0], 0, 0)
    bt = a4.device.Batch(ptrn, 4, 4, 4, ladder_slab_triples(R, Vbuf[0], T, 0, 0, v_slab=True),
                         precision=1, slices=5)
    with torch.cuda.stream(st):
        bt.hold(1, True, stream=st)
        for s, (a, b) in enumerate([(a, b) for a in range(4) for b in range(4)]):
            buf = Vbuf[s % 2]
            load(buf, a, b)
            bt.rebind(ladder_slab_triples(R, buf, T, a, b, v_slab=True), stream=st)
            bt.run(st)
    st.synchronize()
    for a in range(4):
        for b in range(4):
            f = a4.device.Batch(ptrn, 4, 4, 4, ladder_slab_triples(R2, V, T, a, b), precision=1, slices=5)
            f.run(st)
            st.synchronize()
            f.close()
    bt.close()
    assert torch.equal(R.buf, R2.buf)


def test_hold_reslice_after_change(a4):
    """Held digits are reused until the operand is held again: changing T
    without re-holding keeps the old product; holding again picks it up."""
    from aces4_gb300.blocks import ladder_triples

    vs, os_ = [12] * 3, [5, 5]
    V, T, R = _ladder(3, vs, os_, outliers=False)
    ptrn = _ptrn()
    trip = ladder_triples(R, V, T)
    b = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=1, slices=5)
    b.hold(1, True)
    b.run()
    a4.device.sync()
    first = R.buf.clone()
    T.buf.mul_(2.0)
    b.run()
    a4.device.sync()
    assert torch.equal(R.buf, first)  # old digits of T
    b.hold(1, True)
    b.run()
    a4.device.sync()
    assert torch.equal(R.buf, 2.0 * first)  # powers of two scale exactly
    b.hold(1, False)
    T.buf.mul_(0.5)
    b.run()
    a4.device.sync()
    assert torch.equal(R.buf, first)
    b.close()


def test_tuning_cache(a4, tmp_path):
    """The second batch of a structure takes the first one's tuning, and the
    result does not change; save/load round-trips the cache."""
    from aces4_gb300.blocks import ladder_triples

    vs, os_ = [24, 32], [8, 8]
    V, T, R = _ladder(4, vs, os_)
    V2, T2, R2 = _ladder(4, vs, os_)
    ptrn = _ptrn()
    a4.device.tune_cache_clear()
    b1 = a4.device.Batch(ptrn, 4, 4, 4, ladder_triples(R, V, T), precision=1, slices=5)
    t1 = b1.tuning()
    assert not t1["from_cache"] and t1["autotune_ms"] > 0
    b2 = a4.device.Batch(ptrn, 4, 4, 4, ladder_triples(R2, V2, T2), precision=1, slices=5)
    t2 = b2.tuning()
    assert t2["from_cache"] and t2["autotune_ms"] == 0
    assert b1.form()["form"] == b2.form()["form"] and b1.splits()["nsplit"] == b2.splits()["nsplit"]
    b1.run()
    b2.run()
    a4.device.sync()
    assert torch.equal(R.buf, R2.buf)
    path = str(tmp_path / "tune.txt")
    a4.device.tune_cache_save(path)
    a4.device.tune_cache_clear()
    b3 = a4.device.Batch(ptrn, 4, 4, 4, ladder_triples(R2, V2, T2), precision=1, slices=4)
    assert not b3.tuning()["from_cache"]  # another slice count is another structure
    a4.device.tune_cache_load(path)
    b4 = a4.device.Batch(ptrn, 4, 4, 4, ladder_triples(R2, V2, T2), precision=1, slices=5)
    assert b4.tuning()["from_cache"] and b4.form()["form"] == b1.form()["form"]
    for b in (b1, b2, b3, b4):
        b.close()


def test_rebind_rejections(a4):
    from aces4_gb300.blocks import ladder_slab_triples

    vs, os_ = [12, 12], [5, 5]
    V, T, R = _ladder(5, vs, os_)
    ptrn = _ptrn()
    trip = ladder_slab_triples(R, V, T, 0, 0)
    b = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=1, slices=5)

    def rejected(tl):
        with pytest.raises(a4.device.A4GError) as e:
            b.rebind(tl)
        assert e.value.rc == A4G_ERR_ARG

    rejected(trip[:-1])  # another triple count
    d, l, r, de, le, re = trip[0]
    rejected([(d, l, r, de, le, [5, 12, 12, 5])] + trip[1:])  # other extents
    rejected([(d, None, r, de, le, re)] + trip[1:])  # a live pair turned into a zero block
    other = ladder_slab_triples(R, V, T, 1, 1)
    other[0] = (other[0][0], V.block((1, 1, 1, 1)), *other[0][2:])  # V(0,0,0,0) -> two new blocks
    rejected(other)
    b.hold(1, True)
    rejected([(t[0], t[1], t[2].clone(), *t[3:]) for t in trip])  # a held operand cannot move
    b.rebind(ladder_slab_triples(R, V, T, 1, 1))  # a legal rebind still works after the rejections
    b.run()
    a4.device.sync()
    b.close()
