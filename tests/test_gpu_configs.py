"""Full-size parity runs of the ring (config 2) and batched sparse ladder
(config 3) pardo steps: the split-precision batch against the plain FP64
batch on every destination block, and both against the CPU oracle's BLAS path
on sampled blocks."""
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


def _ptrn(labels):
    d, l, r = labels
    ierr, p = oracle.get_contraction_ptrn(len(d), len(l), len(r), d + l + r)
    assert ierr == 0
    return p


def _block_errors(R, ref_buf):
    import torch

    errs = {}
    for k in R.keys():
        o, n = R.offsets[k], R.size(k)
        a, b = R.buf[o:o + n], ref_buf[o:o + n]
        errs[k] = float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
    return errs


def _oracle_block(R, key, trip, ptrn):
    want = np.zeros(R.size(key))
    dptr = R.block(key).data_ptr()
    for d, l, r, de, le, re in trip:
        if d.data_ptr() != dptr or l is None or r is None:
            continue
        want += oracle.contract_blas(ptrn, l.cpu().numpy(), le, r.cpu().numpy(), re, de)
    return want


def _run_both(a4, R, trip, ptrn):
    import torch

    fp = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=a4.device.PREC_FP64)
    fp.run()
    a4.device.sync()
    ref = R.buf.clone()
    sp = a4.device.Batch(ptrn, 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=5)
    sp.run_graph()
    a4.device.sync()
    torch.cuda.synchronize()
    return fp, sp, ref


def test_config2_ring_full_size(a4):
    """R(a,i,b,j) += V(a,k,c,i) T(c,b,k,j), o=40 (2x20), v=300 in seeded
    segments of 24..40, V ~ U[-1,1]/sqrt(o*v), T ~ N(0, 1e-2): 3.456e12 flop."""
    import torch

    from aces4_gb300.blocks import RING_LABELS, BlockArray, ring_triples, segments_uniform

    vs = segments_uniform(300, 24, 40, seed=2)
    os_ = [20, 20]
    V = BlockArray([vs, os_, vs, os_])
    T = BlockArray([vs, vs, os_, os_])
    R = BlockArray([vs, os_, vs, os_])
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    V.buf.uniform_(-1.0, 1.0, generator=g).div_(np.sqrt(40 * 300))
    T.buf.normal_(0.0, 0.1, generator=g)
    trip = ring_triples(R, V, T)
    ptrn = _ptrn(RING_LABELS)
    fp, sp, ref = _run_both(a4, R, trip, ptrn)
    assert abs(sp.info()["flops"] - 2 * 40 ** 3 * 300 ** 3) / (2 * 40 ** 3 * 300 ** 3) < 1e-12
    errs = _block_errors(R, ref)
    assert max(errs.values()) <= 1e-10, max(errs.values())
    for key in [R.keys()[0], R.keys()[-1]]:
        want = _oracle_block(R, key, trip, ptrn)
        o, n = R.offsets[key], R.size(key)
        got_fp = ref[o:o + n].cpu().numpy()
        assert np.linalg.norm(got_fp - want) <= 1e-12 * np.linalg.norm(want)
        got_sp = R.buf[o:o + n].cpu().numpy()
        assert np.linalg.norm(got_sp - want) <= 1e-10 * np.linalg.norm(want)


def test_config3_batched_sparse_ladder_step(a4):
    """One pardo step of the ladder at o=48 (2x24), v=400 in segments from
    {12,16,24,32,48}, 30% of the V blocks zero and skipped, four (a,b) segment
    pairs x all (c,d,i,j): several thousand uneven block pairs, one graph."""
    import torch

    from aces4_gb300.blocks import LADDER_LABELS, BlockArray, ladder_triples, segments_choice

    vs = segments_choice(400, [12, 16, 24, 32, 48], seed=3)
    os_ = [24, 24]
    rng = np.random.default_rng(3)
    zero = {}

    def present(k):
        zero.setdefault(k, rng.random() < 0.3)
        return not zero[k]

    V = BlockArray([vs[:2], vs[:2], vs, vs], present=present)
    T = BlockArray([vs, vs, os_, os_])
    R = BlockArray([vs[:2], vs[:2], os_, os_])
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    V.buf.uniform_(-1.0, 1.0, generator=g).div_(400.0)
    T.buf.normal_(0.0, 0.1, generator=g)
    trip = ladder_triples(R, V, T)
    live = sum(1 for t in trip if t[1] is not None)
    assert live > 2000 and live < len(trip)
    ptrn = _ptrn(LADDER_LABELS)
    fp, sp, ref = _run_both(a4, R, trip, ptrn)
    assert sp.info()["pairs"] == live
    errs = _block_errors(R, ref)
    assert max(errs.values()) <= 1e-10, max(errs.values())
    key = R.keys()[1]
    want = _oracle_block(R, key, trip, ptrn)
    o, n = R.offsets[key], R.size(key)
    assert np.linalg.norm(ref[o:o + n].cpu().numpy() - want) <= 1e-12 * np.linalg.norm(want)
    # replaying the captured graph reproduces the step bit for bit
    first = R.buf.clone()
    sp.run_graph()
    a4.device.sync()
    assert torch.equal(first, R.buf)
