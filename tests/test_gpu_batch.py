"""Batched (one pardo step) contraction through the C ABI: the grouped FP64
kernel and the split-precision tcgen05 pipeline, against the CPU oracle's BLAS
path per destination block.

Tolerances (relative Frobenius error per destination block):
  plain FP64 grouped kernel   1e-12
  split precision, 5 slices   1e-10   (the stated bound of the split form)
  split precision, 1 slice on integer data in [-127, 127]: bit-exact
"""
import itertools

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_SPLIT = 1e-10


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


def _make(a4, kind, vsegs, osegs, zero_frac, seed, outliers=False, integer=False):
    from aces4_gb300.blocks import BlockArray, ladder_triples, ring_triples, LADDER_LABELS, RING_LABELS

    rng = np.random.default_rng(seed)
    v = sum(vsegs)
    o = sum(osegs)
    zero = {}

    def vpresent(k):
        zero.setdefault(k, rng.random() < zero_frac)
        return not zero[k]

    def vfill(k, e):
        n = int(np.prod(e))
        if integer:
            return rng.integers(-127, 128, n).astype(np.float64)
        return rng.uniform(-1, 1, n) / (v if kind == "ladder" else np.sqrt(o * v))

    def tfill(k, e):
        n = int(np.prod(e))
        if integer:
            return rng.integers(-127, 128, n).astype(np.float64)
        x = rng.normal(0.0, 0.1, n)
        if outliers:
            x[rng.random(n) < 0.01] *= 1e3
        return x

    if kind == "ladder":
        V = BlockArray([vsegs] * 4, present=vpresent)
        T = BlockArray([vsegs, vsegs, osegs, osegs])
        R = BlockArray([vsegs, vsegs, osegs, osegs])
        V.fill_from(vfill)
        T.fill_from(tfill)
        trip = ladder_triples(R, V, T)
        labels = LADDER_LABELS
    else:
        V = BlockArray([vsegs, osegs, vsegs, osegs], present=vpresent)
        T = BlockArray([vsegs, vsegs, osegs, osegs])
        R = BlockArray([vsegs, osegs, vsegs, osegs])
        V.fill_from(vfill)
        T.fill_from(tfill)
        trip = ring_triples(R, V, T)
        labels = RING_LABELS
    return R, V, T, trip, labels


def _reference(R, trip, labels):
    """Per destination block: sum over live pairs of the BLAS-path oracle."""
    p = _ptrn(labels)
    ref = {}
    ptr_to_key = {R.block(k).data_ptr(): k for k in R.keys()}
    for d, l, r, de, le, re in trip:
        key = ptr_to_key[d.data_ptr()]
        acc = ref.setdefault(key, np.zeros(int(np.prod(de))))
        if l is None or r is None:
            continue
        acc += oracle.contract_blas(p, l.cpu().numpy(), le, r.cpu().numpy(), re, de)
    return ref


def _errors(R, ref):
    errs = []
    for k, want in ref.items():
        got = R.block(k).cpu().numpy()
        nb = np.linalg.norm(want)
        errs.append(np.linalg.norm(got - want) / (nb if nb > 0 else 1.0))
    return np.array(errs)


def _run(a4, R, trip, labels, precision, slices=5, beta=0, graph=False, variant=0):
    import torch

    b = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=precision, slices=slices, beta=beta,
                        variant=variant)
    if graph:
        b.run_graph()
    else:
        b.run()
    a4.device.sync()
    torch.cuda.synchronize()
    return b


def test_fp64_ladder_config1_shape(a4):
    # o=10 as 2 segments of 5, v=48 as 4 segments of 12, all blocks dense
    R, V, T, trip, labels = _make(a4, "ladder", [12] * 4, [5, 5], 0.0, 1)
    R.buf.fill_(np.nan)
    b = _run(a4, R, trip, labels, a4.device.PREC_FP64)
    info = b.info()
    assert info["pairs"] == 4 ** 4 * 2 ** 2
    assert abs(info["flops"] - 2 * 48 ** 4 * 10 ** 2) < 1
    assert _errors(R, _reference(R, trip, labels)).max() <= TOL_FP64


def test_fp64_uneven_sparse_ring(a4):
    R, V, T, trip, labels = _make(a4, "ring", [12, 16, 24], [5, 8], 0.3, 2)
    R.buf.fill_(np.nan)
    _run(a4, R, trip, labels, a4.device.PREC_FP64)
    errs = _errors(R, _reference(R, trip, labels))
    assert errs.max() <= TOL_FP64


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6])
def test_split_one_slice_integer_exact(a4, variant):
    # integers in [-127, 127] are exact single 8-bit digits: the tensor-core
    # products and the chunked FP32 accumulation must reproduce FP64 exactly,
    # in both GEMM forms (one SM per 128x128 tile, CTA pair per 256x128 tile)
    R, V, T, trip, labels = _make(a4, "ladder", [32, 32], [16, 16], 0.0, 3, integer=True)
    b = _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=1, variant=variant)
    assert b.form()["form"] == variant
    ref = _reference(R, trip, labels)
    for k, want in ref.items():
        np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6])
def test_split_long_k_integer_exact(a4, variant):
    # K per destination row = 16 * 48^2 = 36864 (several exact flush chunks,
    # several levels' chunk sizes) with 2 slices on integer data
    R, V, T, trip, labels = _make(a4, "ladder", [48] * 4, [8], 0.0, 4, integer=True)
    _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=2, variant=variant)
    ref = _reference(R, trip, labels)
    for k, want in ref.items():
        np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)


def test_split_count_autotune_keeps_results_exact(a4):
    # the autotuner scores the balance-driven split-K count against its
    # double; whichever it keeps, integer data must come back exact
    R, V, T, trip, labels = _make(a4, "ladder", [48] * 4, [8], 0.0, 4, integer=True)
    b = _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=2)
    sp = b.splits()
    if b.form()["form"] <= 4:
        assert sp["nsplit"] in sp["tuned_ms"], sp
        assert all(v > 0 for v in sp["tuned_ms"].values()), sp
    else:  # a direct form won: one split, nothing to tune
        assert sp == {"nsplit": 1, "tuned_ms": {}}, sp
    ref = _reference(R, trip, labels)
    for k, want in ref.items():
        np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)
    f64 = _run(a4, R, trip, labels, a4.device.PREC_FP64)
    assert f64.splits()["nsplit"] == 0


@pytest.mark.parametrize("slices,tol", [(3, 1e-5), (4, 1e-7), (5, TOL_SPLIT), (6, 1e-12), (7, 1e-13)])
def test_split_ladder_outliers(a4, slices, tol):
    # config-4 distributions (V ~ U[-1,1]/v, T ~ N(0,1e-2) with 1% x1e3) on a
    # smaller ladder: v=64 in 2 segments of 32, o=32 in 2 segments of 16
    R, V, T, trip, labels = _make(a4, "ladder", [32, 32], [16, 16], 0.0, 5, outliers=True)
    _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=slices, variant=1 + slices % 4)
    errs = _errors(R, _reference(R, trip, labels))
    assert errs.max() <= tol, (slices, errs.max())


def _bits(t):
    import torch

    return t.clone().view(torch.int64)


@pytest.mark.parametrize("variant", [5, 6])
def test_direct_forms_bit_identical_to_workspace_forms(a4, variant):
    """The direct forms fold a tile's levels exactly in TMEM and store FP64
    from the GEMM's epilogue; they must give the bits of the workspace +
    recombine form with the same tile shape: the ladder with outliers at 5
    slices, then the accumulate and negate modes on an uneven sparse ring."""
    import torch

    R, V, T, trip, labels = _make(a4, "ladder", [32, 32], [16, 16], 0.0, 5, outliers=True)
    ws_form = _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=5, variant=variant - 4)
    want = _bits(R.buf)
    R.buf.fill_(float("nan"))
    direct = _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=5, variant=variant)
    assert direct.form()["form"] == variant
    assert direct.launches()["kernels_per_run"] == ws_form.launches()["kernels_per_run"] - 1
    assert direct.splits()["nsplit"] == 1
    assert torch.equal(_bits(R.buf), want)
    assert _errors(R, _reference(R, trip, labels)).max() <= TOL_SPLIT

    R, V, T, trip, labels = _make(a4, "ring", [12, 16, 24, 32], [5, 8], 0.3, 6)
    base = torch.randn(R.buf.numel(), dtype=torch.float64, device=R.buf.device)
    outs = []
    for v in (variant - 4, variant):
        R.buf.copy_(base)
        b = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=5,
                            beta=1, negate=True, variant=v)
        b.run_graph()
        a4.device.sync()
        torch.cuda.synchronize()
        outs.append(_bits(R.buf))
    assert torch.equal(outs[0], outs[1])
    ref = _reference(R, trip, labels)
    for k, w in ref.items():
        got = R.block(k).cpu().numpy()
        want2 = base[R.offsets[k]:R.offsets[k] + w.size].cpu().numpy() - w
        assert np.linalg.norm(got - want2) <= TOL_SPLIT * np.linalg.norm(want2)


@pytest.mark.parametrize("variant", [0, 1, 4, 5, 6])
def test_destination_unit_stride_on_the_right_operand(a4, variant):
    """D(a,b) = sum_k L(b,k) R(k,a): D's unit-stride index comes from the
    right operand, so the split form multiplies with the operands' roles
    exchanged.  Integer data with 2 slices is exact; several tiles, ragged
    edges, three pairs per destination block."""
    import torch

    rng = np.random.default_rng(77)
    dl, ll, rl = [1, 2], [2, 3], [3, 1]
    de, le, re = [300, 261], [261, 45], [45, 300]
    ierr, p = oracle.get_contraction_ptrn(2, 2, 2, dl + ll + rl)
    assert ierr == 0
    Ls = [rng.integers(-127, 128, int(np.prod(le))).astype(np.float64) for _ in range(3)]
    Rs = [rng.integers(-127, 128, int(np.prod(re))).astype(np.float64) for _ in range(3)]
    D = torch.full((int(np.prod(de)),), float("nan"), dtype=torch.float64, device="cuda")
    tl = [torch.tensor(x, device="cuda") for x in Ls]
    tr = [torch.tensor(x, device="cuda") for x in Rs]
    trip = [(D, tl[q], tr[q], de, le, re) for q in range(3)]
    b = a4.device.Batch(p, 2, 2, 2, trip, precision=a4.device.PREC_OZAKI_BF16, slices=2, variant=variant)
    b.run()
    a4.device.sync()
    torch.cuda.synchronize()
    if variant:
        assert b.form()["form"] == variant
    want = sum(oracle.contract_blas(p, Ls[q], le, Rs[q], re, de) for q in range(3))
    np.testing.assert_array_equal(D.cpu().numpy(), want)


@pytest.mark.parametrize("variant", [1, 4, 5])
def test_non_finite_operands_poison_their_rows_and_columns(a4, variant):
    """A NaN in a left block and an infinity in a right block: digits cannot
    carry them, so the split form stores NaN wherever FP64 gives a non-finite
    result (the whole row / column they feed) and the FP64 values elsewhere."""
    import torch

    R, V, T, trip, labels = _make(a4, "ladder", [32, 32], [16, 16], 0.0, 31)
    V.buf[V.offsets[(0, 1, 1, 0)] + 5] = float("nan")
    T.buf[T.offsets[(1, 1, 0, 1)] + 77] = float("inf")
    _run(a4, R, trip, labels, a4.device.PREC_FP64)
    want = R.buf.clone()
    R.buf.fill_(0.0)
    _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, variant=variant)
    got = R.buf.clone()
    bad = ~torch.isfinite(want)
    assert int(bad.sum()) > 0
    assert torch.equal(torch.isnan(got), bad)
    ok = ~bad
    assert float((got[ok] - want[ok]).abs().max()) <= TOL_SPLIT * float(want[ok].abs().max())


def test_split_uneven_sparse_ring_graph_and_beta(a4):
    import torch

    R, V, T, trip, labels = _make(a4, "ring", [12, 16, 24, 32], [5, 8], 0.3, 6)
    ref = _reference(R, trip, labels)
    _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=5, graph=True, variant=2)
    assert _errors(R, ref).max() <= TOL_SPLIT
    first = R.buf.clone()
    # replaying the captured graph gives identical bits
    b = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=5)
    b.run_graph()
    b.run_graph()
    a4.device.sync()
    assert torch.equal(first, R.buf)
    # beta = 1 accumulates on top of the existing blocks
    base = R.buf.clone()
    bb = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=5, beta=1)
    bb.run()
    a4.device.sync()
    for k, want in ref.items():
        got = R.block(k).cpu().numpy()
        want2 = want + base[R.offsets[k]:R.offsets[k] + want.size].cpu().numpy()
        assert np.linalg.norm(got - want2) <= TOL_SPLIT * np.linalg.norm(want2)


def test_zero_destination_blocks_are_cleared(a4):
    # every V block zero -> R blocks receive no pair and are overwritten with 0
    R, V, T, trip, labels = _make(a4, "ladder", [12, 12], [5], 1.0, 7)
    for prec in (a4.device.PREC_FP64, a4.device.PREC_OZAKI_BF16):
        R.buf.fill_(5.0)
        b = _run(a4, R, trip, labels, prec)
        assert b.info()["pairs"] == 0
        assert all(float(R.block(k).abs().max()) == 0.0 for k in R.keys())


def test_split_odd_extents_non_vector_paths(a4):
    # odd segment sizes: row counts and k lengths that are not multiples of
    # 2 or 4 exercise the scalar branches of the layout-specialised kernels
    R, V, T, trip, labels = _make(a4, "ladder", [5, 7, 9], [3, 5], 0.2, 8)
    ref = _reference(R, trip, labels)
    _run(a4, R, trip, labels, a4.device.PREC_OZAKI_BF16, slices=5)
    assert _errors(R, ref).max() <= TOL_SPLIT
    R2, V2, T2, trip2, labels2 = _make(a4, "ladder", [5, 7, 9], [3, 5], 0.2, 8, integer=True)
    _run(a4, R2, trip2, labels2, a4.device.PREC_OZAKI_BF16, slices=1)
    for k, want in _reference(R2, trip2, labels2).items():
        np.testing.assert_array_equal(R2.block(k).cpu().numpy(), want)


@pytest.mark.parametrize("variant", [1, 4])
def test_split_shared_panels_in_different_pair_orders(a4, variant):
    """Destination blocks that use the same operand blocks in different orders
    share a panel whose k layout cannot be contiguous for all of them: the
    stretches break up and every stretch must still multiply zeros past its
    end.  Uneven small K (5 and 7 wide segments, K = 25 .. 49) makes most
    stretch ends ragged.  Integer data with one slice: bit-exact."""
    import random

    R, V, T, trip, labels = _make(a4, "ladder", [5, 7, 6], [3, 4], 0.0, 12, integer=True)
    by_d = {}
    for t in trip:
        by_d.setdefault(t[0].data_ptr(), []).append(t)
    rnd = random.Random(5)
    shuffled = []
    for i, (dp, ts) in enumerate(sorted(by_d.items())):
        ts = list(ts)
        if i % 2:
            rnd.shuffle(ts)
        shuffled += ts
    _run(a4, R, shuffled, labels, a4.device.PREC_OZAKI_BF16, slices=1, variant=variant)
    for k, want in _reference(R, trip, labels).items():
        np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)


@pytest.mark.parametrize("variant", [1, 4])
def test_split_pipelined_right_operand(a4, variant):
    """pipeline=4: the GEMM runs as several launches over split-K ranges while
    a second stream slices the right operand's later ranges; eager and
    graph-captured runs are bit-exact on integer data."""
    import torch

    R, V, T, trip, labels = _make(a4, "ladder", [48] * 4, [8], 0.0, 4, integer=True)
    ref = _reference(R, trip, labels)
    b = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=2,
                        variant=variant, pipeline=4)
    assert b.launches()["gemm_parts"] > 1
    for graph in (False, True):
        R.buf.fill_(float("nan"))
        b.run_graph() if graph else b.run()
        a4.device.sync()
        torch.cuda.synchronize()
        for k, want in ref.items():
            np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)


def test_graph_replay_on_the_legacy_default_stream(a4):
    """run_graph with the caller's legacy default stream (handle 0): the graph
    is captured on the batch's own stream and replayed on the caller's."""
    import torch

    R, V, T, trip, labels = _make(a4, "ladder", [12, 12], [5], 0.0, 21, integer=True)
    ref = _reference(R, trip, labels)
    b = a4.device.Batch(_ptrn(labels), 4, 4, 4, trip, precision=a4.device.PREC_OZAKI_BF16, slices=1)
    for _ in range(2):
        R.buf.fill_(float("nan"))
        b.run_graph(torch.cuda.default_stream())
        torch.cuda.synchronize()
        for k, want in ref.items():
            np.testing.assert_array_equal(R.block(k).cpu().numpy(), want)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matrix_and_outer_product_patterns(a4, precision):
    """Rank-2 blocks (a plain matrix product per pair) and an outer product
    (no contracted index, K = 1) through the batch, both precisions, against
    the oracle."""
    import torch

    rng = np.random.default_rng(41)
    cases = [
        ([1, 2], [1, 3], [3, 2], [37, 29], [37, 45], [45, 29]),  # D(i,j) = L(i,k) R(k,j)
        ([1, 2, 3], [1, 2], [3], [7, 6, 9], [7, 6], [9]),      # D(a,b,c) = L(a,b) R(c)
    ]
    for dl, ll, rl, de, le, re in cases:
        ierr, p = oracle.get_contraction_ptrn(len(dl), len(ll), len(rl), dl + ll + rl)
        assert ierr == 0
        pairs = 3
        Ls = [rng.integers(-60, 61, int(np.prod(le))).astype(np.float64) for _ in range(pairs)]
        Rs = [rng.integers(-60, 61, int(np.prod(re))).astype(np.float64) for _ in range(pairs)]
        D = torch.full((int(np.prod(de)),), float("nan"), dtype=torch.float64, device="cuda")
        tl = [torch.tensor(x, device="cuda") for x in Ls]
        tr = [torch.tensor(x, device="cuda") for x in Rs]
        trip = [(D, tl[q], tr[q], de, le, re) for q in range(pairs)]
        b = a4.device.Batch(p, len(dl), len(ll), len(rl), trip, precision=precision, slices=2)
        b.run()
        a4.device.sync()
        want = sum(oracle.contract_blas(p, Ls[q], le, Rs[q], re, de) for q in range(pairs))
        np.testing.assert_array_equal(D.cpu().numpy(), want)


def test_batch_edge_cases(a4):
    """An empty step; rank-6 operands (four contracted indices); triples that
    disagree on a destination block's extents and a rank-0 destination are
    rejected with a status, not a fault."""
    import torch

    # empty step: creation and runs are no-ops
    p = _ptrn(([1, 2], [1, 3], [3, 2]))
    for prec in (0, 1):
        b = a4.device.Batch(p, 2, 2, 2, [], precision=prec)
        b.run()
        b.run_graph()
        a4.device.sync()
        assert b.info()["pairs"] == 0
    # rank-6 operands: D(a,b,c,d) = L(a,b,e,f,g,h) R(e,f,g,h,c,d)
    rng = np.random.default_rng(17)
    dl, ll, rl = [1, 2, 3, 4], [1, 2, 5, 6, 7, 8], [5, 6, 7, 8, 3, 4]
    de, le, re = [5, 4, 3, 6], [5, 4, 3, 2, 4, 3], [3, 2, 4, 3, 3, 6]
    ierr, p6 = oracle.get_contraction_ptrn(4, 6, 6, dl + ll + rl)
    assert ierr == 0
    Ls = [rng.integers(-50, 51, int(np.prod(le))).astype(np.float64) for _ in range(2)]
    Rs = [rng.integers(-50, 51, int(np.prod(re))).astype(np.float64) for _ in range(2)]
    want = sum(oracle.contract_blas(p6, Ls[q], le, Rs[q], re, de) for q in range(2))
    for prec, slices in ((0, 5), (1, 2)):
        D = torch.full((int(np.prod(de)),), float("nan"), dtype=torch.float64, device="cuda")
        trip = [(D, torch.tensor(Ls[q], device="cuda"), torch.tensor(Rs[q], device="cuda"), de, le, re)
                for q in range(2)]
        b = a4.device.Batch(p6, 4, 6, 6, trip, precision=prec, slices=slices)
        b.run()
        a4.device.sync()
        np.testing.assert_array_equal(D.cpu().numpy(), want)
    # two triples on one destination with different extents
    D = torch.zeros(64, dtype=torch.float64, device="cuda")
    x = torch.zeros(256, dtype=torch.float64, device="cuda")
    bad = [(D, x, x, [8, 8], [8, 8], [8, 8]), (D, x, x, [4, 16], [4, 8], [8, 16])]
    with pytest.raises(a4.device.A4GError):
        a4.device.Batch(p, 2, 2, 2, bad, precision=1)
    # a scalar destination is not a batched contraction
    ierr, p0 = oracle.get_contraction_ptrn(0, 2, 2, [1, 2, 1, 2])
    assert ierr == 0
    with pytest.raises(a4.device.A4GError):
        a4.device.Batch(p0, 0, 2, 2, [(D, x, x, [], [8, 8], [8, 8])], precision=1)
