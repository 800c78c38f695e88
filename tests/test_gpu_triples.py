"""Triples energy on the GPU: the fused denominator + contraction-to-scalar
pass (a4g_energy_contract) against the oracle's restatement of the reference
(T) pattern (rccsdpt_aaa.sialx:2163-2172), and whole triples steps
W = sum_d V1 T - sum_l V2 T -> E = sum W (W / D) through two batches (the
second with negate = 1, beta = 1) in plain FP64 and in split precision.

Tolerances (relative): energy of a given block vs the oracle 1e-13 (the
quotients are the same bits; only the order of the long FP64 sum differs, and
the oracle's own sequential sum carries most of that), and vs the exact sum
(math.fsum) of the oracle's rounded products w * fl(w / eps) 1e-14; W and E of
a step in FP64 1e-12, in split precision (5 slices) 1e-10."""
import math

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


def _energies(o, v, seed):
    rng = np.random.default_rng(seed)
    e = np.concatenate([rng.uniform(-2.0, -0.5, o), rng.uniform(0.2, 5.0, v)])
    return e, np.diag(e).ravel(order="F").copy()


@pytest.mark.parametrize("rank0,rank1,permuted", [(6, 2, False), (6, 2, True), (4, 1, True), (4, 2, False),
                                                  (2, 1, False)])
def test_energy_contract_matches_oracle(a4, rank0, rank1, permuted):
    import torch

    rng = np.random.default_rng(7 + rank0 * 10 + rank1 + permuted)
    segs = [5, 7, 6, 8]  # one occupied segment, three virtual
    norb = sum(segs)
    e, fock = _energies(5, 21, 11)
    f1 = fock if rank1 == 2 else e.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    iv_d = [2 + (q // 2) % 3 if q % 2 == 0 else 1 for q in range(rank0)]
    ext_d = [segs[x - 1] for x in iv_d]
    store = list(range(rank0))
    if permuted:
        store = list(range(0, rank0, 2)) + list(range(1, rank0, 2))
    ext_s = [ext_d[p] for p in store]
    iv_s = [iv_d[p] for p in store]
    den_order = [store.index(q) for q in range(rank0)] if permuted else None
    w = rng.standard_normal(int(np.prod(ext_s)))
    want = oracle.energy_contract(iv_s, ext_s, w, ext1, f1, segs, 0.5, den_order=den_order)
    tw = torch.tensor(w, device="cuda")
    te = torch.tensor(f1, device="cuda")
    esum = torch.full((1,), 0.25, dtype=torch.float64, device="cuda")
    for _ in range(2):  # accumulates
        a4.device.energy_contract(iv_s, ext_s, tw, ext1, te, segs, 0.5, esum, den_order=den_order)
    a4.device.sync()
    got = float(esum.item())
    assert abs(got - (0.25 + 2 * want)) <= 1e-13 * abs(2 * want)
    assert torch.equal(tw.cpu(), torch.tensor(w))  # the block is left unchanged
    # the oracle's quotients (the reference's division, bit for bit), the
    # rounded products summed exactly: the GPU's FP64 sum must be within 1e-14
    order = den_order if den_order is not None else list(range(rank0))
    wp = w
    if order != list(range(rank0)):
        o2n = [0] * rank0
        for q, dim in enumerate(order):
            o2n[dim] = q + 1
        ierr, wp = oracle.tensor_block_copy(ext_s, o2n, w)
        assert ierr == 0
    wd = np.array(wp, dtype=np.float64)
    assert oracle.energy_denominator_rhf([iv_s[d] for d in order], [ext_s[d] for d in order], wd, ext1,
                                         np.ascontiguousarray(f1), segs) == 0
    exact = 0.5 * math.fsum((np.asarray(wp) * wd).tolist())
    one = (got - 0.25) / 2
    assert abs(one - exact) <= 1e-14 * abs(exact), (one, exact)


def test_energy_contract_rejects_bad_order(a4):
    import torch

    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    e = torch.ones(4, dtype=torch.float64, device="cuda")
    with pytest.raises(a4.device.A4GError):
        a4.device.energy_contract([1, 1], [2, 4], x, [4], e, [4], 1.0, x, den_order=[0, 0])


def _triples_problem(o_segs, v_segs, seed):
    import torch

    from aces4_gb300.blocks import BlockArray

    o, v = sum(o_segs), sum(v_segs)
    V1 = BlockArray([v_segs, v_segs, v_segs, o_segs])
    V2 = BlockArray([o_segs, v_segs, o_segs, o_segs])
    T = BlockArray([v_segs, v_segs, o_segs, o_segs])
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    V1.buf.uniform_(-1.0, 1.0, generator=g).div_(v)
    V2.buf.uniform_(-1.0, 1.0, generator=g).div_(v)
    T.buf.normal_(0.0, 0.1, generator=g)
    e, fock = _energies(o, v, seed)
    return V1, V2, T, e, fock


def _run_step(a4, V1, V2, T, o_segs, v_segs, a, b, precision, fock_t, variant=0):
    import torch

    from aces4_gb300.blocks import (TRIPLES_TERM1_LABELS, TRIPLES_TERM2_LABELS, BlockArray,
                                    triples_index_values, triples_step)

    W = BlockArray([v_segs, o_segs, v_segs, o_segs, v_segs, o_segs], present=lambda k: k[0] == a and k[2] == b)
    W.buf.fill_(float("nan"))
    t1, t2 = triples_step(W, V1, V2, T, a, b)
    p1 = oracle.get_contraction_ptrn(6, 4, 4, sum(TRIPLES_TERM1_LABELS, []))[1]
    p2 = oracle.get_contraction_ptrn(6, 4, 4, sum(TRIPLES_TERM2_LABELS, []))[1]
    kw = dict(precision=precision, slices=5, variant=variant)
    b1 = a4.device.Batch(p1, 6, 4, 4, t1, **kw)
    b2 = a4.device.Batch(p2, 6, 4, 4, t2, beta=1, negate=True, **kw)
    b1.run()
    b2.run()
    segs = list(o_segs) + list(v_segs)
    norb = sum(segs)
    esum = torch.zeros(1, dtype=torch.float64, device="cuda")
    for key in W.keys():
        a4.device.energy_contract(triples_index_values(key, len(o_segs)), W.ext(key), W.block(key), [norb, norb],
                                  fock_t, segs, 1.0, esum)
    a4.device.sync()
    flops = b1.info()["flops"] + b2.info()["flops"]
    b1.close()
    b2.close()
    return W, float(esum.item()), flops, (t1, t2, p1, p2)


def test_triples_step_small_vs_oracle(a4):
    """o=6 (one segment), v=24 (2 x 12): both precisions against the oracle's
    BLAS path for W and the oracle's (T) energy pattern for E."""
    import torch

    o_segs, v_segs = [6], [12, 12]
    V1, V2, T, e, fock = _triples_problem(o_segs, v_segs, 5)
    ft = torch.tensor(fock, device="cuda")
    res = {}
    for prec in (a4.device.PREC_FP64, a4.device.PREC_OZAKI_BF16):
        res[prec] = _run_step(a4, V1, V2, T, o_segs, v_segs, 0, 1, prec, ft)
    W, E64, flops, (t1, t2, p1, p2) = res[a4.device.PREC_FP64]
    Wsp, Esp, _, _ = res[a4.device.PREC_OZAKI_BF16]
    segs = o_segs + v_segs
    norb = sum(segs)
    E_ref = 0.0
    for key in W.keys():
        dptr = W.block(key).data_ptr()
        de = W.ext(key)
        want = np.zeros(W.size(key))
        for trip, p, sign in ((t1, p1, 1.0), (t2, p2, -1.0)):
            for d, l, r, _, le, re in trip:
                if d.data_ptr() == dptr:
                    want += sign * oracle.contract_blas(p, l.cpu().numpy(), le, r.cpu().numpy(), re, de)
        got64 = W.block(key).cpu().numpy()
        gotsp = Wsp.block(key).cpu().numpy()
        nrm = np.linalg.norm(want)
        assert np.linalg.norm(got64 - want) <= 1e-12 * nrm
        assert np.linalg.norm(gotsp - want) <= 1e-10 * nrm
        from aces4_gb300.blocks import triples_index_values

        E_ref += oracle.energy_contract(triples_index_values(key, len(o_segs)), de, want, [norb, norb], fock, segs, 1.0)
    assert E_ref < 0
    assert abs(E64 - E_ref) <= 1e-12 * abs(E_ref)
    assert abs(Esp - E_ref) <= 1e-10 * abs(E_ref)
    assert abs(flops - 2 * 24 * 12 * 12 * 6 ** 3 * (24 + 6)) < 1  # 2 v_a v_b v o^3 (v + o) for this step


def test_triples_step_every_form_gives_the_same_bits(a4):
    """o=8, v=48 (3 x 16): the two terms through each tensor-core form (the
    workspace forms and the direct ones, W unit-stride on the right operand so
    both batches run with the operands' roles exchanged) give identical W."""
    import torch

    o_segs, v_segs = [8], [16, 16, 16]
    V1, V2, T, e, fock = _triples_problem(o_segs, v_segs, 13)
    ft = torch.tensor(fock, device="cuda")
    ref = None
    for variant in range(1, 7):
        W, E, _, _ = _run_step(a4, V1, V2, T, o_segs, v_segs, 1, 2, a4.device.PREC_OZAKI_BF16, ft, variant)
        bits = W.buf.clone().view(torch.int64)
        if ref is None:
            ref, E_ref = bits, E
        else:
            assert torch.equal(bits, ref), variant
            assert E == E_ref, variant


def test_triples_full_size_step(a4):
    """o=24 (one segment of 24), v=240 (10 x 24): one pardo step (a, b) =
    (0, 1) with every c: 10 W blocks of 24^6, 110 block pairs, 1.01e12 flop.
    Split precision against plain FP64 on every W block and on E."""
    import torch

    o_segs, v_segs = [24], [24] * 10
    V1, V2, T, e, fock = _triples_problem(o_segs, v_segs, 9)
    ft = torch.tensor(fock, device="cuda")
    W64, E64, flops, _ = _run_step(a4, V1, V2, T, o_segs, v_segs, 0, 1, a4.device.PREC_FP64, ft)
    assert abs(flops - 2 * 24 ** 2 * 240 * 24 ** 3 * (240 + 24)) < 1e3
    ref = W64.buf.clone()
    del W64
    Wsp, Esp, _, _ = _run_step(a4, V1, V2, T, o_segs, v_segs, 0, 1, a4.device.PREC_OZAKI_BF16, ft)
    for key in Wsp.keys():
        o, n = Wsp.offsets[key], Wsp.size(key)
        a, b = Wsp.buf[o:o + n], ref[o:o + n]
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) <= 1e-10
    assert E64 < 0
    assert abs(Esp - E64) <= 1e-10 * abs(E64)
