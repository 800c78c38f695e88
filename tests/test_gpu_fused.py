"""The fused triples step on the GPU (a4g_fused_*): both contraction terms of
W(a,i,b,j,c,k) = sum_d V1(b,c,d,k) T(a,d,i,j) - sum_l V2(l,c,j,k) T(a,b,i,l)
in one split-precision pass (rccsdpt_aaa.sialx:2163-2172), W either stored or
reduced straight to the (T) energy E = sum W fl(W / eps) without being
stored.

Tolerances (relative, 5 slices): W against the oracle's BLAS path 1e-10 per
block (Frobenius), E against the oracle's (T) energy pattern 1e-10, the same
bound the two-batch split path is held to; two runs of the energy form give
the same bits."""
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


def _problem(o_segs, v_segs, seed):
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
    rng = np.random.default_rng(seed)
    e = np.concatenate([rng.uniform(-2.0, -0.5, o), rng.uniform(0.2, 5.0, v)])
    fock = np.diag(e).ravel(order="F").copy()
    return V1, V2, T, fock


def _step(V1, V2, T, o_segs, v_segs, a, b):
    from aces4_gb300.blocks import (TRIPLES_TERM1_LABELS, TRIPLES_TERM2_LABELS, BlockArray, triples_step)

    W = BlockArray([v_segs, o_segs, v_segs, o_segs, v_segs, o_segs], present=lambda k: k[0] == a and k[2] == b)
    W.buf.fill_(float("nan"))
    t1, t2 = triples_step(W, V1, V2, T, a, b)
    p1 = oracle.get_contraction_ptrn(6, 4, 4, sum(TRIPLES_TERM1_LABELS, []))[1]
    p2 = oracle.get_contraction_ptrn(6, 4, 4, sum(TRIPLES_TERM2_LABELS, []))[1]
    return W, [(p1, t1, 1), (p2, t2, -1)]


def _energy_args(W, o_segs, v_segs, fock_t):
    from aces4_gb300.blocks import triples_index_values

    segs = list(o_segs) + list(v_segs)
    norb = sum(segs)
    keys = list(W.keys())
    return dict(blocks=[W.block(k) for k in keys], index_values=[triples_index_values(k, len(o_segs)) for k in keys],
                ext1=[norb, norb], e_or_fock=fock_t, seg_sizes=segs, efact=1.0)


def _oracle_W_E(W, terms, o_segs, v_segs, fock):
    from aces4_gb300.blocks import triples_index_values

    segs = list(o_segs) + list(v_segs)
    norb = sum(segs)
    Ws, E = {}, 0.0
    for key in W.keys():
        dptr, de = W.block(key).data_ptr(), W.ext(key)
        want = np.zeros(W.size(key))
        for p, trip, sign in terms:
            for d, l, r, _, le, re in trip:
                if d.data_ptr() == dptr:
                    want += sign * oracle.contract_blas(p, l.cpu().numpy(), le, r.cpu().numpy(), re, de)
        Ws[key] = want
        E += oracle.energy_contract(triples_index_values(key, len(o_segs)), de, want, [norb, norb], fock, segs, 1.0)
    return Ws, E


@pytest.mark.parametrize("o_segs,v_segs,a,b", [([6], [12, 12], 0, 1),         # even segments
                                               ([3, 5], [5, 7, 4], 0, 2)])   # uneven, odd k lengths
def test_fused_store_and_energy_match_oracle(a4, o_segs, v_segs, a, b):
    import torch

    V1, V2, T, fock = _problem(o_segs, v_segs, 21 + len(v_segs))
    ft = torch.tensor(fock, device="cuda")
    W, terms = _step(V1, V2, T, o_segs, v_segs, a, b)
    Wref, Eref = _oracle_W_E(W, terms, o_segs, v_segs, fock)
    f = a4.device.Fused(6, 4, 4, terms)
    f.run()
    a4.device.sync()
    for key in W.keys():
        got = W.block(key).cpu().numpy()
        nrm = np.linalg.norm(Wref[key])
        assert np.all(np.isfinite(got)), key  # every element written
        assert np.linalg.norm(got - Wref[key]) <= 1e-10 * nrm, key
    f.close()
    W.buf.fill_(float("nan"))  # the energy form stores nothing
    fe = a4.device.Fused(6, 4, 4, terms, energy=_energy_args(W, o_segs, v_segs, ft))
    esum = torch.full((1,), 0.5, dtype=torch.float64, device="cuda")
    fe.run(esum)
    a4.device.sync()
    got = float(esum.item()) - 0.5
    assert Eref < 0
    assert abs(got - Eref) <= 1e-10 * abs(Eref)
    assert bool(torch.isnan(W.buf).all())
    info = fe.info()
    assert info["elements"] == sum(W.size(k) for k in W.keys())
    o, v = sum(o_segs), sum(v_segs)
    va, vb = v_segs[a], v_segs[b]
    assert abs(info["flops"] - 2 * va * vb * v * o ** 3 * (v + o)) < 1
    fe.close()


def test_fused_energy_is_deterministic_and_accumulates(a4):
    import torch

    o_segs, v_segs = [8], [16, 16, 16]
    V1, V2, T, fock = _problem(o_segs, v_segs, 5)
    ft = torch.tensor(fock, device="cuda")
    W, terms = _step(V1, V2, T, o_segs, v_segs, 1, 2)
    ea = _energy_args(W, o_segs, v_segs, ft)
    ea["efact"] = 0.5
    fe = a4.device.Fused(6, 4, 4, terms, energy=ea)
    e1 = torch.zeros(1, dtype=torch.float64, device="cuda")
    e2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    fe.run(e1)
    fe.run(e2)
    fe.run(e2)
    a4.device.sync()
    assert float(e1.item()) != 0.0
    assert abs(float(e2.item()) - 2 * float(e1.item())) <= 1e-15 * abs(float(e2.item()))
    e3 = torch.zeros(1, dtype=torch.float64, device="cuda")
    fe.run(e3)
    a4.device.sync()
    assert float(e3.item()) == float(e1.item())
    _, Eref = _oracle_W_E(W, terms, o_segs, v_segs, fock)
    assert abs(float(e1.item()) - 0.5 * Eref) <= 1e-10 * abs(0.5 * Eref)
    fe.close()


def test_fused_store_beta_and_single_term(a4):
    """beta = 1 adds the fused sum to D; one term alone is a plain direct-form
    contraction."""
    import torch

    o_segs, v_segs = [6], [12, 12]
    V1, V2, T, fock = _problem(o_segs, v_segs, 8)
    W, terms = _step(V1, V2, T, o_segs, v_segs, 1, 0)
    W.buf.fill_(0.25)
    f = a4.device.Fused(6, 4, 4, terms, beta=1)
    f.run()
    a4.device.sync()
    Wref, _ = _oracle_W_E(W, terms, o_segs, v_segs, fock)
    for key in W.keys():
        want = Wref[key] + 0.25
        got = W.block(key).cpu().numpy()
        assert np.linalg.norm(got - want) <= 1e-10 * np.linalg.norm(want), key
    f.close()
    W.buf.fill_(float("nan"))
    f1 = a4.device.Fused(6, 4, 4, terms[:1])
    f1.run()
    a4.device.sync()
    Wref1, _ = _oracle_W_E(W, terms[:1], o_segs, v_segs, fock)
    for key in W.keys():
        got = W.block(key).cpu().numpy()
        assert np.linalg.norm(got - Wref1[key]) <= 1e-10 * np.linalg.norm(Wref1[key]), key
    f1.close()


def test_fused_rejects_what_it_does_not_cover(a4):
    import torch

    o_segs, v_segs = [4], [6, 6]
    V1, V2, T, fock = _problem(o_segs, v_segs, 3)
    W, terms = _step(V1, V2, T, o_segs, v_segs, 0, 1)
    with pytest.raises(a4.device.A4GError):
        a4.device.Fused(6, 4, 4, [terms[0], terms[1], terms[0]])  # at most two terms
    with pytest.raises(a4.device.A4GError):
        a4.device.Fused(6, 4, 4, [(terms[0][0], terms[0][1], 2)])  # sign must be +-1
    ft = torch.tensor(fock, device="cuda")
    ea = _energy_args(W, o_segs, v_segs, ft)
    ea["den_order"] = [0, 1, 4, 3, 2, 5]  # the last term on b, a fixed index of the sub-problems
    with pytest.raises(a4.device.A4GError) as ei:
        a4.device.Fused(6, 4, 4, terms, energy=ea)
    assert ei.value.rc == 6


def test_fused_rebind_equals_fresh_creation(a4):
    """The (T) loop's next (a, b) step through a4g_fused_rebind: the same bits
    as a step created on those blocks, in the energy and the store form; a
    structure that differs is rejected."""
    import torch

    o_segs, v_segs = [6], [12, 12, 12]
    V1, V2, T, fock = _problem(o_segs, v_segs, 31)
    ft = torch.tensor(fock, device="cuda")
    W01, terms01 = _step(V1, V2, T, o_segs, v_segs, 0, 1)
    W20, terms20 = _step(V1, V2, T, o_segs, v_segs, 2, 0)
    fe = a4.device.Fused(6, 4, 4, terms01, energy=_energy_args(W01, o_segs, v_segs, ft))
    e = torch.zeros(2, dtype=torch.float64, device="cuda")
    fe.run(e[0:1])
    fe.rebind(terms20, energy=_energy_args(W20, o_segs, v_segs, ft))
    fe.run(e[1:2])
    fresh = a4.device.Fused(6, 4, 4, terms20, energy=_energy_args(W20, o_segs, v_segs, ft))
    e2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    fresh.run(e2)
    a4.device.sync()
    assert float(e[1].item()) == float(e2.item())
    _, Eref = _oracle_W_E(W20, terms20, o_segs, v_segs, fock)
    assert abs(float(e[1].item()) - Eref) <= 1e-10 * abs(Eref)
    _, Eref01 = _oracle_W_E(W01, terms01, o_segs, v_segs, fock)
    assert abs(float(e[0].item()) - Eref01) <= 1e-10 * abs(Eref01)
    fresh.close()
    # store form: rebound W20 equals a fresh creation's W20, bit for bit
    fs = a4.device.Fused(6, 4, 4, terms01)
    fs.rebind(terms20)
    fs.run()
    a4.device.sync()
    got = W20.buf.clone()
    W20.buf.fill_(float("nan"))
    f2 = a4.device.Fused(6, 4, 4, terms20)
    f2.run()
    a4.device.sync()
    assert torch.equal(got.view(torch.int64), W20.buf.view(torch.int64))
    # another structure: one term only
    with pytest.raises(a4.device.A4GError):
        fs.rebind(terms20[:1])
    fe.close(), fs.close(), f2.close()


def test_fused_permuted_storage_and_rank4(a4):
    """Other storage orders and ranks through the same planner: W stored as
    (a,b,c,i,j,k) with the denominator's order given (den_order), and a
    single-term rank-4 ring contraction R(a,i,b,j) = V(a,k,c,i) T(c,b,k,j)
    with a 1-D orbital-energy array, whose denominator's last term (b) is a
    column index.  Store and energy forms against the oracle."""
    import itertools

    import torch

    from aces4_gb300.blocks import BlockArray, ring_triples

    # (a,b,c,i,j,k) storage; labels a=1 i=2 b=3 j=4 c=5 k=6 d=7 l=8
    o_segs, v_segs = [5], [6, 7]
    nocc = len(o_segs)
    V1, V2, T, fock = _problem(o_segs, v_segs, 41)
    a, b = 1, 0
    W = BlockArray([v_segs, v_segs, v_segs, o_segs, o_segs, o_segs], present=lambda k: k[0] == a and k[1] == b)
    W.buf.fill_(float("nan"))
    wl = [1, 3, 5, 2, 4, 6]
    p1 = oracle.get_contraction_ptrn(6, 4, 4, wl + [3, 5, 7, 6] + [1, 7, 2, 4])[1]
    p2 = oracle.get_contraction_ptrn(6, 4, 4, wl + [8, 5, 4, 6] + [1, 3, 2, 8])[1]
    t1, t2 = [], []
    nv, no = len(v_segs), len(o_segs)
    for c in range(nv):
        for i, j, k in itertools.product(range(no), repeat=3):
            wk = (a, b, c, i, j, k)
            for d in range(nv):
                t1.append((W.block(wk), V1.block((b, c, d, k)), T.block((a, d, i, j)), W.ext(wk),
                           V1.ext((b, c, d, k)), T.ext((a, d, i, j))))
            for l in range(no):
                t2.append((W.block(wk), V2.block((l, c, j, k)), T.block((a, b, i, l)), W.ext(wk),
                           V2.ext((l, c, j, k)), T.ext((a, b, i, l))))
    terms = [(p1, t1, 1), (p2, t2, -1)]
    segs = list(o_segs) + list(v_segs)
    norb = sum(segs)
    den_order = [0, 3, 1, 4, 2, 5]  # denominator positions (a,i,b,j,c,k) -> storage dims
    keys = W.keys()
    ivs = {k: [nocc + k[0] + 1, nocc + k[1] + 1, nocc + k[2] + 1, k[3] + 1, k[4] + 1, k[5] + 1] for k in keys}
    Wref, Eref = {}, 0.0
    for key in keys:
        dp, de = W.block(key).data_ptr(), W.ext(key)
        want = np.zeros(W.size(key))
        for p, trip, sign in terms:
            for d_, l_, r_, _, le, re in trip:
                if d_.data_ptr() == dp:
                    want += sign * oracle.contract_blas(p, l_.cpu().numpy(), le, r_.cpu().numpy(), re, de)
        Wref[key] = want
        Eref += oracle.energy_contract(ivs[key], de, want, [norb, norb], fock, segs, 1.0, den_order=den_order)
    f = a4.device.Fused(6, 4, 4, terms)
    f.run()
    a4.device.sync()
    for key in keys:
        got = W.block(key).cpu().numpy()
        assert np.linalg.norm(got - Wref[key]) <= 1e-10 * np.linalg.norm(Wref[key]), key
    f.close()
    ft = torch.tensor(fock, device="cuda")
    fe = a4.device.Fused(6, 4, 4, terms, energy=dict(blocks=[W.block(k) for k in keys],
                                                    index_values=[ivs[k] for k in keys], ext1=[norb, norb],
                                                    e_or_fock=ft, seg_sizes=segs, den_order=den_order))
    e = torch.zeros(1, dtype=torch.float64, device="cuda")
    fe.run(e)
    a4.device.sync()
    assert abs(float(e.item()) - Eref) <= 1e-10 * abs(Eref)
    fe.close()

    # rank 4, one term: R(a,i,b,j) = V(a,k,c,i) T(c,b,k,j), labels a=1 i=3 b=2 j=4 c=5 k=7
    o_s, v_s = [4, 3], [5, 6]
    R = BlockArray([v_s, o_s, v_s, o_s])
    V = BlockArray([v_s, o_s, v_s, o_s])
    T4 = BlockArray([v_s, v_s, o_s, o_s])
    g = torch.Generator(device="cuda")
    g.manual_seed(43)
    V.buf.uniform_(-1.0, 1.0, generator=g)
    T4.buf.normal_(0.0, 0.1, generator=g)
    trip = ring_triples(R, V, T4)
    ptrn = oracle.get_contraction_ptrn(4, 4, 4, [1, 3, 2, 4] + [1, 7, 5, 3] + [5, 2, 7, 4])[1]
    rng = np.random.default_rng(43)
    n_o, n_v = sum(o_s), sum(v_s)
    e1 = np.concatenate([rng.uniform(-2.0, -0.5, n_o), rng.uniform(0.2, 5.0, n_v)])
    segs4 = list(o_s) + list(v_s)
    no4 = len(o_s)
    keys4 = R.keys()
    iv4 = {k: [no4 + k[0] + 1, k[1] + 1, no4 + k[2] + 1, k[3] + 1] for k in keys4}
    E4 = 0.0
    for key in keys4:
        dp, de = R.block(key).data_ptr(), R.ext(key)
        want = np.zeros(R.size(key))
        for d_, l_, r_, _, le, re in trip:
            if d_.data_ptr() == dp:
                want += oracle.contract_blas(ptrn, l_.cpu().numpy(), le, r_.cpu().numpy(), re, de)
        E4 += oracle.energy_contract(iv4[key], de, want, [n_o + n_v], e1, segs4, 0.25)
    f4 = a4.device.Fused(4, 4, 4, [(ptrn, trip, 1)], energy=dict(
        blocks=[R.block(k) for k in keys4], index_values=[iv4[k] for k in keys4], ext1=[n_o + n_v],
        e_or_fock=torch.tensor(e1, device="cuda"), seg_sizes=segs4, efact=0.25))
    e4 = torch.zeros(1, dtype=torch.float64, device="cuda")
    f4.run(e4)
    a4.device.sync()
    assert abs(float(e4.item()) - E4) <= 1e-10 * abs(E4)
    f4.close()


@pytest.mark.parametrize("o_segs,v_segs,a,b,slices", [([6], [12, 12], 0, 1, 5),          # one tile column
                                                      ([3, 5], [5, 7, 4], 0, 2, 5),     # ragged tiles, odd k
                                                      ([8], [16, 16, 16], 1, 2, 4),     # 256-row sub-problems
                                                      ([8], [16, 16, 16], 2, 0, 3)])
def test_fused_forms_agree(a4, o_segs, v_segs, a, b, slices):
    """The two GEMM forms of the fused step: all levels at once (variant 7,
    128 x 64 tiles, levels 3 and 4 over two k halves) and one level at a time
    (variant 5, 128 x 128 tiles) form the same exact integer sums, so the
    stored W has the same bits (overwrite and beta = 1); the energies differ
    in the order of the partial sums only."""
    import torch

    V1, V2, T, fock = _problem(o_segs, v_segs, 50 + slices)
    ft = torch.tensor(fock, device="cuda")
    W, terms = _step(V1, V2, T, o_segs, v_segs, a, b)
    out = {}
    for variant in (5, 7):
        for beta in (0, 1):
            W.buf.fill_(0.375 if beta else float("nan"))
            f = a4.device.Fused(6, 4, 4, terms, slices=slices, beta=beta, variant=variant)
            assert f.info()["form"] == variant
            f.run()
            a4.device.sync()
            out[variant, beta] = W.buf.clone()
            f.close()
    for beta in (0, 1):
        for key in W.keys():  # every element written (the gaps between blocks are not)
            off = W.offsets[key]
            assert bool(torch.isfinite(out[7, beta][off:off + W.size(key)]).all()), (key, beta)
        assert torch.equal(out[5, beta].view(torch.int64), out[7, beta].view(torch.int64)), beta
    if slices == 5:
        Wref, Eref = _oracle_W_E(W, terms, o_segs, v_segs, fock)
        for key in W.keys():
            off = W.offsets[key]
            got = out[7, 0][off:off + W.size(key)].cpu().numpy()
            assert np.linalg.norm(got - Wref[key]) <= 1e-10 * np.linalg.norm(Wref[key]), key
    e = {}
    for variant in (5, 7):
        fe = a4.device.Fused(6, 4, 4, terms, slices=slices, energy=_energy_args(W, o_segs, v_segs, ft),
                             variant=variant)
        e[variant] = torch.zeros(1, dtype=torch.float64, device="cuda")
        fe.run(e[variant])
        a4.device.sync()
        fe.close()
    e5, e7 = float(e[5].item()), float(e[7].item())
    assert e5 < 0 and abs(e7 - e5) <= 1e-13 * abs(e5)
    if slices == 5:
        assert abs(e7 - Eref) <= 1e-10 * abs(Eref)


def test_fused_form_choice(a4):
    """Automatic choice: the all-levels form where it fits, else one level at
    a time (six slices; a k range above 320); variant 7 beyond its range is
    A4G_ERR_UNSUPPORTED."""
    o_segs, v_segs = [4], [6, 6]
    V1, V2, T, _ = _problem(o_segs, v_segs, 3)
    W, terms = _step(V1, V2, T, o_segs, v_segs, 0, 1)
    f = a4.device.Fused(6, 4, 4, terms)
    assert f.info()["form"] == 7
    f.close()
    f6 = a4.device.Fused(6, 4, 4, terms, slices=6)
    assert f6.info()["form"] == 5
    f6.close()
    with pytest.raises(a4.device.A4GError) as ei:
        a4.device.Fused(6, 4, 4, terms, slices=6, variant=7)
    assert ei.value.rc == 6
    # k of term 1: 41 virtual segments of 8 = 328, a stretch of 384 (> 320)
    o_segs, v_segs = [1], [8] * 41
    V1, V2, T, _ = _problem(o_segs, v_segs, 4)
    W, terms = _step(V1, V2, T, o_segs, v_segs, 0, 1)
    f = a4.device.Fused(6, 4, 4, terms)
    assert f.info()["form"] == 5
    f.close()
    with pytest.raises(a4.device.A4GError) as ei:
        a4.device.Fused(6, 4, 4, terms, variant=7)
    assert ei.value.rc == 6
