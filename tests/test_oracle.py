"""The CPU oracle pinned against the reference's known-answer tests and against
independent numpy restatements of each block operation (CPU only)."""
import zlib

import numpy as np
import pytest

from oracle import oracle
from tests import kat


def _einsum_labels(dl, ll, rl):
    letters = {}
    for lab in list(dl) + list(ll) + list(rl):
        letters.setdefault(lab, "abcdefghijklmnopqrstuvwxyz"[len(letters)])
    f = lambda labs: "".join(letters[x] for x in labs)
    return f"{f(ll)},{f(rl)}->{f(dl)}"


def _blk(flat, ext):
    return flat.reshape(ext, order="F") if len(ext) else flat.reshape(())


@pytest.mark.parametrize("name", ["contraction_small_test", "contraction_small_test2", "contract_to_scalar"])
def test_kat_contractions(name):
    c = kat.case(name)
    L = kat.fill(c["l_fill"], kat.size(c["l_ext"]))
    R = kat.fill(c["r_fill"], kat.size(c["r_ext"]))
    ierr, D = oracle.contract_labels(c["d_labels"], c["l_labels"], c["r_labels"], L, c["l_ext"], R,
                                     c["r_ext"], c["d_ext"])
    assert ierr == 0
    np.testing.assert_array_equal(D, np.array(c["expected"]))


@pytest.mark.parametrize("name", ["transpose_tmp", "transpose4d_tmp", "transpose4d_square_tmp"])
def test_kat_permutes(name):
    c = kat.case(name)
    S = kat.fill(c["s_fill"], kat.size(c["s_ext"]))
    perm = kat.perm_from_labels(c["d_labels"], c["s_labels"])
    ierr, D = oracle.tensor_block_copy(c["s_ext"], perm, S)
    assert ierr == 0
    np.testing.assert_array_equal(D, np.array(c["expected"]))
    if "esum" in c:
        sl, dl = c["s_labels"], c["d_labels"]
        e1 = oracle.contract_labels([], sl, sl, S, c["s_ext"], S, c["s_ext"], [])[1][0]
        e2 = oracle.contract_labels([], dl, dl, D, c["d_ext"], D, c["d_ext"], [])[1][0]
        e3 = oracle.contract_labels([], sl, dl, S, c["s_ext"], D, c["d_ext"], [])[1][0]
        assert [e1, e2, e3] == c["esum"]


def test_kat_sum_op_and_self_multiply():
    c = kat.case("sum_op")
    n = kat.size(c["ext"])
    a = kat.fill(c["a_fill"], n)
    cc = kat.fill(c["c_fill"], n)
    d = np.empty(n)
    e = np.empty(n)
    ids = [1, 2]
    assert oracle.block_add_sub(0, ids, ids, ids, c["ext"], 0, d, a, cc) == 0
    assert oracle.block_add_sub(1, ids, ids, ids, c["ext"], 0, e, d, cc) == 0
    np.testing.assert_array_equal(d, c["expected_d"])
    np.testing.assert_array_equal(e, c["expected_e"])

    s = kat.case("self_multiply_test")
    a = kat.fill(s["a_fill"], n)
    assert oracle.block_add_sub(0, ids, ids, ids, s["ext"], 1, a, a.copy(), a.copy()) == 0
    assert oracle.tensor_block_scale(a, s["ext"], s["factor"]) == 0
    np.testing.assert_array_equal(a, s["expected"])


def test_get_contraction_ptrn_errors():
    # ierr 1: negative rank; 2: odd label count; 3: no operands; 4: unpaired
    # label; 5: label used more than twice; 6: trace / operand-only pairing
    assert oracle.get_contraction_ptrn(-1, 1, 1, [1, 1])[0] == 1
    assert oracle.get_contraction_ptrn(1, 1, 1, [1, 1, 2])[0] == 2
    assert oracle.get_contraction_ptrn(2, 0, 0, [1, 1])[0] == 3
    assert oracle.get_contraction_ptrn(0, 0, 0, [])[0] == 0
    assert oracle.get_contraction_ptrn(1, 1, 2, [1, 2, 1, 3])[0] == 4
    assert oracle.get_contraction_ptrn(0, 2, 2, [1, 1, 1, 1])[0] == 5
    assert oracle.get_contraction_ptrn(2, 2, 0, [1, 2, 1, 1])[0] == 4  # sorted 1,1,1,2
    assert oracle.get_contraction_ptrn(2, 2, 0, [1, 1, 1, 1])[0] == 5
    assert oracle.get_contraction_ptrn(0, 2, 2, [1, 1, 2, 2])[0] == 6  # trace in left
    assert oracle.get_contraction_ptrn(2, 1, 1, [1, 1, 2, 2])[0] == 6  # repeated dest label


def test_get_contraction_ptrn_values():
    # ladder: R(a,b,i,j) = V(a,b,c,d) T(c,d,i,j)
    ierr, p = oracle.get_contraction_ptrn(4, 4, 4, [1, 2, 3, 4, 1, 2, 5, 6, 5, 6, 3, 4])
    assert ierr == 0 and p == [1, 2, -1, -2, -3, -4, 3, 4]
    # ring: R(a,i,b,j) = V(a,k,c,i) T(c,b,k,j)
    ierr, p = oracle.get_contraction_ptrn(4, 4, 4, [1, 2, 3, 4, 1, 5, 6, 2, 6, 3, 5, 4])
    assert ierr == 0 and p == [1, -3, -1, 2, -3, 3, -2, 4]


def test_contr_ptrn_ok():
    assert oracle.contr_ptrn_ok([1, 2, -1, -2, -3, -4, 3, 4], [3, 3, 4, 4], [4, 4, 5, 5], [3, 3, 5, 5])
    assert not oracle.contr_ptrn_ok([1, 2, -1, -2, -3, -4, 3, 4], [3, 3, 4, 4], [4, 9, 5, 5], [3, 3, 5, 5])
    assert not oracle.contr_ptrn_ok([1, 1, -1, -2, -3, -4, 3, 4], [3, 3, 4, 4], [4, 4, 5, 5], [3, 3, 5, 5])


RANDOM_PATTERNS = [
    # (d labels, l labels, r labels)
    ("abij", "abcd", "cdij"),      # ladder
    ("aibj", "akci", "cbkj"),      # ring (both operands permuted)
    ("abcijk", "bcdk", "adij"),    # triples term 1
    ("il", "ijkl", "jk"),
    ("ba", "ac", "cb"),            # destination permuted
    ("", "abc", "cab"),            # full contraction, permuted right
    ("ab", "a", "b"),              # outer product
    ("ab", "ab", ""),              # right scalar
    ("ba", "", "ab"),              # left scalar, permuted dest
    ("", "", ""),                  # scalar * scalar
    ("fedcba", "abcx", "xdef"),    # rank 6 destination
]


@pytest.mark.parametrize("dl,ll,rl", RANDOM_PATTERNS)
def test_contract_random_vs_einsum(dl, ll, rl):
    rng = np.random.default_rng(zlib.crc32((dl + "|" + ll + "|" + rl).encode()))
    ext = {lab: int(rng.integers(2, 6)) for lab in set(dl + ll + rl)}
    lid = {lab: i + 1 for i, lab in enumerate(sorted(set(dl + ll + rl)))}
    le, re, de = [ext[x] for x in ll], [ext[x] for x in rl], [ext[x] for x in dl]
    L = rng.standard_normal(kat.size(le))
    R = rng.standard_normal(kat.size(re))
    ierr, D = oracle.contract_labels([lid[x] for x in dl], [lid[x] for x in ll], [lid[x] for x in rl],
                                     L, le, R, re, de)
    assert ierr == 0
    ref = np.einsum(_einsum_labels(dl, ll, rl), _blk(L, le), _blk(R, re))
    np.testing.assert_allclose(D, np.asarray(ref).ravel(order="F"), rtol=1e-12, atol=1e-12)
    # the BLAS-path restatement used as the CPU baseline agrees too
    if dl and ll and rl:
        _, p = oracle.get_contraction_ptrn(len(dl), len(ll), len(rl),
                                           [lid[x] for x in dl + ll + rl])
        D2 = oracle.contract_blas(p, L, le, R, re, de)
        np.testing.assert_allclose(D2, D, rtol=1e-12, atol=1e-12)


def test_contract_overwrites_and_bad_pattern():
    L = np.ones(6)
    R = np.ones(6)
    D = np.full(4, 7.0)
    # D(a,b) = L(a,c) R(c,b): 2x3 * 3x2
    assert oracle.tensor_block_contract([1, -1, -2, 2], L, [2, 3], R, [3, 2], D, [2, 2]) == 0
    np.testing.assert_array_equal(D, 3.0)
    # extent mismatch -> ierr 1, negative rank -> -1
    assert oracle.tensor_block_contract([1, -1, -2, 2], L, [2, 3], R, [4, 2], D, [2, 2]) == 1


def test_permute_random_vs_numpy():
    rng = np.random.default_rng(3)
    for rank in range(1, 7):
        ext = [int(x) for x in rng.integers(1, 6, rank)]
        perm = [int(x) + 1 for x in rng.permutation(rank)]
        S = rng.standard_normal(kat.size(ext))
        ierr, D = oracle.tensor_block_copy(ext, perm, S)
        assert ierr == 0
        n2o = [0] * rank
        for i, p in enumerate(perm):
            n2o[p - 1] = i
        ref = np.transpose(S.reshape(ext, order="F"), n2o).ravel(order="F")
        np.testing.assert_array_equal(D, ref)


def test_elementwise_ops():
    rng = np.random.default_rng(5)
    ext = [3, 4, 5]
    t0 = rng.standard_normal(60)
    t1 = rng.standard_normal(60)
    a = t0.copy()
    assert oracle.tensor_block_add(ext, a, t1, 0.5) == 0
    np.testing.assert_array_equal(a, t0 + t1 * 0.5)
    a = t0.copy()
    oracle.tensor_block_add(ext, a, t1, 1.0 + 5e-14)  # treated as exactly 1
    np.testing.assert_array_equal(a, t0 + t1)
    a = t0.copy()
    oracle.tensor_block_scale(a, ext, -2.5)
    np.testing.assert_array_equal(a, t0 * -2.5)
    v, ierr = oracle.tensor_block_norm2(t0, ext)
    assert ierr == 0 and abs(v - float(np.sum(t0 * t0))) < 1e-12
    a = t0.copy()
    oracle.tensor_block_init(a, ext, 3.25)
    np.testing.assert_array_equal(a, 3.25)
    d = np.empty(60)
    oracle.block_scale_and_copy(d, t0, 3.0)
    np.testing.assert_array_equal(d, t0 * 3.0)
    a = t0.copy()
    oracle.block_increment(a, 0.125)
    np.testing.assert_array_equal(a, t0 + 0.125)
    a = t0.copy()
    oracle.block_accumulate(a, t1)
    np.testing.assert_array_equal(a, t0 + t1)


def test_slice_insert():
    rng = np.random.default_rng(6)
    text, sext, beg = [6, 5, 4], [3, 2, 2], [2, 1, 1]
    T = rng.standard_normal(120)
    ierr, S = oracle.tensor_block_slice(T, text, sext, beg)
    assert ierr == 0
    Tb = T.reshape(text, order="F")
    np.testing.assert_array_equal(S, Tb[2:5, 1:3, 1:3].ravel(order="F"))
    T2 = np.zeros(120)
    assert oracle.tensor_block_insert(T2, text, S, sext, beg) == 0
    ref = np.zeros(text)
    ref[2:5, 1:3, 1:3] = Tb[2:5, 1:3, 1:3]
    np.testing.assert_array_equal(T2, ref.ravel(order="F"))


def test_block_add_permuted_rhs():
    rng = np.random.default_rng(7)
    ext_d = [3, 4, 5]  # d(i,j,k) += r(k,i,j)
    r_ext = [5, 3, 4]
    d = rng.standard_normal(60)
    r = rng.standard_normal(60)
    out = d.copy()
    assert oracle.block_add_sub(0, [1, 2, 3], [1, 2, 3], [3, 1, 2], r_ext, 1, out, d.copy(), r) == 0
    ref = d.reshape(ext_d, order="F") + np.transpose(r.reshape(r_ext, order="F"), (1, 2, 0))
    np.testing.assert_array_equal(out, ref.ravel(order="F"))
    # without the += form the labels must agree
    assert oracle.block_add_sub(0, [1, 2, 3], [1, 2, 3], [3, 1, 2], r_ext, 0, out, d, r) == 2


@pytest.mark.parametrize("rank0,rank1", [(2, 2), (2, 1), (4, 2), (4, 1), (6, 2)])
def test_energy_denominator(rank0, rank1):
    rng = np.random.default_rng(rank0 * 10 + rank1)
    segs = [3, 4, 2, 5]
    norb = sum(segs)
    eps = np.sort(rng.uniform(-2, 5, norb))
    fock = np.diag(eps) + 0.01 * rng.standard_normal((norb, norb))
    f1 = fock.ravel(order="F") if rank1 == 2 else eps.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    iv = [int(x) for x in rng.integers(1, len(segs) + 1, rank0)]
    ext0 = [segs[v - 1] for v in iv]
    if rank0 == 6:
        ext0[4] = 1  # a simple index: offset = value - 1
        iv[4] = 7
    data = rng.standard_normal(kat.size(ext0))
    out = data.copy()
    assert oracle.energy_denominator_rhf(iv, ext0, out, ext1, f1, segs) == 0
    e = np.diag(fock) if rank1 == 2 else eps
    offs = []
    for q in range(rank0):
        if rank0 == 6 and ext0[q] == 1:
            offs.append(iv[q] - 1)
        else:
            offs.append(sum(segs[: iv[q] - 1]))
    blk = data.reshape(ext0, order="F")
    ref = np.empty_like(blk)
    for idx in np.ndindex(*ext0):
        ev = [e[idx[q] + offs[q]] for q in range(rank0)]
        if rank0 == 2:
            den = ev[1] - ev[0]
        elif rank0 == 4:
            den = ev[1] + ev[3] - ev[0] - ev[2]
        else:
            den = ev[1] + ev[3] + ev[5] - ev[0] - ev[2] - ev[4]
        ref[idx] = blk[idx] / den
    np.testing.assert_array_equal(out, ref.ravel(order="F"))


@pytest.mark.parametrize("rank0,rank1,permuted", [(6, 2, False), (6, 2, True), (4, 1, True), (2, 2, False)])
def test_energy_contract_oracle_against_loops(rank0, rank1, permuted):
    """The oracle's (T) energy pattern (permute, divide, contract to scalar,
    scale) against a plain loop over the block."""
    rng = np.random.default_rng(100 + rank0 * 10 + rank1 + permuted)
    segs = [2, 3, 3]
    norb = sum(segs)
    e = np.concatenate([rng.uniform(-2, -0.5, 2), rng.uniform(0.2, 5, 6)])
    f1 = np.diag(e).ravel(order="F") if rank1 == 2 else e.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    # denominator order: virtual, occupied, virtual, ...
    iv_d = [[2, 3][q // 2 % 2] if q % 2 == 0 else 1 for q in range(rank0)]
    ext_d = [segs[v - 1] for v in iv_d]
    store = list(range(rank0))
    if permuted:
        store = [q for q in range(0, rank0, 2)] + [q for q in range(1, rank0, 2)]  # (v.., o..)
    ext_s = [ext_d[p] for p in store]
    iv_s = [iv_d[p] for p in store]
    den_order = [store.index(q) for q in range(rank0)]
    w = rng.standard_normal(kat.size(ext_s))
    got = oracle.energy_contract(iv_s, ext_s, w, ext1, f1, segs, 0.75, den_order=den_order)
    W = w.reshape(ext_s, order="F")
    offs = [sum(segs[: v - 1]) for v in iv_s]
    ref = 0.0
    for idx in np.ndindex(*ext_s):
        ev = {store[s]: e[idx[s] + offs[s]] for s in range(rank0)}
        occ = sum(ev[q] for q in range(1, rank0, 2))
        vir = sum(ev[q] for q in range(0, rank0, 2))
        ref += W[idx] * (W[idx] / (occ - vir))
    assert abs(got - 0.75 * ref) <= 1e-13 * abs(ref)


@pytest.mark.parametrize("diagonal", [False, True])
def test_update_t2_oracle_against_loops(diagonal):
    """The oracle's updatet2 (reference block operations) against a plain loop
    of the procedure's arithmetic, bit for bit."""
    rng = np.random.default_rng(31 + diagonal)
    segs = [4, 5, 6]
    norb = sum(segs)
    e = np.concatenate([rng.uniform(-2, -0.5, 4), rng.uniform(0.2, 5, 11)])
    fock = np.diag(e).ravel(order="F")
    iv = [2, 1, 2, 1] if diagonal else [2, 1, 3, 1]
    ext = [segs[v - 1] for v in iv]
    n = kat.size(ext)
    xn, xo = rng.standard_normal(n) * 0.1, rng.standard_normal(n) * 0.1
    xnp = xn if diagonal else rng.standard_normal(n) * 0.1
    xop = xo if diagonal else rng.standard_normal(n) * 0.1
    err, nxt, nrm = oracle.update_t2(iv, ext, xn, xnp, xo, xop, [norb, norb], fock, segs)
    offs = [sum(segs[: v - 1]) for v in iv]
    pe = [ext[2], ext[3], ext[0], ext[1]]
    Xn, Xo = xn.reshape(ext, order="F"), xo.reshape(ext, order="F")
    Pn, Po = xnp.reshape(pe, order="F"), xop.reshape(pe, order="F")
    er, nr = np.empty(ext), np.empty(ext)
    for a, i, b, j in np.ndindex(*ext):
        eps = ((e[i + offs[1]] + e[j + offs[3]]) - e[a + offs[0]]) - e[b + offs[2]]
        t = Pn[b, j, a, i] + Xn[a, i, b, j]
        t1 = Po[b, j, a, i] + Xo[a, i, b, j]
        er[a, i, b, j] = (t1 - t / eps) * -0.5
        nr[a, i, b, j] = (t * 0.5) / eps
    np.testing.assert_array_equal(err, er.ravel(order="F"))
    np.testing.assert_array_equal(nxt, nr.ravel(order="F"))
    assert abs(nrm - (er ** 2).sum()) <= 1e-13 * nrm


# ---------------------------------------------------------------- restated reference routines
def _golden(kind):
    return [c for c in kat.cases() if c["kind"] == kind]


@pytest.mark.parametrize("c", _golden("pattern"), ids=lambda c: c["name"])
def test_golden_pattern(c):
    """get_contraction_ptrn: the oracle's counting restatement against the
    fixtures transliterated from tensor_dil_omp.F90:87-142 (ierr and pattern)."""
    ierr, my = oracle.get_contraction_ptrn(c["drank"], c["lrank"], c["rrank"], c["aces"])
    assert ierr == c["ierr"]
    if ierr == 0:
        assert my[: c["lrank"] + c["rrank"]] == c["my_ptrn"]


@pytest.mark.parametrize("c", _golden("denominator"), ids=lambda c: c["name"])
def test_golden_denominator(c):
    """energy_denominator_rhf, bit for bit against the fixtures' loops."""
    x = np.array(c["data"], dtype=np.float64)
    assert oracle.energy_denominator_rhf(c["index_values"], c["ext"], x, c["ext1"], np.array(c["e"]),
                                         c["seg_sizes"]) == 0
    np.testing.assert_array_equal(x, np.array(c["expected"]))


@pytest.mark.parametrize("c", _golden("update_t2"), ids=lambda c: c["name"])
def test_golden_update_t2(c):
    """updatet2's two passes: error block and next amplitudes bit for bit; the
    squared norm (a long sum) to 1e-14 of the exact sum."""
    a = lambda k: np.array(c[k], dtype=np.float64)
    err, nxt, nrm = oracle.update_t2(c["index_values"], c["ext"], a("t2new"), a("t2new_pair"), a("t2old"),
                                     a("t2old_pair"), c["ext1"], a("fock"), c["seg_sizes"])
    np.testing.assert_array_equal(err, a("expected_err"))
    np.testing.assert_array_equal(nxt, a("expected_next"))
    assert abs(nrm - c["expected_norm2"]) <= 1e-14 * c["expected_norm2"]


@pytest.mark.parametrize("c", _golden("energy"), ids=lambda c: c["name"])
def test_golden_energy(c):
    """The (T) energy pattern: the same quotients as the fixture, summed in
    another order: 1e-14 of the fixture's exact sum."""
    got = oracle.energy_contract(c["index_values"], c["ext"], np.array(c["w"]), c["ext1"], np.array(c["fock"]),
                                 c["seg_sizes"], c["efact"], den_order=c["den_order"])
    assert abs(got - c["expected"]) <= 1e-14 * abs(c["expected"])
