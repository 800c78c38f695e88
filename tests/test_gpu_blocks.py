"""GPU parity of the block path through the C ABI against the CPU oracle and the
reference's known-answer fixtures.  Integer/permutation/element-wise results
are bit-exact; FP64 contractions (different summation order) are held to a
relative Frobenius error of 1e-12."""
import zlib

import numpy as np
import pytest

from oracle import oracle
from tests import kat

pytestmark = pytest.mark.gpu

REL_TOL_FP64 = 1e-12


@pytest.fixture(scope="module")
def lib():
    import aces4_gb300

    aces4_gb300.build()
    return aces4_gb300


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


# --------------------------------------------------------- known answers
@pytest.mark.parametrize("name", ["contraction_small_test", "contraction_small_test2", "contract_to_scalar"])
def test_kat_contract_host_dropin(lib, name):
    c = kat.case(name)
    L = kat.fill(c["l_fill"], kat.size(c["l_ext"]))
    R = kat.fill(c["r_fill"], kat.size(c["r_ext"]))
    ierr, D = lib.ref.contract_labels(c["d_labels"], c["l_labels"], c["r_labels"], L, c["l_ext"], R,
                                      c["r_ext"], c["d_ext"])
    assert ierr == 0
    np.testing.assert_array_equal(D, np.array(c["expected"]))


@pytest.mark.parametrize("name", ["transpose_tmp", "transpose4d_tmp", "transpose4d_square_tmp"])
def test_kat_permute_host_dropin(lib, name):
    c = kat.case(name)
    S = kat.fill(c["s_fill"], kat.size(c["s_ext"]))
    ierr, D = lib.ref.tensor_block_copy(c["s_ext"], kat.perm_from_labels(c["d_labels"], c["s_labels"]), S)
    assert ierr == 0
    np.testing.assert_array_equal(D, np.array(c["expected"]))
    if "esum" in c:
        sl, dl = c["s_labels"], c["d_labels"]
        e1 = lib.ref.contract_labels([], sl, sl, S, c["s_ext"], S, c["s_ext"], [])[1][0]
        e2 = lib.ref.contract_labels([], dl, dl, D, c["d_ext"], D, c["d_ext"], [])[1][0]
        e3 = lib.ref.contract_labels([], sl, dl, S, c["s_ext"], D, c["d_ext"], [])[1][0]
        assert [e1, e2, e3] == c["esum"]


def test_kat_sum_op_self_multiply_device(lib):
    import torch

    c = kat.case("sum_op")
    n = kat.size(c["ext"])
    a = torch.tensor(kat.fill(c["a_fill"], n), device="cuda")
    cc = torch.tensor(kat.fill(c["c_fill"], n), device="cuda")
    d = torch.empty_like(a)
    e = torch.empty_like(a)
    ids = [1, 2]
    lib.device.add_sub(False, ids, ids, c["ext"], d, a, cc)
    lib.device.add_sub(True, ids, ids, c["ext"], e, d, cc)
    lib.device.sync()
    np.testing.assert_array_equal(d.cpu().numpy(), c["expected_d"])
    np.testing.assert_array_equal(e.cpu().numpy(), c["expected_e"])
    s = kat.case("self_multiply_test")
    a = torch.tensor(kat.fill(s["a_fill"], n), device="cuda")
    lib.device.add_sub(False, ids, ids, s["ext"], a, a, a)  # a += a (d aliases l and r)
    lib.device.scale(a, s["factor"])
    lib.device.sync()
    np.testing.assert_array_equal(a.cpu().numpy(), s["expected"])


# --------------------------------------------------------- random parity
PATTERNS = [
    ("abij", "abcd", "cdij"), ("aibj", "akci", "cbkj"), ("abcijk", "bcdk", "adij"),
    ("il", "ijkl", "jk"), ("ba", "ac", "cb"), ("", "abc", "cab"), ("ab", "a", "b"),
    ("ab", "ab", ""), ("ba", "", "ab"), ("", "", ""), ("fedcba", "abcx", "xdef"),
    ("ij", "ki", "kj"), ("ijab", "ijcd", "abcd"),
]


def _setup(dl, ll, rl, lo=2, hi=9):
    rng = np.random.default_rng(zlib.crc32(f"{dl}|{ll}|{rl}".encode()))
    labs = sorted(set(dl + ll + rl))
    ext = {x: int(rng.integers(lo, hi)) for x in labs}
    lid = {x: i + 1 for i, x in enumerate(labs)}
    le, re, de = [ext[x] for x in ll], [ext[x] for x in rl], [ext[x] for x in dl]
    L = rng.standard_normal(kat.size(le))
    R = rng.standard_normal(kat.size(re))
    return rng, lid, le, re, de, L, R


@pytest.mark.parametrize("dl,ll,rl", PATTERNS)
def test_contract_host_dropin_vs_oracle(lib, dl, ll, rl):
    _, lid, le, re, de, L, R = _setup(dl, ll, rl)
    ids = lambda s: [lid[x] for x in s]
    ierr, D = lib.ref.contract_labels(ids(dl), ids(ll), ids(rl), L, le, R, re, de)
    assert ierr == 0
    ierr, Do = oracle.contract_labels(ids(dl), ids(ll), ids(rl), L, le, R, re, de)
    assert ierr == 0
    if not ll or not rl:  # scalar cases are element-wise: bit-exact
        np.testing.assert_array_equal(D, Do)
    else:
        assert rel_err(D, Do) <= REL_TOL_FP64


@pytest.mark.parametrize("dl,ll,rl", PATTERNS[:6])
def test_contract_device_beta_accumulate(lib, dl, ll, rl):
    import torch

    _, lid, le, re, de, L, R = _setup(dl, ll, rl, 3, 12)
    ids = lambda s: [lid[x] for x in s]
    Do = oracle.contract_labels(ids(dl), ids(ll), ids(rl), L, le, R, re, de)[1]
    d0 = np.random.default_rng(1).standard_normal(Do.size)
    tl, tr = torch.tensor(L, device="cuda"), torch.tensor(R, device="cuda")
    td = torch.tensor(d0, device="cuda")
    lib.device.contract_labels(ids(dl), ids(ll), ids(rl), tl, le, tr, re, td, de, beta=1)
    lib.device.sync()
    assert rel_err(td.cpu().numpy(), d0 + Do) <= REL_TOL_FP64


def test_contract_large_ladder_block(lib):
    # one block pair of the o=10/v=48 ladder (144 x 25 x 144) and a bigger ring pair
    for dl, ll, rl, ext in [("abij", "abcd", "cdij", dict(a=12, b=12, c=12, d=12, i=5, j=5)),
                            ("aibj", "akci", "cbkj", dict(a=24, b=31, c=40, k=20, i=20, j=20))]:
        rng = np.random.default_rng(11)
        lid = {x: i + 1 for i, x in enumerate(sorted(ext))}
        ids = lambda s: [lid[x] for x in s]
        le, re, de = [ext[x] for x in ll], [ext[x] for x in rl], [ext[x] for x in dl]
        L = rng.uniform(-1, 1, kat.size(le))
        R = rng.normal(0, 0.1, kat.size(re))
        ierr, D = lib.ref.contract_labels(ids(dl), ids(ll), ids(rl), L, le, R, re, de)
        assert ierr == 0
        ptrn = oracle.get_contraction_ptrn(len(dl), len(ll), len(rl), ids(dl + ll + rl))[1]
        assert rel_err(D, oracle.contract_blas(ptrn, L, le, R, re, de)) <= REL_TOL_FP64


def test_contract_errors_match_reference(lib):
    L = np.ones(6)
    R = np.ones(6)
    D = np.zeros(4)
    assert lib.ref.tensor_block_contract([1, -1, -2, 2], L, [2, 3], R, [4, 2], D, [2, 2]) == 1
    assert lib.ref.get_contraction_ptrn(1, 1, 2, [1, 2, 1, 3])[0] == 4


def test_permute_vs_oracle_all_ranks(lib):
    rng = np.random.default_rng(3)
    for rank in range(1, 7):
        for _ in range(4):
            ext = [int(x) for x in rng.integers(1, 12, rank)]
            perm = [int(x) + 1 for x in rng.permutation(rank)]
            S = rng.standard_normal(kat.size(ext))
            ierr, D = lib.ref.tensor_block_copy(ext, perm, S)
            assert ierr == 0
            np.testing.assert_array_equal(D, oracle.tensor_block_copy(ext, perm, S)[1])


def test_permute_device_large(lib):
    import torch

    ext = [32, 32, 16, 16]
    for perm in ([3, 4, 1, 2], [2, 1, 4, 3], [4, 3, 2, 1], [1, 2, 3, 4], [1, 3, 2, 4]):
        S = np.random.default_rng(4).standard_normal(kat.size(ext))
        src = torch.tensor(S, device="cuda")
        dst = torch.empty_like(src)
        lib.device.permute(ext, perm, src, dst)
        lib.device.sync()
        np.testing.assert_array_equal(dst.cpu().numpy(), oracle.tensor_block_copy(ext, perm, S)[1])


def test_elementwise_bit_exact(lib):
    rng = np.random.default_rng(5)
    ext = [7, 9, 11]
    n = kat.size(ext)
    t0 = rng.standard_normal(n)
    t1 = rng.standard_normal(n)
    for scale in (0.5, 1.0 + 5e-14, -3.75):
        a, b = t0.copy(), t0.copy()
        assert lib.ref.tensor_block_add(ext, a, t1, scale) == 0
        oracle.tensor_block_add(ext, b, t1, scale)
        np.testing.assert_array_equal(a, b)
    a, b = t0.copy(), t0.copy()
    lib.ref.tensor_block_scale(a, ext, -2.5)
    oracle.tensor_block_scale(b, ext, -2.5)
    np.testing.assert_array_equal(a, b)
    a = t0.copy()
    lib.ref.tensor_block_init(a, ext, 3.25)
    np.testing.assert_array_equal(a, 3.25)
    v, ierr = lib.ref.tensor_block_norm2(t0, ext)
    assert ierr == 0 and abs(v - np.sum(t0 * t0)) <= 1e-12 * np.sum(t0 * t0)


def test_device_elementwise(lib):
    import torch

    rng = np.random.default_rng(8)
    n = 100_003  # odd: exercises the vector tail
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    tx, ty = torch.tensor(x, device="cuda"), torch.tensor(y, device="cuda")
    lib.device.scale_copy(ty, tx, 3.0)
    lib.device.increment(ty, 0.125)
    lib.device.sync()
    ref = x * 3.0
    ref = ref + 0.125
    np.testing.assert_array_equal(ty.cpu().numpy(), ref)
    lib.device.fill(tx, -1.5)
    lib.device.sync()
    assert float(tx.min()) == float(tx.max()) == -1.5
    v = lib.device.norm2(torch.tensor(y, device="cuda"))
    assert abs(v - float(np.dot(y, y))) <= 1e-12 * float(np.dot(y, y))


def test_slice_insert(lib):
    rng = np.random.default_rng(6)
    text, sext, beg = [6, 5, 4], [3, 2, 2], [2, 1, 1]
    T = rng.standard_normal(120)
    ierr, S = lib.ref.tensor_block_slice(T, text, sext, beg)
    assert ierr == 0
    np.testing.assert_array_equal(S, oracle.tensor_block_slice(T, text, sext, beg)[1])
    T2, T3 = np.zeros(120), np.zeros(120)
    assert lib.ref.tensor_block_insert(T2, text, S, sext, beg) == 0
    oracle.tensor_block_insert(T3, text, S, sext, beg)
    np.testing.assert_array_equal(T2, T3)


@pytest.mark.parametrize("rank0,rank1", [(2, 2), (2, 1), (4, 2), (4, 1), (6, 2)])
def test_energy_denominator_bit_exact(lib, rank0, rank1):
    rng = np.random.default_rng(rank0 * 10 + rank1)
    segs = [3, 4, 2, 5]
    norb = sum(segs)
    eps = np.sort(rng.uniform(-2, 5, norb))
    fock = np.diag(eps) + 0.01 * rng.standard_normal((norb, norb))
    f1 = fock.ravel(order="F").copy() if rank1 == 2 else eps.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    iv = [int(x) for x in rng.integers(1, len(segs) + 1, rank0)]
    ext0 = [segs[v - 1] for v in iv]
    if rank0 == 6:
        ext0[4], iv[4] = 1, 7
    data = rng.standard_normal(kat.size(ext0))
    a, b = data.copy(), data.copy()
    assert lib.ref.set_predefined_int_array("moa_seg_ranges", segs) == 0
    assert lib.ref.energy_denominator_rhf(iv, ext0, a, ext1, f1) == 0
    assert oracle.energy_denominator_rhf(iv, ext0, b, ext1, f1, segs) == 0
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("rank0,rank1,ext0", [(4, 2, [40, 30, 37, 11]), (4, 1, [17, 33, 5, 3]),
                                               (6, 2, [24, 7, 23, 6, 13, 5])])
def test_energy_denominator_large_bit_exact(lib, rank0, rank1, ext0):
    """Blocks that spread over several CTAs, with x2 (and x4) ranges that are
    not multiples of the loads in flight, zeros among the data (0 / eps keeps
    the IEEE sign): bit for bit against the oracle."""
    rng = np.random.default_rng(sum(ext0))
    segs = [40, 30, 37, 11, 17, 33, 5, 3, 24, 7, 23, 6, 13]
    norb = sum(segs)
    eps = np.concatenate([rng.uniform(-2, -0.3, norb // 3), rng.uniform(0.2, 5, norb - norb // 3)])
    fock = np.diag(eps) + 0.01 * rng.standard_normal((norb, norb))
    f1 = fock.ravel(order="F").copy() if rank1 == 2 else eps.copy()
    ext1 = [norb, norb] if rank1 == 2 else [norb]
    iv = [segs.index(x) + 1 for x in ext0]
    data = rng.standard_normal(kat.size(ext0))
    data[::17] = 0.0
    a, b = data.copy(), data.copy()
    assert lib.ref.set_predefined_int_array("moa_seg_ranges", segs) == 0
    assert lib.ref.energy_denominator_rhf(iv, ext0, a, ext1, f1) == 0
    assert oracle.energy_denominator_rhf(iv, ext0, b, ext1, f1, segs) == 0
    assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_legacy_gpu_api(lib):
    import ctypes

    import torch

    L = lib.lib()
    L.a4g_clear_error()  # errors recorded by earlier tests' rejected calls
    rng = np.random.default_rng(9)
    # y(a,i,b,j) = x1(a,k,c,i) * x2(c,b,k,j) with labels
    ext = dict(a=6, i=4, b=5, j=3, k=7, c=8)
    lid = {x: i + 1 for i, x in enumerate("aibjkc")}
    y_l, x1_l, x2_l = "aibj", "akci", "cbkj"
    e = lambda s: [ext[x] for x in s]
    x1 = rng.standard_normal(kat.size(e(x1_l)))
    x2 = rng.standard_normal(kat.size(e(x2_l)))
    tx1, tx2 = torch.tensor(x1, device="cuda"), torch.tensor(x2, device="cuda")
    ty = torch.full((kat.size(e(y_l)),), np.nan, dtype=torch.float64, device="cuda")
    ids = lambda s: [lid[x] for x in s]
    lib.device.gpu_contract(ty, e(y_l), ids(y_l), tx1, e(x1_l), ids(x1_l), tx2, e(x2_l), ids(x2_l))
    ref = oracle.contract_labels(ids(y_l), ids(x1_l), ids(x2_l), x1, e(x1_l), x2, e(x2_l), e(y_l))[1]
    assert rel_err(ty.cpu().numpy(), ref) <= REL_TOL_FP64
    # _gpu_permute: y(c,a,k,i) = x1(a,k,c,i)
    tp = torch.empty_like(tx1)
    lib.device.gpu_permute(tp, e("caki"), ids("caki"), tx1, e(x1_l), ids(x1_l))
    perm = kat.perm_from_labels(ids("caki"), ids(x1_l))
    np.testing.assert_array_equal(tp.cpu().numpy(), oracle.tensor_block_copy(e(x1_l), perm, x1)[1])
    # alloc / copies / axpy / memset / selfmultiply
    n = 1000
    g = L._gpu_allocate(n)
    h = rng.standard_normal(n)
    L._gpu_host_to_device(h.ctypes.data, g, n)
    L._gpu_selfmultiply(g, 2.0, n)
    g2 = L._gpu_allocate(n)
    L._gpu_double_memset(g2, 1.0, n)
    L._gpu_axpy(g2, g, 0.5, n)
    out = np.empty(n)
    L._gpu_device_to_host(out.ctypes.data, g2, n)
    np.testing.assert_allclose(out, 1.0 + 0.5 * (2.0 * h), rtol=0, atol=1e-15)
    L._gpu_device_to_device(g, g2, n)
    L._gpu_device_to_host(out.ctypes.data, g, n)
    np.testing.assert_allclose(out, 1.0 + 0.5 * (2.0 * h), rtol=0, atol=1e-15)
    L._gpu_free(g)
    L._gpu_free(g2)
    assert ctypes.c_char_p(L.a4g_last_error()).value in (b"", None)


# ---------------------------------------------------------------- restated reference routines on the GPU
def _golden(kind):
    return [c for c in kat.cases() if c["kind"] == kind]


@pytest.mark.parametrize("c", _golden("denominator"), ids=lambda c: c["name"])
def test_golden_denominator_gpu(lib, c):
    """The fp2 drop-in and the device entry against the fixtures restated
    from energy_denominator_rhf.F, bit for bit (rank 6 with 1-D energies:
    left untouched, as the reference leaves it)."""
    import torch

    x = np.array(c["data"], dtype=np.float64)
    e = np.array(c["e"], dtype=np.float64)
    assert lib.ref.set_predefined_int_array("moa_seg_ranges", c["seg_sizes"]) == 0
    assert lib.ref.energy_denominator_rhf(c["index_values"], c["ext"], x, c["ext1"], e) == 0
    np.testing.assert_array_equal(x, np.array(c["expected"]))
    if c["rank0"] == 6 and c["rank1"] != 2:
        return  # the device entry rejects the combination the reference ignores
    t = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    lib.device.energy_denominator(c["index_values"], c["ext"], t, c["ext1"], torch.tensor(e, device="cuda"),
                                  c["seg_sizes"])
    np.testing.assert_array_equal(t.cpu().numpy(), np.array(c["expected"]))


@pytest.mark.parametrize("c", _golden("update_t2"), ids=lambda c: c["name"])
def test_golden_update_t2_gpu(lib, c):
    import torch

    d = lambda k: torch.tensor(c[k], dtype=torch.float64, device="cuda")
    err, nxt = torch.empty_like(d("t2new")), torch.empty_like(d("t2new"))
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib.device.update_t2(c["index_values"], c["ext"], d("t2new"), d("t2new_pair"), d("t2old"), d("t2old_pair"),
                         err, nxt, c["ext1"], d("fock"), c["seg_sizes"], nrm)
    lib.device.sync()
    np.testing.assert_array_equal(err.cpu().numpy(), np.array(c["expected_err"]))
    np.testing.assert_array_equal(nxt.cpu().numpy(), np.array(c["expected_next"]))
    assert abs(float(nrm.item()) - c["expected_norm2"]) <= 1e-14 * c["expected_norm2"]


@pytest.mark.parametrize("c", _golden("energy"), ids=lambda c: c["name"])
def test_golden_energy_gpu(lib, c):
    import torch

    esum = torch.zeros(1, dtype=torch.float64, device="cuda")
    f64 = dict(dtype=torch.float64, device="cuda")
    lib.device.energy_contract(c["index_values"], c["ext"], torch.tensor(c["w"], **f64), c["ext1"],
                               torch.tensor(c["fock"], **f64), c["seg_sizes"], c["efact"], esum,
                               den_order=c["den_order"])
    lib.device.sync()
    assert abs(float(esum.item()) - c["expected"]) <= 1e-14 * abs(c["expected"])


@pytest.mark.parametrize("c", [c for c in _golden("pattern") if min(c["drank"], c["lrank"], c["rrank"]) >= 0],
                         ids=lambda c: c["name"])
def test_golden_pattern_dropin(lib, c):
    ierr, my = lib.ref.get_contraction_ptrn(c["drank"], c["lrank"], c["rrank"], c["aces"])
    assert ierr == c["ierr"]
    if ierr == 0:
        assert list(my)[: c["lrank"] + c["rrank"]] == c["my_ptrn"]
