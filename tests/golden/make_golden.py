"""Generate the known-answer fixtures of the reference's own block-op tests.

Each case restates, with plain Python loops over named indices, a known-answer
test of the reference (shapes, fill super instruction, index labels and the
expected-value loop).  Nothing here uses the oracle or the library, so the
fixtures pin both independently.  Blocks are column-major (first index
fastest); the fills reproduce fill_block_cyclic / fill_block_sequential
(src/sip/super_instructions/qm/tests/fill_block_cyclic.f:45-60,
fill_block_sequential.f:45-60), which walk the block in memory order.

Cases (reference file:line of the test it restates):
  contraction_small_test   test/test_basic_sial.cpp:695-770,
                           src/sialx/test/contraction_small_test.sialx
  contraction_small_test2  test/test_basic_sial.cpp:773-815, test/test_contraction_small2.F
  transpose_tmp            test/test_basic_sial.cpp:653-693, test/test_transpose_op.F
  transpose4d_tmp          test/test_basic_sial.cpp:1285-1327, test/test_transpose4d_op.F
  transpose4d_square_tmp   test/test_basic_sial.cpp:1329-1405
  sum_op                   test/test_basic_sial.cpp:817-916
  contract_to_scalar       test/test_basic_sial.cpp:1037-1084
  self_multiply_test       test/test_basic_sial.cpp:1111-1156

Run:  python tests/golden/make_golden.py   (writes kat_reference_tests.json)
"""
import itertools
import json
import os


def cyclic(n, start):
    out, v = [], float(start)
    for _ in range(n):
        out.append(v)
        if v == 20.0:
            v = 0.0
        v += 1.0
    return out


def sequential(n, start):
    return [float(start) + i for i in range(n)]


def lin(idx, ext):
    """column-major linear position of a multi-index"""
    p, s = 0, 1
    for i, e in zip(idx, ext):
        p += i * s
        s *= e
    return p


def size(ext):
    n = 1
    for e in ext:
        n *= e
    return n


def contraction(dl, ll, rl, de, le, re, L, R):
    """D(dl) = sum over labels shared by L and R of L(ll)*R(rl) (reference loop)."""
    ext = {}
    for labs, exts in ((dl, de), (ll, le), (rl, re)):
        for a, e in zip(labs, exts):
            ext[a] = e
    con = [a for a in ll if a in rl]
    D = [0.0] * max(1, size(de))
    for didx in itertools.product(*[range(ext[a]) for a in dl]):
        env = dict(zip(dl, didx))
        acc = 0.0
        for cidx in itertools.product(*[range(ext[a]) for a in con]):
            env.update(zip(con, cidx))
            acc += L[lin([env[a] for a in ll], le)] * R[lin([env[a] for a in rl], re)]
        D[lin(didx, de) if dl else 0] = acc
    return D


def permute(dl, sl, se, S):
    """D(dl) = S(sl): a pure relabelling (transpose) of block S."""
    ext = dict(zip(sl, se))
    de = [ext[a] for a in dl]
    D = [0.0] * size(de)
    for sidx in itertools.product(*[range(e) for e in se]):
        env = dict(zip(sl, sidx))
        D[lin([env[a] for a in dl], de)] = S[lin(sidx, se)]
    return D, de


def main():
    cases = []

    # c[i,l] = a[i,j,k,l] * b[j,k], extents 15, cyclic fills from 1.0
    e = 15
    a = cyclic(e ** 4, 1.0)
    b = cyclic(e ** 2, 1.0)
    c = contraction("il", "ijkl", "jk", [e, e], [e] * 4, [e, e], a, b)
    cases.append(dict(name="contraction_small_test", kind="contract", d_labels=[1, 4],
                      l_labels=[1, 2, 3, 4], r_labels=[2, 3], d_ext=[e, e], l_ext=[e] * 4,
                      r_ext=[e, e], l_fill=["cyclic", 1.0], r_fill=["cyclic", 1.0], expected=c))

    # c[mu,i1,a1,i] = b[lambda,a1] * a[mu,i1,i,lambda]; mu,lambda=9; i,i1=5; a1=4
    mu, la, i_, a1 = 9, 9, 5, 4
    bl = cyclic(la * a1, 1.0)
    ar = cyclic(mu * i_ * i_ * la, 1.0)
    # labels: mu=1 i1=2 a1=3 i=4 lambda=5
    c2 = contraction("MJAIL"[0:4], "LA", "MJIL", [mu, i_, a1, i_], [la, a1], [mu, i_, i_, la], bl, ar)
    cases.append(dict(name="contraction_small_test2", kind="contract", d_labels=[1, 2, 3, 4],
                      l_labels=[5, 3], r_labels=[1, 2, 4, 5], d_ext=[mu, i_, a1, i_],
                      l_ext=[la, a1], r_ext=[mu, i_, i_, la], l_fill=["cyclic", 1.0],
                      r_fill=["cyclic", 1.0], expected=c2))

    # b[j,k,i] = a[i,j,k], 8^3, sequential from 53
    a3 = sequential(512, 53.0)
    b3, be3 = permute("jki", "ijk", [8, 8, 8], a3)
    cases.append(dict(name="transpose_tmp", kind="permute", d_labels=[2, 3, 1], s_labels=[1, 2, 3],
                      s_ext=[8, 8, 8], s_fill=["sequential", 53.0], d_ext=be3, expected=b3))

    # b[k,j,i,l] = a[i,j,k,l] with i,k virtual (5) and j,l occupied (1), from 53
    a4 = sequential(25, 53.0)
    b4, be4 = permute("kjil", "ijkl", [5, 1, 5, 1], a4)
    cases.append(dict(name="transpose4d_tmp", kind="permute", d_labels=[3, 2, 1, 4],
                      s_labels=[1, 2, 3, 4], s_ext=[5, 1, 5, 1], s_fill=["sequential", 53.0],
                      d_ext=be4, expected=b4))

    # 8^4 cyclic from 1: b[k,j,i,l] = a[i,j,k,l]; esum1 = a.a, esum2 = b.b, esum3 = a.b
    a5 = cyclic(8 ** 4, 1.0)
    b5, be5 = permute("kjil", "ijkl", [8] * 4, a5)
    es1 = contraction("", "ijkl", "ijkl", [], [8] * 4, [8] * 4, a5, a5)[0]
    es2 = contraction("", "kjil", "kjil", [], be5, be5, b5, b5)[0]
    es3 = contraction("", "ijkl", "kjil", [], [8] * 4, be5, a5, b5)[0]
    cases.append(dict(name="transpose4d_square_tmp", kind="permute_esum", d_labels=[3, 2, 1, 4],
                      s_labels=[1, 2, 3, 4], s_ext=[8] * 4, s_fill=["cyclic", 1.0], d_ext=be5,
                      expected=b5, esum=[es1, es2, es3]))

    # d = a + c; e = d - c   (20x20; a seq from 100, c seq from 50)
    n = 400
    a6 = sequential(n, 100.0)
    c6 = sequential(n, 50.0)
    d6 = [x + y for x, y in zip(a6, c6)]
    e6 = [x - y for x, y in zip(d6, c6)]
    cases.append(dict(name="sum_op", kind="add_sub", ext=[20, 20], a_fill=["sequential", 100.0],
                      c_fill=["sequential", 50.0], expected_d=d6, expected_e=e6))

    # x = a[i,j] * b[i,j]   (8x8; a cyclic from 1, b cyclic from 5)
    a7 = cyclic(64, 1.0)
    b7 = cyclic(64, 5.0)
    x7 = contraction("", "ij", "ij", [], [8, 8], [8, 8], a7, b7)[0]
    cases.append(dict(name="contract_to_scalar", kind="contract", d_labels=[], l_labels=[1, 2],
                      r_labels=[1, 2], d_ext=[], l_ext=[8, 8], r_ext=[8, 8],
                      l_fill=["cyclic", 1.0], r_fill=["cyclic", 5.0], expected=[x7]))

    # a = seq from 100; a += a; a *= 1.5
    a8 = sequential(n, 100.0)
    exp8 = [(x + x) * 1.5 for x in a8]
    cases.append(dict(name="self_multiply_test", kind="self_add_scale", ext=[20, 20],
                      a_fill=["sequential", 100.0], factor=1.5, expected=exp8))

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_reference_tests.json")
    with open(out, "w") as f:
        json.dump({"source": "restated known-answer tests of the reference (see make_golden.py)",
                   "cases": cases}, f, separators=(",", ":"))
    print("wrote", out, len(cases), "cases")


if __name__ == "__main__":
    main()
