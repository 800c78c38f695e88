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

Further cases restate, as plain loops, reference routines whose own tests
need inputs this project cannot run (the SIAL compiler, integrals):
  pattern            get_contraction_ptrn, src/sip/tensor_algebra/tensor_dil_omp.F90:87-142
                     (transliterated: stable sort of the labels, pair check, pattern build),
                     every ierr case and valid patterns of ranks 0..4
  denominator        energy_denominator_rhf, src/sip/super_instructions/qm/qm-generic/
                     energy_denominator_rhf.F:15-447 (offsets from moa_seg_ranges, rank 6
                     simple indices, do_rhf_den2/_1d :241-308, do_rhf_den4/_1d :310-395,
                     do_rhf_den6 :399-436, rank 6 with 1-D energies left untouched), on
                     integer-friendly energies (multiples of 1/8, data = eps x small
                     integers: every quotient exact) and on random data (the order of the
                     additions decides the bits)
  update_t2          procedure updatet2, src/sialx/qm/cc/rlccd_rhf.sialx:557-600 (both
                     pardo passes on one (a,i,b,j) block and its (b,j,a,i) partner)
  energy             the (T) energy pattern, src/sialx/qm/cc/rccsdpt_aaa.sialx:2163-2172
                     (permute to the denominator's order, divide, contract the divided
                     block with the undivided one, times efact); the expected value is
                     the exact sum (math.fsum) of the rounded products

Run:  python tests/golden/make_golden.py   (writes kat_reference_tests.json)
"""
import itertools
import json
import math
import os
import random


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


def get_contraction_ptrn_f90(drank, lrank, rrank, aces):
    """tensor_dil_omp.F90:87-142 line by line: (ierr, my_ptrn)."""
    if not (drank >= 0 and lrank >= 0 and rrank >= 0):
        return 1, []
    m = lrank + rrank
    n = drank + m
    if n % 2 != 0:
        return 2, []
    if m <= 0:
        return (3 if drank > 0 else 0), []
    trn = sorted(range(1, n + 1), key=lambda i: aces[i - 1])  # merge sort: stable
    for i in range(1, n, 2):  # i = 1, 3, ..., n-1 (1-based pairs (i, i+1))
        if aces[trn[i - 1] - 1] == aces[trn[i] - 1]:
            if i > 1 and aces[trn[i - 1] - 1] == aces[trn[i - 2] - 1]:
                return 5, []
        else:
            return 4, []
    my = [0] * m
    for i in range(1, n, 2):
        j, k = trn[i - 1], trn[i]
        if j <= drank and k > drank:
            my[k - drank - 1] = j
        elif drank < j <= drank + lrank and k > drank + lrank:
            my[j - drank - 1] = -(k - (drank + lrank))
            my[k - drank - 1] = -(j - drank)
        else:
            return 6, []
    return 0, my


def pattern_cases():
    pats = [
        (-1, 2, 2, [1, 2, 1, 2]),  # negative rank: ierr 1
        (1, 1, 1, [1, 1, 2]),  # odd total: ierr 2
        (2, 0, 0, [1, 2]),  # operands of rank 0 with a tensor destination: ierr 3
        (0, 0, 0, []),  # scalar * scalar
        (2, 2, 2, [1, 2, 1, 3, 3, 4]),  # a label used once: ierr 4
        (2, 2, 2, [1, 1, 1, 1, 2, 2]),  # a label used four times: ierr 5
        (2, 2, 2, [1, 1, 2, 3, 2, 3]),  # both occurrences in D: ierr 6
        (2, 2, 2, [1, 2, 3, 3, 1, 2]),  # a contraction inside L: ierr 6
        (2, 2, 2, [1, 2, 1, 3, 3, 2]),  # matrix product D(i,j) = L(i,k) R(k,j)
        (4, 4, 4, [1, 2, 3, 4, 1, 2, 5, 6, 5, 6, 3, 4]),  # the ladder
        (4, 4, 4, [1, 3, 2, 4, 1, 7, 5, 3, 5, 2, 7, 4]),  # the ring, both operands permuted
        (0, 2, 2, [1, 2, 1, 2]),  # full contraction to a scalar
        (0, 2, 2, [1, 2, 2, 1]),
        (2, 2, 0, [1, 2, 2, 1]),  # tensor * scalar
        (2, 0, 2, [3, 4, 4, 3]),
        (2, 4, 2, [1, 4, 1, 2, 3, 4, 2, 3]),  # contraction_small_test
        (4, 2, 4, [1, 2, 3, 4, 5, 3, 1, 2, 4, 5]),  # contraction_small_test2
        (6, 4, 4, [1, 2, 3, 4, 5, 6, 3, 5, 7, 6, 1, 7, 2, 4]),  # triples term 1
        (6, 4, 4, [1, 2, 3, 4, 5, 6, 8, 5, 4, 6, 1, 3, 2, 8]),  # triples term 2
        (3, 3, 2, [9, 8, 7, 8, 6, 9, 6, 7]),
        (1, 2, 3, [5, 5, 2, 2, 1, 1]),
    ]
    rng = random.Random(87)
    for _ in range(40):  # random label lists of ranks 0..4
        dr, lr, rr = rng.randint(0, 4), rng.randint(0, 4), rng.randint(0, 4)
        pats.append((dr, lr, rr, [rng.randint(1, 5) for _ in range(dr + lr + rr)]))
    out = []
    for dr, lr, rr, aces in pats:
        ierr, my = get_contraction_ptrn_f90(dr, lr, rr, aces)
        out.append(dict(name=f"pattern {dr},{lr},{rr} {aces}", kind="pattern", drank=dr, lrank=lr, rrank=rr,
                        aces=aces, ierr=ierr, my_ptrn=my))
    return out


def den_offsets(rank0, iv, ext, segs):
    """energy_denominator_rhf.F:57-88 (ranks 2, 4) and :139-208 (rank 6: an
    extent of 1 is a simple index, offset = value - 1)."""
    off = []
    for q in range(rank0):
        if rank0 == 6 and ext[q] == 1:
            off.append(iv[q] - 1)
        else:
            o = 0
            for i in range(1, iv[q]):
                o += segs[i - 1]
            off.append(o)
    return off


def den_loops(rank0, ext, off, data, rank1, ld, e1, store_eps=False):
    """do_rhf_den2(_1d) / do_rhf_den4(_1d) / do_rhf_den6: the array divided in
    place, eps evaluated as written (left to right); store_eps: eps itself."""
    x = list(data)

    def fk(o):  # fock(o, o) of the 2-D block (leading dimension ld), or the 1-D energy
        return e1[(o - 1) + (o - 1) * ld] if rank1 == 2 else e1[o - 1]

    if rank0 == 6 and rank1 != 2:
        return x  # the reference calls nothing for rank 6 with 1-D energies
    E = list(ext) + [1] * (6 - rank0)
    for f in range(1, E[5] + 1):
        for ee in range(1, E[4] + 1):
            for d in range(1, E[3] + 1):
                for c in range(1, E[2] + 1):
                    for b in range(1, E[1] + 1):
                        for a in range(1, E[0] + 1):
                            epsa = fk(a + off[0])
                            epsb = fk(b + off[1])
                            if rank0 == 2:
                                eps = epsb - epsa
                            elif rank0 == 4:
                                epsc, epsd = fk(c + off[2]), fk(d + off[3])
                                eps = epsb + epsd - epsa - epsc
                            else:
                                epsc, epsd = fk(c + off[2]), fk(d + off[3])
                                epse, epsf = fk(ee + off[4]), fk(f + off[5])
                                eps = epsb + epsd + epsf - epsa - epsc - epse
                            p = lin([a - 1, b - 1, c - 1, d - 1, ee - 1, f - 1], E)
                            x[p] = eps if store_eps else x[p] / eps
    return x


def _energies(rng, n_occ, n_vir, exact):
    if exact:  # multiples of 1/8: every sum and difference of six is exact
        occ = [-rng.randint(4, 16) / 8.0 for _ in range(n_occ)]
        vir = [rng.randint(2, 40) / 8.0 for _ in range(n_vir)]
    else:
        occ = [rng.uniform(-2.0, -0.5) for _ in range(n_occ)]
        vir = [rng.uniform(0.2, 5.0) for _ in range(n_vir)]
    return occ + vir


def denominator_cases():
    rng = random.Random(241)
    segs = [2, 3, 3, 2]  # moa_seg_ranges: occupied segments 1-2, virtual 3-4
    norb = sum(segs)
    out = []
    specs = [  # (rank0, rank1, index values (virtual, occupied, ...), simple-index dims, exact)
        (2, 2, [3, 1], [], True), (2, 1, [4, 2], [], False),
        (4, 2, [3, 1, 4, 2], [], True), (4, 1, [4, 1, 3, 2], [], False), (4, 2, [3, 2, 3, 2], [], False),
        (6, 2, [3, 1, 4, 2, 3, 1], [], True), (6, 2, [4, 2, 3, 1, 4, 2], [], False),
        (6, 2, [3, 1, 7, 2, 4, 5], [2, 5], False),  # two simple indices (extent 1, offset = value - 1)
        (6, 1, [3, 1, 4, 2, 3, 1], [], False),  # 1-D energies at rank 6: left untouched
    ]
    for rank0, rank1, iv, simple, exact in specs:
        e = _energies(rng, 5, 5, exact)
        ext = [1 if q in simple else segs[iv[q] - 1] for q in range(rank0)]
        off = den_offsets(rank0, iv, ext, segs)
        n = size(ext)
        e1 = [0.0] * (norb * norb) if rank1 == 2 else list(e)
        if rank1 == 2:
            for o in range(norb):
                e1[o + o * norb] = e[o]
                for o2 in range(norb):  # off-diagonal Fock elements: never read
                    if o2 != o:
                        e1[o + o2 * norb] = 0.001 * (o + 2 * o2)
        if exact and not (rank0 == 6 and rank1 != 2):  # data = k * eps: every quotient is the integer k
            eps = den_loops(rank0, ext, off, [0.0] * n, rank1, norb, e1, store_eps=True)
            data = [float(rng.randint(-9, 9)) * x for x in eps]  # k * eps: exact (eps has few bits)
        else:
            data = [rng.gauss(0.0, 1.0) for _ in range(n)]
        expected = den_loops(rank0, ext, off, data, rank1, norb, e1)
        out.append(dict(name=f"denominator rank{rank0} {'fock' if rank1 == 2 else '1-D'} iv={iv}"
                             f"{' exact' if exact else ''}", kind="denominator", rank0=rank0, index_values=iv,
                        ext=ext, seg_sizes=segs, rank1=rank1, ext1=[norb, norb] if rank1 == 2 else [norb],
                        e=e1, data=data, expected=expected))
    return out


def update_t2_cases():
    """updatet2 (rlccd_rhf.sialx:557-600) on block (a,i,b,j) with its partner
    (b,j,a,i): pass 1 Taibj = T2new(b,j,a,i); Taibj += T2new(a,i,b,j);
    T1 = T2old(b,j,a,i); T1 += T2old(a,i,b,j); Taibj /= eps; T1 -= Taibj;
    T1 *= -0.5 (the DIIS error block); pass 2 Taibj = T2new(b,j,a,i);
    Taibj += T2new(a,i,b,j); Taibj *= 0.5; Taibj /= eps (the next T2old)."""
    rng = random.Random(557)
    segs = [2, 3, 3, 2]
    norb = sum(segs)
    out = []
    for iv, exact in (([3, 1, 4, 2], False), ([3, 2, 3, 2], False), ([4, 1, 3, 1], True)):
        e = _energies(rng, 5, 5, exact)
        fock = [0.0] * (norb * norb)
        for o in range(norb):
            fock[o + o * norb] = e[o]
        ext = [segs[v - 1] for v in iv]
        pe = [ext[2], ext[3], ext[0], ext[1]]
        n = size(ext)
        off = den_offsets(4, iv, ext, segs)
        diagonal = iv[0] == iv[2] and iv[1] == iv[3]

        def draw():
            return [float(rng.randint(-20, 20)) / 4.0 if exact else rng.gauss(0.0, 0.1) for _ in range(n)]

        t2new, t2old = draw(), draw()
        t2new_p, t2old_p = (list(t2new), list(t2old)) if diagonal else (draw(), draw())

        def partner(x):  # Taibj[a,i,b,j] = X(b,j,a,i), X stored with extents pe
            y = [0.0] * n
            for a, i, b, j in itertools.product(*[range(v) for v in ext]):
                y[lin([a, i, b, j], ext)] = x[lin([b, j, a, i], pe)]
            return y

        taibj = [p + s for p, s in zip(partner(t2new_p), t2new)]
        t1 = [p + s for p, s in zip(partner(t2old_p), t2old)]
        taibj = den_loops(4, ext, off, taibj, 2, norb, fock)
        err = [(x - y) * -0.5 for x, y in zip(t1, taibj)]
        t2 = [(p + s) * 0.5 for p, s in zip(partner(t2new_p), t2new)]
        nxt = den_loops(4, ext, off, t2, 2, norb, fock)
        out.append(dict(name=f"update_t2 iv={iv}{' quarter-integer data' if exact else ''}", kind="update_t2", index_values=iv,
                        ext=ext, seg_sizes=segs, ext1=[norb, norb], fock=fock, t2new=t2new, t2new_pair=t2new_p,
                        t2old=t2old, t2old_pair=t2old_p, expected_err=err, expected_next=nxt,
                        expected_norm2=math.fsum(x * x for x in err)))
    return out


def energy_cases():
    """(T) energy of one block (rccsdpt_aaa.sialx:2163-2172): W stored as
    xaaaiii[a,a1,a2,k1,ii,jj]; taiaiai[a,ii,a1,jj,a2,k1] = W (permute);
    energy_denominator_rhf taiaiai; etemp = sum(taiaiai * W permuted alike);
    esum += efact * etemp."""
    rng = random.Random(2163)
    segs = [2, 2, 3]  # one occupied... two occupied segments of 2, one virtual of 3
    norb = sum(segs)
    out = []
    e = _energies(rng, 4, 3, False)
    fock = [0.0] * (norb * norb)
    for o in range(norb):
        fock[o + o * norb] = e[o]
    # storage (a, a1, a2, k1, ii, jj): virtual x3 then occupied x3
    iv_s = [3, 3, 3, 1, 2, 1]
    ext_s = [segs[v - 1] for v in iv_s]
    den_order = [0, 4, 1, 5, 2, 3]  # storage dimension at denominator position q: a, ii, a1, jj, a2, k1
    ext_d = [ext_s[d] for d in den_order]
    iv_d = [iv_s[d] for d in den_order]
    n = size(ext_s)
    w = [rng.gauss(0.0, 1.0) for _ in range(n)]
    wp = [0.0] * n  # W in the denominator's order
    for idx in itertools.product(*[range(v) for v in ext_s]):
        wp[lin([idx[d] for d in den_order], ext_d)] = w[lin(list(idx), ext_s)]
    off = den_offsets(6, iv_d, ext_d, segs)
    q = den_loops(6, ext_d, off, wp, 2, norb, fock)
    efact = 0.75
    expected = efact * math.fsum(x * y for x, y in zip(q, wp))
    out.append(dict(name="energy (T) pattern, permuted storage", kind="energy", index_values=iv_s, ext=ext_s,
                    den_order=den_order, seg_sizes=segs, ext1=[norb, norb], fock=fock, w=w, efact=efact,
                    expected=expected))
    # the same block stored in the denominator's order
    out.append(dict(name="energy (T) pattern, denominator order", kind="energy", index_values=iv_d, ext=ext_d,
                    den_order=None, seg_sizes=segs, ext1=[norb, norb], fock=fock, w=wp, efact=efact,
                    expected=expected))
    return out


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

    cases += pattern_cases()
    cases += denominator_cases()
    cases += update_t2_cases()
    cases += energy_cases()

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_reference_tests.json")
    with open(out, "w") as f:
        json.dump({"source": "restated known-answer tests of the reference (see make_golden.py)",
                   "cases": cases}, f, separators=(",", ":"))
    print("wrote", out, len(cases), "cases")


if __name__ == "__main__":
    main()
