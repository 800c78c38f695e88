"""Segmented block arrays for driving a pardo step (host-side helper).

A SIAL array is a set of dense column-major blocks, one per tuple of segment
numbers, whose extents are the segment sizes (the reference's BlockManager /
SipTables role, src/sip/dynamic_data/block_manager.cpp,
src/sip/static_data/sip_tables.cpp:296).  ``BlockArray`` keeps every block of
an array in one device allocation (contiguous, 256-byte aligned blocks) and
hands out per-block views; a block may be marked zero (absent), which is how
`where`-clause sparsity reaches the batched contraction.
"""
from __future__ import annotations

import itertools

import numpy as np


def _align(n: int, a: int) -> int:
    return (n + a - 1) // a * a


class BlockArray:
    """All blocks of one array, by segment tuple, in one CUDA buffer."""

    def __init__(self, segs_per_index, present=None, device="cuda", dtype=None):
        import torch

        self.segs = [list(s) for s in segs_per_index]
        self.rank = len(self.segs)
        keys = list(itertools.product(*[range(len(s)) for s in self.segs]))
        self.present = {k: (present(k) if present else True) for k in keys}
        self.offsets, off = {}, 0
        for k in keys:
            if self.present[k]:
                self.offsets[k] = off
                off = _align(off + self.size(k), 32)  # 256-byte aligned blocks
        self.total = max(off, 1)
        self.buf = torch.zeros(self.total, dtype=dtype or torch.float64, device=device)

    def ext(self, key):
        return [self.segs[q][key[q]] for q in range(self.rank)]

    def size(self, key) -> int:
        return int(np.prod(self.ext(key)))

    def keys(self):
        return [k for k, p in self.present.items() if p]

    def block(self, key):
        """Flat device view of block `key`, or None for a zero block."""
        if not self.present.get(key, False):
            return None
        o = self.offsets[key]
        return self.buf[o:o + self.size(key)]

    def fill_from(self, fn):
        """fn(key, ext) -> flat float64 numpy array; copied to the device."""
        import torch

        for k in self.keys():
            self.block(k).copy_(torch.from_numpy(np.ascontiguousarray(fn(k, self.ext(k)))))


def ladder_triples(R: BlockArray, V: BlockArray, T: BlockArray):
    """R(a,b,i,j) += V(a,b,c,d) T(c,d,i,j) over every segment tuple: the
    particle-particle ladder statement of rlccd_rhf.sialx:399-433 as block
    triples (zero V or T blocks give a NULL operand, skipped by the batch)."""
    na, nb, nc, nd = (len(V.segs[q]) for q in range(4))
    ni, nj = len(T.segs[2]), len(T.segs[3])
    out = []
    for a, b, i, j in itertools.product(range(na), range(nb), range(ni), range(nj)):
        for c, d in itertools.product(range(nc), range(nd)):
            rk, vk, tk = (a, b, i, j), (a, b, c, d), (c, d, i, j)
            out.append((R.block(rk), V.block(vk), T.block(tk), R.ext(rk), V.ext(vk), T.ext(tk)))
    return out


# labels: a=1 b=2 i=3 j=4 c=5 d=6 (k=7 for the ring)
LADDER_LABELS = ([1, 2, 3, 4], [1, 2, 5, 6], [5, 6, 3, 4])
# R(a,i,b,j) = V(a,k,c,i) T(c,b,k,j)
RING_LABELS = ([1, 3, 2, 4], [1, 7, 5, 3], [5, 2, 7, 4])


def ring_triples(R: BlockArray, V: BlockArray, T: BlockArray):
    """R(a,i,b,j) += V(a,k,c,i) T(c,b,k,j): ring term with both operands
    permuted relative to the matrix form."""
    na, nk, nc, ni = (len(V.segs[q]) for q in range(4))
    nb, nj = len(T.segs[1]), len(T.segs[3])
    out = []
    for a, i, b, j in itertools.product(range(na), range(ni), range(nb), range(nj)):
        for k, c in itertools.product(range(nk), range(nc)):
            rk, vk, tk = (a, i, b, j), (a, k, c, i), (c, b, k, j)
            out.append((R.block(rk), V.block(vk), T.block(tk), R.ext(rk), V.ext(vk), T.ext(tk)))
    return out


def segments_uniform(total: int, lo: int, hi: int, seed: int):
    """Segment sizes drawn uniformly from [lo, hi] (seeded) until they cover
    `total`; the last segment absorbs the remainder."""
    rng = np.random.default_rng(seed)
    segs, acc = [], 0
    while total - acc > hi:
        s = int(rng.integers(lo, hi + 1))
        segs.append(s)
        acc += s
    if total - acc > 0:
        segs.append(total - acc)
    return segs


def segments_choice(total: int, choices, seed: int):
    """Segment sizes drawn from `choices` (seeded) summing exactly to `total`."""
    rng = np.random.default_rng(seed)
    choices = sorted(choices)
    segs, acc = [], 0
    while acc < total:
        fit = [c for c in choices if acc + c <= total and (total - acc - c == 0 or total - acc - c >= choices[0])]
        s = int(rng.choice(fit))
        segs.append(s)
        acc += s
    return segs


# (T)-type connected triples, W(a,i,b,j,c,k) = sum_d V1(b,c,d,k) T(a,d,i,j)
#                                            - sum_l V2(l,c,j,k) T(a,b,i,l)
# labels: a=1 i=2 b=3 j=4 c=5 k=6 d=7 l=8; W is stored in the denominator's
# index order (virtual, occupied, virtual, occupied, virtual, occupied), the
# order energy_denominator_rhf's rank-6 form expects (rccsdpt_aaa.sialx:2163-2172).
TRIPLES_TERM1_LABELS = ([1, 2, 3, 4, 5, 6], [3, 5, 7, 6], [1, 7, 2, 4])
TRIPLES_TERM2_LABELS = ([1, 2, 3, 4, 5, 6], [8, 5, 4, 6], [1, 3, 2, 8])


def triples_step(W: BlockArray, V1: BlockArray, V2: BlockArray, T: BlockArray, a: int, b: int, w_key=None):
    """Block triples of one pardo step of the triples energy: the fixed
    virtual segments (a, b), every c and every occupied (i, j, k).  Returns
    (term-1 triples, term-2 triples); the second term is run with negate=1
    and beta=1 into the same W blocks.  w_key maps a W block key to the key
    of the W block that stands for it (a step whose W is never stored can
    name another step's blocks of the same extents)."""
    nv, no = len(T.segs[0]), len(T.segs[2])
    t1, t2 = [], []
    for c in range(nv):
        for i, j, k in itertools.product(range(no), repeat=3):
            wk = (a, i, b, j, c, k)
            if w_key is not None:
                wk = w_key(wk)
            wb, we = W.block(wk), W.ext(wk)
            for d in range(nv):
                lk, rk = (b, c, d, k), (a, d, i, j)
                t1.append((wb, V1.block(lk), T.block(rk), we, V1.ext(lk), T.ext(rk)))
            for l in range(no):
                lk, rk = (l, c, j, k), (a, b, i, l)
                t2.append((wb, V2.block(lk), T.block(rk), we, V2.ext(lk), T.ext(rk)))
    return t1, t2


def triples_index_values(key, n_occ_segs: int):
    """1-based global segment numbers of W block `key` (occupied segments
    first, then virtual, as moa_seg_ranges lists them)."""
    a, i, b, j, c, k = key
    return [n_occ_segs + a + 1, i + 1, n_occ_segs + b + 1, j + 1, n_occ_segs + c + 1, k + 1]


def ladder_slab_triples(R: BlockArray, V: BlockArray, T: BlockArray, a: int, b: int, v_slab: bool = False):
    """Triples of one (a,b) slab of the ladder: R(a,b,i,j) += V(a,b,c,d)
    T(c,d,i,j) for every (i,j) and (c,d).  v_slab: V holds only this slab's
    blocks, keyed (0,0,c,d) (a buffer reused slab after slab)."""
    nc, nd = len(V.segs[2]), len(V.segs[3])
    ni, nj = len(T.segs[2]), len(T.segs[3])
    out = []
    for i, j in itertools.product(range(ni), range(nj)):
        for c, d in itertools.product(range(nc), range(nd)):
            rk, vk, tk = (a, b, i, j), ((0, 0, c, d) if v_slab else (a, b, c, d)), (c, d, i, j)
            out.append((R.block(rk), V.block(vk), T.block(tk), R.ext(rk), V.ext(vk), T.ext(tk)))
    return out


def ladder_slab_array(R: BlockArray, V: BlockArray, T: BlockArray, a: int, b: int, v_slab: bool = True):
    """The triples of ladder_slab_triples as a numpy a4g_triple array (block
    addresses and extents), which the batch calls take without building a
    Python tuple per triple."""
    from .device import TRIPLE_DTYPE

    nc, nd = len(V.segs[2]), len(V.segs[3])
    ni, nj = len(T.segs[2]), len(T.segs[3])
    ij = list(itertools.product(range(ni), range(nj)))
    cd = list(itertools.product(range(nc), range(nd)))
    rks = [(a, b) + x for x in ij for _ in cd]
    vks = [((0, 0) if v_slab else (a, b)) + y for _ in ij for y in cd]
    tks = [y + x for x in ij for y in cd]
    out = np.zeros(len(rks), TRIPLE_DTYPE)
    for col, arr, ks in (("d", R, rks), ("l", V, vks), ("r", T, tks)):
        out[col] = np.uint64(arr.buf.data_ptr()) + np.uint64(8) * np.array([arr.offsets[k] for k in ks], np.uint64)
        ext = out[col + "ext"]
        ext[:, :4] = np.array([arr.ext(k) for k in ks], np.int32)
        ext[:, 4:] = 1
    return out
