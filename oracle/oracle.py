"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference ACES4 block kernels in plain C
(``oracle/a4_oracle.c``).  Tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` load it to check results against (and to time the
CPU baseline); the product library never does.  Arrays are numpy float64 in column-major (Fortran) element order, passed
as flat buffers exactly like the reference's ``double*`` blocks.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liba4oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build() -> str:
    """Compile the oracle with its Makefile (seconds; gcc only)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(
            os.path.join(_HERE, "a4_oracle.c")
        ):
            build()
        L = ctypes.CDLL(_SO)
        L.a4o_tensor_block_norm2.restype = ctypes.c_double
        L.a4o_tensor_size_by_shape.restype = ctypes.c_int64
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.c_contiguous or a.flags.f_contiguous)
    return a.ctypes.data_as(_dp)


def _i(seq) -> ctypes.Array:
    seq = list(seq)
    return (ctypes.c_int * max(1, len(seq)))(*seq)


def flat(a: np.ndarray) -> np.ndarray:
    """Column-major flat view/copy of an n-d array (block memory order)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def get_contraction_ptrn(drank: int, lrank: int, rrank: int, aces_ptrn):
    out = (ctypes.c_int * max(1, lrank + rrank))()
    ierr = lib().a4o_get_contraction_ptrn(drank, lrank, rrank, _i(aces_ptrn), out)
    return ierr, list(out)[: lrank + rrank]


def contr_ptrn_ok(ptrn, lext, rext, dext) -> bool:
    return bool(
        lib().a4o_contr_ptrn_ok(
            _i(ptrn), len(lext), len(rext), len(dext), _i(lext), _i(rext), _i(dext)
        )
    )


def tensor_block_copy(ext, perm_o2n_1based, tin: np.ndarray) -> tuple[int, np.ndarray]:
    """perm_o2n_1based excludes the sign slot; it is added here."""
    tin = np.ascontiguousarray(tin, dtype=np.float64).reshape(-1)
    out = np.empty_like(tin)
    ierr = lib().a4o_tensor_block_copy(len(ext), _i(ext), _i([1] + list(perm_o2n_1based)), _d(tin), _d(out))
    return ierr, out


def tensor_block_contract(ptrn, l, lext, r, rext, d, dext) -> int:
    """D is overwritten in place (flat float64 buffers)."""
    return lib().a4o_tensor_block_contract(
        _i(ptrn), _d(l), len(lext), _i(lext), _d(r), len(rext), _i(rext), _d(d), len(dext), _i(dext)
    )


def contract_labels(dlab, llab, rlab, l, lext, r, rext, dext):
    """Interpreter-style contraction: labels -> pattern -> overwrite D."""
    ierr, ptrn = get_contraction_ptrn(len(dlab), len(llab), len(rlab), list(dlab) + list(llab) + list(rlab))
    if ierr:
        return ierr, None
    n = int(np.prod(dext)) if len(dext) else 1
    d = np.full(n, np.nan)
    ierr = tensor_block_contract(ptrn, l, lext, r, rext, d, dext)
    return ierr, d


def tensor_block_init(t, ext, v) -> int:
    return lib().a4o_tensor_block_init(_d(t), len(ext), _i(ext), ctypes.c_double(v))


def tensor_block_scale(t, ext, f) -> int:
    return lib().a4o_tensor_block_scale(_d(t), len(ext), _i(ext), ctypes.c_double(f))


def tensor_block_norm2(t, ext) -> tuple[float, int]:
    ierr = ctypes.c_int(0)
    v = lib().a4o_tensor_block_norm2(_d(t), len(ext), _i(ext), ctypes.byref(ierr))
    return v, ierr.value


def tensor_block_add(ext, t0, t1, scale) -> int:
    return lib().a4o_tensor_block_add(len(ext), _i(ext), _d(t0), _d(t1), ctypes.c_double(scale))


def tensor_block_slice(t, text, sext, beg) -> tuple[int, np.ndarray]:
    s = np.empty(int(np.prod(sext)) if len(sext) else 1)
    ierr = lib().a4o_tensor_block_slice(len(text), _d(t), _i(text), _d(s), _i(sext), _i(beg))
    return ierr, s


def tensor_block_insert(t, text, s, sext, beg) -> int:
    return lib().a4o_tensor_block_insert(len(text), _d(t), _i(text), _d(s), _i(sext), _i(beg))


def block_add_sub(subtract, d_ids, l_ids, r_ids, r_ext, d_is_l, d, l, r) -> int:
    return lib().a4o_block_add_sub(
        int(subtract), len(r_ext), _i(d_ids), _i(l_ids), _i(r_ids), _i(r_ext), int(d_is_l), _d(d), _d(l), _d(r)
    )


def block_scale_and_copy(d, s, f):
    lib().a4o_block_scale_and_copy(_d(d), _d(s), ctypes.c_int64(d.size), ctypes.c_double(f))


def block_increment(d, delta):
    lib().a4o_block_increment(_d(d), ctypes.c_int64(d.size), ctypes.c_double(delta))


def block_accumulate(d, s):
    lib().a4o_block_accumulate(_d(d), _d(s), ctypes.c_int64(d.size))


def energy_denominator_rhf(index_values, ext0, data0, ext1, data1, seg_sizes) -> int:
    return lib().a4o_energy_denominator_rhf(
        len(ext0), _i(index_values), _i(ext0), _d(data0), len(ext1), _i(ext1), _d(data1),
        len(seg_sizes), _i(seg_sizes),
    )


def fill_block_cyclic(n: int, start: float) -> np.ndarray:
    d = np.empty(n)
    lib().a4o_fill_block_cyclic(_d(d), ctypes.c_int64(n), ctypes.c_double(start))
    return d


def fill_block_sequential(n: int, start: float) -> np.ndarray:
    d = np.empty(n)
    lib().a4o_fill_block_sequential(_d(d), ctypes.c_int64(n), ctypes.c_double(start))
    return d


def contract_plan(ptrn, lext, rext, dext):
    """Python restatement of determine_index_permutations (F90:799-859) used by
    the CPU baseline to drive an external BLAS GEMM.  Returns
    (lo2n, ro2n, do2n) as 1-based O2N lists without sign slot, and (lld, lrd, lcd)."""
    lrank, rrank, drank = len(lext), len(rext), len(dext)
    do2n = [p for p in ptrn if p > 0] if drank else []
    ro2n = [0] * rrank
    j1 = 0
    lcd = lrd = lld = 1
    for j0 in range(rrank):
        if ptrn[lrank + j0] < 0:
            j1 += 1
            ro2n[j0] = j1
            lcd *= rext[j0]
    for j0 in range(rrank):
        if ptrn[lrank + j0] > 0:
            j1 += 1
            ro2n[j0] = j1
            lrd *= rext[j0]
    lo2n = [0] * lrank
    con = [(j0, -ptrn[j0]) for j0 in range(lrank) if ptrn[j0] < 0]
    for pos, (j0, _) in enumerate(sorted(con, key=lambda t: t[1])):
        lo2n[j0] = pos + 1
    j1 = len(con)
    for j0 in range(lrank):
        if ptrn[j0] > 0:
            j1 += 1
            lo2n[j0] = j1
            lld *= lext[j0]
    return lo2n, ro2n, do2n, (lld, lrd, lcd)


def contract_blas(ptrn, l, lext, r, rext, dext, threads: int | None = None) -> np.ndarray:
    """The reference's CPU BLAS path (tensor_dil_omp.F90:729-785): permute the
    operands into temporaries with the oracle's tensor_block_copy, call
    dgemm('T','N') (numpy's bundled OpenBLAS), permute the result back.
    Used as the timed CPU baseline; returns the overwritten D (flat)."""
    lo2n, ro2n, do2n, (lld, lrd, lcd) = contract_plan(ptrn, lext, rext, dext)
    ltp = l if lo2n == sorted(lo2n) else tensor_block_copy(lext, lo2n, l)[1]
    rtp = r if ro2n == sorted(ro2n) else tensor_block_copy(rext, ro2n, r)[1]
    # column-major lcd x lld  ==  row-major lld x lcd
    dtp = np.matmul(ltp.reshape(lld, lcd), rtp.reshape(lrd, lcd).T)  # lld x lrd (row-major)
    dtp = np.ascontiguousarray(dtp.T).reshape(-1)  # column-major lld x lrd
    if do2n == sorted(do2n):
        return dtp
    mext = [dext[p - 1] for p in do2n]
    return tensor_block_copy(mext, do2n, dtp)[1]


def energy_contract(index_values, ext0, w, ext1, fock, seg_sizes, efact, den_order=None) -> float:
    """The (T) energy pattern of one block, rccsdpt_aaa.sialx:2163-2172, as
    the reference's operations: permute the block into the denominator's index
    order (tensor_block_copy_), divide a copy by the orbital-energy
    denominators (energy_denominator_rhf), contract the divided block with the
    undivided one to a scalar (tensor_block_contract_ with drank 0, i.e.
    tensor_block_fcontract), multiply by efact.  Returns the contribution
    added to esum."""
    w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1)
    r = len(ext0)
    order = list(den_order) if den_order is not None else list(range(r))
    if order != list(range(r)):
        o2n = [0] * r
        for q, dim in enumerate(order):
            o2n[dim] = q + 1
        ierr, wp = tensor_block_copy(ext0, o2n, w)
        assert ierr == 0
    else:
        wp = w.copy()
    ext_p = [ext0[d] for d in order]
    iv_p = [index_values[d] for d in order]
    wd = wp.copy()
    assert energy_denominator_rhf(iv_p, ext_p, wd, ext1, np.ascontiguousarray(fock, dtype=np.float64), seg_sizes) == 0
    labels = list(range(1, r + 1))
    ierr, ptrn = get_contraction_ptrn(0, r, r, labels + labels)
    assert ierr == 0
    etemp = np.zeros(1)
    assert tensor_block_contract(ptrn, wd, ext_p, wp, ext_p, etemp, []) == 0
    return float(etemp[0] * efact)


def update_t2(index_values, ext, t2new, t2new_pair, t2old, t2old_pair, ext1, fock, seg_sizes):
    """Procedure updatet2 of rlccd_rhf.sialx:557-600 for one block (a,i,b,j),
    as the reference's block operations: permuted copies of the (b,j,a,i)
    partner blocks (tensor_block_copy_), in-place block adds/subtracts
    (handle_block_add/subtract), energy_denominator_rhf, Block::scale; the
    error block's squared norm by tensor_block_norm2_.  Returns (E, next
    T2old block, norm2)."""
    ea, ei, eb, ej = ext
    pair_ext = [eb, ej, ea, ei]
    o2n = [3, 4, 1, 2]  # (b,j,a,i) -> (a,i,b,j)
    ids = [1, 2, 3, 4]
    f = np.ascontiguousarray(fock, dtype=np.float64)

    def perm(x):
        ierr, out = tensor_block_copy(pair_ext, o2n, np.ascontiguousarray(x, dtype=np.float64))
        assert ierr == 0
        return out

    t2new = np.ascontiguousarray(t2new, dtype=np.float64)
    t2old = np.ascontiguousarray(t2old, dtype=np.float64)
    # first pass
    taibj = perm(t2new_pair)
    assert block_add_sub(0, ids, ids, ids, ext, 1, taibj, taibj.copy(), t2new) == 0
    t1 = perm(t2old_pair)
    assert block_add_sub(0, ids, ids, ids, ext, 1, t1, t1.copy(), t2old) == 0
    assert energy_denominator_rhf(index_values, ext, taibj, ext1, f, seg_sizes) == 0
    assert block_add_sub(1, ids, ids, ids, ext, 1, t1, t1.copy(), taibj) == 0
    assert tensor_block_scale(t1, ext, -0.5) == 0
    err = t1
    # second pass
    t2 = perm(t2new_pair)
    assert block_add_sub(0, ids, ids, ids, ext, 1, t2, t2.copy(), t2new) == 0
    assert tensor_block_scale(t2, ext, 0.5) == 0
    assert energy_denominator_rhf(index_values, ext, t2, ext1, f, seg_sizes) == 0
    nrm, ierr = tensor_block_norm2(err, ext)
    assert ierr == 0
    return err, t2, nrm


# ------------------------------------------------------------ reference GPU path
# The reference's legacy GPU contraction (gpu_super_instructions.cu:369-586):
# its own kernels from oracle/_ref/gpu_super_instructions.cubin (compiled from
# the reference tree by the Makefile, where that tree is present), driven by
# the host steps restated in ref_gpu.cpp.  Test and baseline use only.
_REF_CUBIN = os.path.join(_HERE, "_ref", "gpu_super_instructions.cubin")
_REF_GPU_SO = os.path.join(_HERE, "_build", "libref_gpu.so")
_ref_gpu = None


def ref_gpu_available() -> bool:
    return os.path.exists(_REF_CUBIN) and os.path.exists(_REF_GPU_SO)


def ref_gpu():
    """The loaded driver (raises when the cubin or the driver is missing)."""
    global _ref_gpu
    if _ref_gpu is None:
        if not ref_gpu_available():
            raise RuntimeError("reference GPU path unavailable: " + _REF_CUBIN + " not built")
        L = ctypes.CDLL(_REF_GPU_SO)
        L.ref_gpu_error.restype = ctypes.c_char_p
        if L.ref_gpu_load(_REF_CUBIN.encode()) != 0:
            raise RuntimeError("ref_gpu_load: " + L.ref_gpu_error().decode())
        _ref_gpu = L
    return _ref_gpu


def ref_gpu_contract(y: int, ydims, yinds, x1: int, x1dims, x1inds, x2: int, x2dims, x2inds):
    """_gpu_contract on device addresses: y = x1 * x2 (synchronous, like the reference)."""
    L = ref_gpu()
    rc = L.ref_gpu_contract(ctypes.c_void_p(y), len(ydims), _i(ydims), _i(yinds), ctypes.c_void_p(x1), len(x1dims),
                            _i(x1dims), _i(x1inds), ctypes.c_void_p(x2), len(x2dims), _i(x2dims), _i(x2inds))
    if rc != 0:
        raise RuntimeError("ref_gpu_contract: " + L.ref_gpu_error().decode())
