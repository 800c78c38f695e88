"""Reference-named drop-in entry points on HOST numpy buffers.

Each function calls the C-ABI symbol of the same name (the symbols a C++ or
Fortran host binds through src/sip/tensor_algebra/tensor_ops_c_prototypes.h)
and returns the reference's ierr (0 = success).  Blocks are flat float64
arrays in column-major element order.  Work runs on the GPU; nothing here
computes on the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import last_error, lib

_i = ctypes.c_int
_d = ctypes.c_double


def _iarr(seq):
    seq = [int(x) for x in seq]
    return (ctypes.c_int * max(1, len(seq)))(*seq)


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise TypeError("blocks must be contiguous float64 arrays")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def get_contraction_ptrn(drank: int, lrank: int, rrank: int, aces_ptrn) -> tuple[int, list[int]]:
    out = (ctypes.c_int * max(1, lrank + rrank))()
    ierr = _i(0)
    lib().get_contraction_ptrn_(ctypes.byref(_i(drank)), ctypes.byref(_i(lrank)),
                                ctypes.byref(_i(rrank)), _iarr(aces_ptrn), out, ctypes.byref(ierr))
    return ierr.value, list(out)[: lrank + rrank]


def tensor_block_contract(ptrn, l, lext, r, rext, d, dext, nthreads: int = 8) -> int:
    """D is overwritten with contract(L, R), like tensor_dil_omp.F90:662."""
    ierr = _i(0)
    lib().tensor_block_contract__(
        ctypes.byref(_i(nthreads)), _iarr(ptrn), _dp(l), ctypes.byref(_i(len(lext))), _iarr(lext),
        _dp(r), ctypes.byref(_i(len(rext))), _iarr(rext), _dp(d), ctypes.byref(_i(len(dext))),
        _iarr(dext), ctypes.byref(ierr))
    return ierr.value


def contract_labels(dlab, llab, rlab, l, lext, r, rext, dext):
    """Interpreter::handle_contraction (interpreter.cpp:1210-1262): labels ->
    pattern -> tensor_block_contract__.  Returns (ierr, D)."""
    ierr, ptrn = get_contraction_ptrn(len(dlab), len(llab), len(rlab), list(dlab) + list(llab) + list(rlab))
    if ierr:
        return ierr, None
    n = int(np.prod(dext)) if len(dext) else 1
    d = np.full(n, np.nan)
    return tensor_block_contract(ptrn, l, lext, r, rext, d, dext), d


def tensor_block_copy(ext, perm_o2n_1based, tin: np.ndarray, out: np.ndarray | None = None) -> tuple[int, np.ndarray]:
    """perm without the sign slot (added here); out: the destination block
    (a new array when None)."""
    out = np.empty_like(tin) if out is None else out
    ierr = _i(0)
    lib().tensor_block_copy__(ctypes.byref(_i(8)), ctypes.byref(_i(len(ext))), _iarr(ext),
                              _iarr([1] + list(perm_o2n_1based)), _dp(tin), _dp(out), ctypes.byref(ierr))
    return ierr.value, out


def tensor_block_add(ext, t0, t1, scale) -> int:
    ierr = _i(0)
    lib().tensor_block_add__(ctypes.byref(_i(8)), ctypes.byref(_i(len(ext))), _iarr(ext), _dp(t0),
                             _dp(t1), ctypes.byref(_d(scale)), ctypes.byref(ierr))
    return ierr.value


def tensor_block_scale(t, ext, f) -> int:
    ierr = _i(0)
    lib().tensor_block_scale__(ctypes.byref(_i(8)), _dp(t), ctypes.byref(_i(len(ext))), _iarr(ext),
                               ctypes.byref(_d(f)), ctypes.byref(ierr))
    return ierr.value


def tensor_block_init(t, ext, v) -> int:
    ierr = _i(0)
    lib().tensor_block_init__(ctypes.byref(_i(8)), _dp(t), ctypes.byref(_i(len(ext))), _iarr(ext),
                              ctypes.byref(_d(v)), ctypes.byref(ierr))
    return ierr.value


def tensor_block_norm2(t, ext) -> tuple[float, int]:
    ierr = _i(0)
    v = lib().tensor_block_norm2__(ctypes.byref(_i(8)), _dp(t), ctypes.byref(_i(len(ext))),
                                   _iarr(ext), ctypes.byref(ierr))
    return v, ierr.value


def tensor_block_slice(t, text, sext, beg) -> tuple[int, np.ndarray]:
    s = np.empty(int(np.prod(sext)) if len(sext) else 1)
    ierr = _i(0)
    lib().tensor_block_slice__(ctypes.byref(_i(8)), ctypes.byref(_i(len(text))), _dp(t), _iarr(text),
                               _dp(s), _iarr(sext), _iarr(beg), ctypes.byref(ierr))
    return ierr.value, s


def tensor_block_insert(t, text, s, sext, beg) -> int:
    ierr = _i(0)
    lib().tensor_block_insert__(ctypes.byref(_i(8)), ctypes.byref(_i(len(text))), _dp(t), _iarr(text),
                                _dp(s), _iarr(sext), _iarr(beg), ctypes.byref(ierr))
    return ierr.value


def host_direct(enable: bool) -> int:
    """Drop-ins run on the host blocks in place where the GPU reads host
    memory through the host's page tables (default), or stage them through
    device memory (False).  Returns the a4g status (6: no host access)."""
    return lib().a4g_host_direct(int(bool(enable)))


def set_predefined_int_array(name: str, values) -> int:
    arr = _iarr(values)
    return lib().a4g_set_predefined_int_array(name.encode(), len(values), ctypes.cast(arr, ctypes.c_void_p))


def energy_denominator_rhf(index_values, ext0, data0, ext1, data1) -> int:
    """fp2 super-instruction ABI (special_instructions.h:73-74); data0 in place."""
    ierr = _i(0)
    r0, r1 = len(ext0), len(ext1)
    lib().energy_denominator_rhf(
        ctypes.byref(_i(0)), ctypes.byref(_i(r0)), _iarr(index_values), ctypes.byref(_i(data0.size)),
        _iarr(ext0), _dp(data0), ctypes.byref(_i(1)), ctypes.byref(_i(r1)), _iarr([1] * r1),
        ctypes.byref(_i(data1.size)), _iarr(ext1), _dp(data1), ctypes.byref(ierr))
    return ierr.value


READ, UPDATE, OVERWRITE = 0, 1, 2


class BlockCache:
    """Device residency of host blocks (a4g_blocks_*): the GPU side of the
    reference's BlockManager.  Blocks are numpy float64 arrays (their data
    pointers identify them).  attach() makes the drop-ins above use it."""

    def __init__(self, capacity_bytes: int):
        h = ctypes.c_void_p(0)
        rc = lib().a4g_blocks_create(ctypes.byref(h), ctypes.c_size_t(capacity_bytes))
        if rc:
            raise RuntimeError(f"a4g_blocks_create failed ({rc}): {last_error()}")
        self._h = h

    def _ok(self, rc, what):
        if rc:
            raise RuntimeError(f"{what} failed ({rc}): {last_error()}")

    def attach(self):
        self._ok(lib().a4g_blocks_attach(self._h), "a4g_blocks_attach")

    def detach(self):
        self._ok(lib().a4g_blocks_attach(None), "a4g_blocks_attach")

    def on_device(self, a: np.ndarray, mode: int = READ) -> int:
        d = ctypes.c_void_p(0)
        self._ok(lib().a4g_blocks_on_device(self._h, _dp(a), ctypes.c_int64(a.size), mode, ctypes.byref(d), None),
                 "a4g_blocks_on_device")
        return d.value

    def on_host(self, a: np.ndarray, mode: int = READ):
        self._ok(lib().a4g_blocks_on_host(self._h, _dp(a), mode, None), "a4g_blocks_on_host")

    def flush(self):
        self._ok(lib().a4g_blocks_flush(self._h, None), "a4g_blocks_flush")

    def forget(self, a: np.ndarray):
        self._ok(lib().a4g_blocks_forget(self._h, _dp(a)), "a4g_blocks_forget")

    def stats(self) -> dict:
        v = [ctypes.c_int64(0) for _ in range(4)]
        self._ok(lib().a4g_blocks_stats(self._h, *[ctypes.byref(x) for x in v]), "a4g_blocks_stats")
        return dict(zip(("h2d_bytes", "d2h_bytes", "resident_bytes", "evictions"), (x.value for x in v)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().a4g_blocks_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
