"""Device-resident block operations (the a4g_* C ABI) on CUDA buffers.

Buffers are torch CUDA tensors of float64 (or raw device addresses as ints);
torch only provides device memory and streams here — every operation is one
of the library's own CUDA kernels.  Functions raise ``A4GError`` carrying the
library's error text when the C call reports a failure.
"""
from __future__ import annotations

import ctypes

from ._lib import lib, last_error

_i = ctypes.c_int


class A4GError(RuntimeError):
    def __init__(self, rc: int, what: str):
        super().__init__(f"{what} failed (status {rc}): {last_error()}")
        self.rc = rc


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if getattr(x, "is_cuda", False) is False and hasattr(x, "data_ptr"):
        raise TypeError("device API expects CUDA tensors")
    return x.data_ptr()


def _iarr(seq):
    seq = [int(v) for v in seq]
    return (ctypes.c_int * max(1, len(seq)))(*seq)


def _stream(stream) -> ctypes.c_void_p:
    if stream is None:
        return ctypes.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def _check(rc: int, what: str):
    if rc != 0:
        raise A4GError(rc, what)


def init(device: int = -1):
    _check(lib().a4g_init(device), "a4g_init")


def sync(stream=None):
    _check(lib().a4g_sync(_stream(stream)), "a4g_sync")


def contract(ptrn, l, lext, r, rext, d, dext, beta: int = 0, stream=None):
    """D (=|+=) contract(L, R) with the reference pattern format."""
    rc = lib().a4g_contract(_iarr(ptrn), ctypes.c_void_p(_ptr(l)), _i(len(lext)), _iarr(lext),
                            ctypes.c_void_p(_ptr(r)), _i(len(rext)), _iarr(rext),
                            ctypes.c_void_p(_ptr(d)), _i(len(dext)), _iarr(dext), _i(beta), _stream(stream))
    _check(rc, "a4g_contract")


def contract_labels(dlab, llab, rlab, l, lext, r, rext, d, dext, beta: int = 0, stream=None):
    rc = lib().a4g_contract_labels(_iarr(dlab), _iarr(llab), _iarr(rlab), ctypes.c_void_p(_ptr(l)),
                                   _i(len(lext)), _iarr(lext), ctypes.c_void_p(_ptr(r)), _i(len(rext)),
                                   _iarr(rext), ctypes.c_void_p(_ptr(d)), _i(len(dext)), _iarr(dext),
                                   _i(beta), _stream(stream))
    _check(rc, "a4g_contract_labels")


def permute(ext, perm_o2n_1based, src, dst, stream=None):
    rc = lib().a4g_permute(_i(len(ext)), _iarr(ext), _iarr([1] + list(perm_o2n_1based)),
                           ctypes.c_void_p(_ptr(src)), ctypes.c_void_p(_ptr(dst)), _stream(stream))
    _check(rc, "a4g_permute")


def fill(d, value: float, stream=None):
    _check(lib().a4g_fill(_ptr(d), d.numel(), float(value), _stream(stream)), "a4g_fill")


def scale(d, factor: float, stream=None):
    _check(lib().a4g_scale(_ptr(d), d.numel(), float(factor), _stream(stream)), "a4g_scale")


def scale_copy(d, s, factor: float, stream=None):
    _check(lib().a4g_scale_copy(_ptr(d), _ptr(s), d.numel(), float(factor), _stream(stream)), "a4g_scale_copy")


def increment(d, delta: float, stream=None):
    _check(lib().a4g_increment(_ptr(d), d.numel(), float(delta), _stream(stream)), "a4g_increment")


def add_scaled(t0, t1, scale_fac: float, stream=None):
    _check(lib().a4g_add_scaled(_ptr(t0), _ptr(t1), t0.numel(), float(scale_fac), _stream(stream)),
           "a4g_add_scaled")


def add_sub(subtract: bool, d_labels, r_labels, r_ext, d, l, r, stream=None):
    rc = lib().a4g_add_sub(_i(int(subtract)), _i(len(r_ext)), _iarr(d_labels), _iarr(r_labels), _iarr(r_ext),
                           ctypes.c_void_p(_ptr(d)), ctypes.c_void_p(_ptr(l)), ctypes.c_void_p(_ptr(r)),
                           _stream(stream))
    _check(rc, "a4g_add_sub")


def norm2(t, stream=None) -> float:
    out = ctypes.c_double(0.0)
    _check(lib().a4g_norm2(_ptr(t), t.numel(), ctypes.byref(out), _stream(stream)), "a4g_norm2")
    return out.value


def slice_block(tens, text, slice_, sext, beg, stream=None):
    rc = lib().a4g_slice(_i(len(text)), ctypes.c_void_p(_ptr(tens)), _iarr(text), ctypes.c_void_p(_ptr(slice_)),
                         _iarr(sext), _iarr(beg), _stream(stream))
    _check(rc, "a4g_slice")


def insert_block(tens, text, slice_, sext, beg, stream=None):
    rc = lib().a4g_insert(_i(len(text)), ctypes.c_void_p(_ptr(tens)), _iarr(text), ctypes.c_void_p(_ptr(slice_)),
                          _iarr(sext), _iarr(beg), _stream(stream))
    _check(rc, "a4g_insert")


def energy_denominator(index_values, ext0, data0, ext1, e_or_fock, seg_sizes, stream=None):
    rc = lib().a4g_energy_denominator(_i(len(ext0)), _iarr(index_values), _iarr(ext0),
                                      ctypes.c_void_p(_ptr(data0)), _i(len(ext1)), _iarr(ext1),
                                      ctypes.c_void_p(_ptr(e_or_fock)), _i(len(seg_sizes)), _iarr(seg_sizes),
                                      _stream(stream))
    _check(rc, "a4g_energy_denominator")


# ------------------------------------------------ legacy GPU API (synchronous)
def gpu_contract(y, ydims, yinds, x1, x1dims, x1inds, x2, x2dims, x2inds):
    lib()._gpu_contract(ctypes.c_void_p(_ptr(y)), _i(len(ydims)), _iarr(ydims), _iarr(yinds),
                        ctypes.c_void_p(_ptr(x1)), _i(len(x1dims)), _iarr(x1dims), _iarr(x1inds),
                        ctypes.c_void_p(_ptr(x2)), _i(len(x2dims)), _iarr(x2dims), _iarr(x2inds))


def gpu_permute(y, ydims, yinds, x, xdims, xinds):
    lib()._gpu_permute(ctypes.c_void_p(_ptr(y)), _i(len(ydims)), _iarr(ydims), _iarr(yinds),
                       ctypes.c_void_p(_ptr(x)), _i(len(xdims)), _iarr(xdims), _iarr(xinds))
