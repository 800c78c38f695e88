"""Device-resident block operations (the a4g_* C ABI) on CUDA buffers.

Buffers are torch CUDA tensors of float64 (or raw device addresses as ints);
torch only provides device memory and streams here — every operation is one
of the library's own CUDA kernels.  Functions raise ``A4GError`` carrying the
library's error text when the C call reports a failure.
"""
from __future__ import annotations

import ctypes

import numpy as np

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
    if str(getattr(x, "dtype", "torch.float64")) != "torch.float64":
        raise TypeError(f"device API expects float64 tensors, got {x.dtype}")
    return x.data_ptr()


def _iarr(seq):
    seq = [int(v) for v in seq]
    return (ctypes.c_int * max(1, len(seq)))(*seq)


_LEGACY_DEFAULT_STREAM = 1  # cudaStreamLegacy


def _stream(stream) -> ctypes.c_void_p:
    """None -> the library's own stream; a torch stream object -> that stream
    (torch's default stream, handle 0, is passed as cudaStreamLegacy so work
    is ordered with torch's default-stream kernels and events)."""
    if stream is None:
        return ctypes.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream or _LEGACY_DEFAULT_STREAM)
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


def update_t2(index_values, ext, t2new, t2new_pair, t2old, t2old_pair, diis_err, t2old_next, ext1, e_or_fock,
              seg_sizes, norm2=None, stream=None):
    """updatet2 for one (a,i,b,j) block (a4g_update_t2): writes the DIIS error
    block and the next T2old block, adds sum(err^2) to norm2 (CUDA float64)."""
    p = lambda x: ctypes.c_void_p(_ptr(x)) if x is not None else None
    rc = lib().a4g_update_t2(_iarr(index_values), _iarr(ext), p(t2new), p(t2new_pair), p(t2old), p(t2old_pair),
                             p(diis_err), p(t2old_next), _i(len(ext1)), _iarr(ext1), p(e_or_fock),
                             _i(len(seg_sizes)), _iarr(seg_sizes), p(norm2), _stream(stream))
    _check(rc, "a4g_update_t2")


def energy_contract(index_values, ext0, data0, ext1, e_or_fock, seg_sizes, efact, esum, den_order=None,
                    stream=None):
    """esum (1-element CUDA float64 tensor) += efact * sum w * (w / eps): the
    fused (T)-energy pass of one block (a4g_energy_contract)."""
    order = _iarr(den_order) if den_order is not None else None
    rc = lib().a4g_energy_contract(_i(len(ext0)), _iarr(index_values), _iarr(ext0), ctypes.c_void_p(_ptr(data0)),
                                   order, _i(len(ext1)), _iarr(ext1), ctypes.c_void_p(_ptr(e_or_fock)),
                                   _i(len(seg_sizes)), _iarr(seg_sizes), ctypes.c_double(efact),
                                   ctypes.c_void_p(_ptr(esum)), _stream(stream))
    _check(rc, "a4g_energy_contract")


# ------------------------------------------------ legacy GPU API (synchronous)
def gpu_contract(y, ydims, yinds, x1, x1dims, x1inds, x2, x2dims, x2inds):
    lib()._gpu_contract(ctypes.c_void_p(_ptr(y)), _i(len(ydims)), _iarr(ydims), _iarr(yinds),
                        ctypes.c_void_p(_ptr(x1)), _i(len(x1dims)), _iarr(x1dims), _iarr(x1inds),
                        ctypes.c_void_p(_ptr(x2)), _i(len(x2dims)), _iarr(x2dims), _iarr(x2inds))


def gpu_permute(y, ydims, yinds, x, xdims, xinds):
    lib()._gpu_permute(ctypes.c_void_p(_ptr(y)), _i(len(ydims)), _iarr(ydims), _iarr(yinds),
                       ctypes.c_void_p(_ptr(x)), _i(len(xdims)), _iarr(xdims), _iarr(xinds))


# ------------------------------------------------ batched pardo step
PREC_FP64 = 0
PREC_OZAKI_BF16 = 1


class _Triple(ctypes.Structure):
    _fields_ = [("d", ctypes.c_void_p), ("l", ctypes.c_void_p), ("r", ctypes.c_void_p),
                ("dext", ctypes.c_int * 6), ("lext", ctypes.c_int * 6), ("rext", ctypes.c_int * 6)]


class _Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("slices", ctypes.c_int), ("beta", ctypes.c_int),
                ("variant", ctypes.c_int), ("negate", ctypes.c_int), ("pipeline", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


def _ext6(e):
    e = list(e) + [1] * (6 - len(e))
    return (ctypes.c_int * 6)(*e)


# numpy image of a4g_triple (96 bytes): block addresses and extents
TRIPLE_DTYPE = np.dtype([("d", "<u8"), ("l", "<u8"), ("r", "<u8"), ("dext", "<i4", (6,)),
                         ("lext", "<i4", (6,)), ("rext", "<i4", (6,))])


def _triple_array(tl):
    arr = (_Triple * max(1, len(tl)))()
    for i, (d, l, r, de, le, re) in enumerate(tl):
        arr[i].d, arr[i].l, arr[i].r = _ptr(d), _ptr(l), _ptr(r)
        arr[i].dext, arr[i].lext, arr[i].rext = _ext6(de), _ext6(le), _ext6(re)
    return arr


def _triples_arg(triples):
    """(pointer to an a4g_triple array, count, object keeping it alive) from
    a list of (d, l, r, dext, lext, rext) or a TRIPLE_DTYPE numpy array."""
    if isinstance(triples, np.ndarray):
        if triples.dtype != TRIPLE_DTYPE or not triples.flags.c_contiguous:
            raise TypeError("triple arrays must be contiguous numpy arrays of TRIPLE_DTYPE")
        return ctypes.c_void_p(triples.ctypes.data), len(triples), triples
    tl = list(triples)
    return ctypes.cast(_triple_array(tl), ctypes.c_void_p), len(tl), tl


class _Term(ctypes.Structure):
    _fields_ = [("contr_ptrn", ctypes.c_void_p), ("triples", ctypes.c_void_p), ("n_triples", ctypes.c_int64),
                ("sign", ctypes.c_int)]


class _FusedEnergy(ctypes.Structure):
    _fields_ = [("n_blocks", ctypes.c_int64), ("blocks", ctypes.c_void_p), ("index_values", ctypes.c_void_p),
                ("den_order", ctypes.c_void_p), ("rank1", ctypes.c_int), ("ext1", ctypes.c_void_p),
                ("e_or_fock", ctypes.c_void_p), ("nsegs", ctypes.c_int), ("seg_sizes", ctypes.c_void_p),
                ("efact", ctypes.c_double)]


class Fused:
    """One or two contraction statements into the same destination blocks in
    one split-precision pass (a4g_fused_*).

    terms: [(ptrn, triples, sign), ...] with triples as for Batch and sign +1
    or -1.  energy=None: run() stores D = sum of sign * L R (beta 1: adds).
    energy=dict(blocks, index_values, ext1, e_or_fock, seg_sizes, efact=1.0,
    den_order=None): run(esum) adds efact * sum D * fl(D / eps) to esum (a
    1-element CUDA float64 tensor) and stores nothing.  variant: the GEMM form
    (0 automatic, 5 one level at a time, 7 all levels at once).
    """

    def __init__(self, drank, lrank, rrank, terms, slices=5, beta=0, energy=None, variant=0):
        tarr, en, keep = self._args(terms, energy)
        opts = _Opts(PREC_OZAKI_BF16, slices, beta, variant, 0, 0)
        h = ctypes.c_void_p(0)
        rc = lib().a4g_fused_create(ctypes.byref(h), _i(drank), _i(lrank), _i(rrank), tarr, _i(len(terms)),
                                    ctypes.byref(en) if en is not None else None, ctypes.byref(opts))
        _check(rc, "a4g_fused_create")
        self._h = h
        self._keep = keep  # the caller's buffers must outlive the step
        self.energy = energy is not None

    def rebind(self, terms, energy=None, stream=None):
        """The same structure on other blocks / index values (a4g_fused_rebind)."""
        tarr, en, keep = self._args(terms, energy)
        rc = lib().a4g_fused_rebind(self._h, tarr, _i(len(terms)), ctypes.byref(en) if en is not None else None,
                                    _stream(stream))
        _check(rc, "a4g_fused_rebind")
        self._keep = keep

    @staticmethod
    def _args(terms, energy):
        keep, tarr = [], (_Term * max(1, len(terms)))()
        for i, (ptrn, triples, sign) in enumerate(terms):
            arr, n, k = _triples_arg(triples)
            pt = _iarr(ptrn)
            keep += [k, arr, pt]
            tarr[i].contr_ptrn = ctypes.cast(pt, ctypes.c_void_p)
            tarr[i].triples = arr
            tarr[i].n_triples = n
            tarr[i].sign = int(sign)
        en = None
        if energy is not None:
            blocks = energy["blocks"]
            bl = (ctypes.c_uint64 * max(1, len(blocks)))(*[_ptr(x) for x in blocks])
            iv = _iarr([int(v) for row in energy["index_values"] for v in row])
            e1, sg = _iarr(energy["ext1"]), _iarr(energy["seg_sizes"])
            do = _iarr(energy["den_order"]) if energy.get("den_order") is not None else None
            keep += [bl, iv, e1, sg, do, energy["e_or_fock"]]
            en = _FusedEnergy(len(blocks), ctypes.cast(bl, ctypes.c_void_p), ctypes.cast(iv, ctypes.c_void_p),
                              ctypes.cast(do, ctypes.c_void_p) if do is not None else None, len(energy["ext1"]),
                              ctypes.cast(e1, ctypes.c_void_p), _ptr(energy["e_or_fock"]),
                              len(energy["seg_sizes"]), ctypes.cast(sg, ctypes.c_void_p),
                              float(energy.get("efact", 1.0)))
        return tarr, en, keep + [tarr, en]

    def run(self, esum=None, stream=None):
        _check(lib().a4g_fused_run(self._h, ctypes.c_void_p(_ptr(esum)), _stream(stream)), "a4g_fused_run")

    def info(self):
        pairs, flops, el, nb = ctypes.c_int64(0), ctypes.c_double(0), ctypes.c_int64(0), ctypes.c_int64(0)
        _check(lib().a4g_fused_info(self._h, ctypes.byref(pairs), ctypes.byref(flops), ctypes.byref(el),
                                    ctypes.byref(nb)), "a4g_fused_info")
        return {"pairs": pairs.value, "flops": flops.value, "elements": el.value, "device_bytes": nb.value,
                "form": int(lib().a4g_fused_form(self._h))}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().a4g_fused_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_cache_clear():
    """Forget every autotuned choice of this process (a4g_tune_cache_clear)."""
    lib().a4g_tune_cache_clear()


def tune_cache_save(path: str):
    _check(lib().a4g_tune_cache_save(str(path).encode()), "a4g_tune_cache_save")


def tune_cache_load(path: str):
    _check(lib().a4g_tune_cache_load(str(path).encode()), "a4g_tune_cache_load")


class Batch:
    """One pardo step: every (D, L, R) block triple of one SIAL contraction
    statement, executed by one call.  Triples with the same D are summed into
    it; a triple whose L or R is None is a zero block and is skipped.

    triples: iterable of (d, l, r, dext, lext, rext) with CUDA tensors (or
    device addresses) and per-block extents.
    """

    def __init__(self, ptrn, drank, lrank, rrank, triples, precision=PREC_FP64, slices=5, beta=0, variant=0,
                 negate=False, pipeline=0):
        arr, n, keep = _triples_arg(triples)
        opts = _Opts(precision, slices, beta, variant, int(bool(negate)), int(pipeline))
        h = ctypes.c_void_p(0)
        rc = lib().a4g_batch_create(ctypes.byref(h), _iarr(ptrn), _i(drank), _i(lrank), _i(rrank), arr,
                                    ctypes.c_int64(n), ctypes.byref(opts))
        _check(rc, "a4g_batch_create")
        self._h = h
        self._keep = keep  # the caller's buffers must outlive the batch

    def run(self, stream=None):
        _check(lib().a4g_batch_run(self._h, _stream(stream)), "a4g_batch_run")

    def rebind(self, triples, stream=None):
        """Point the batch at other blocks of the same shapes and sharing
        (a4g_batch_rebind): triple i replaces triple i of the creation."""
        arr, n, keep = _triples_arg(triples)
        _check(lib().a4g_batch_rebind(self._h, arr, ctypes.c_int64(n), _stream(stream)), "a4g_batch_rebind")
        self._keep = keep

    def hold(self, operand: int, on: bool = True, stream=None):
        """Slice operand 0 (L blocks) or 1 (R blocks) now and reuse its digits
        in later runs (on=True), or release it (a4g_batch_hold)."""
        _check(lib().a4g_batch_hold(self._h, _i(operand), _i(int(bool(on))), _stream(stream)), "a4g_batch_hold")

    def error_bound(self, target: float = 0.0, stream=None):
        """Certified relative Frobenius error bound of the last run, largest
        over the destination blocks (a4g_batch_error_bound); raises
        A4GError (status 8) when target > 0 and the bound exceeds it."""
        out = ctypes.c_double(0.0)
        rc = lib().a4g_batch_error_bound(self._h, ctypes.c_double(target), ctypes.byref(out), _stream(stream))
        if rc == 8:
            err = A4GError(rc, "a4g_batch_error_bound")
            err.bound = out.value
            raise err
        _check(rc, "a4g_batch_error_bound")
        return out.value

    def tuning(self):
        """{"from_cache": bool, "autotune_ms": host ms spent autotuning at creation}."""
        c, ms = ctypes.c_int(0), ctypes.c_float(0)
        _check(lib().a4g_batch_tuning(self._h, ctypes.byref(c), ctypes.byref(ms)), "a4g_batch_tuning")
        return {"from_cache": bool(c.value), "autotune_ms": float(ms.value)}

    def run_graph(self, stream=None):
        _check(lib().a4g_batch_run_graph(self._h, _stream(stream)), "a4g_batch_run_graph")

    def run_timed(self, stream=None):
        _check(lib().a4g_batch_run_timed(self._h, _stream(stream)), "a4g_batch_run_timed")

    PHASES = ("zero_fill", "exponents", "split", "gemm", "recombine")

    def timings(self):
        """Summed ms per phase over the timed runs since the last call."""
        arr = (ctypes.c_float * 5)()
        runs = ctypes.c_int(0)
        _check(lib().a4g_batch_timings(self._h, arr, 5, ctypes.byref(runs)), "a4g_batch_timings")
        return {"runs": runs.value, **{k: float(arr[i]) for i, k in enumerate(self.PHASES)}}

    def info(self):
        pairs, flops, ws = ctypes.c_int64(0), ctypes.c_double(0), ctypes.c_int64(0)
        _check(lib().a4g_batch_info(self._h, ctypes.byref(pairs), ctypes.byref(flops), ctypes.byref(ws)),
               "a4g_batch_info")
        return {"pairs": pairs.value, "flops": flops.value, "device_bytes": ws.value}

    def splits(self):
        """Split-K count in use and the autotuner's {count: score ms}."""
        ns = ctypes.c_int(0)
        cand = (ctypes.c_int * 2)()
        cost = (ctypes.c_float * 2)()
        _check(lib().a4g_batch_splits(self._h, ctypes.byref(ns), cand, cost, 2), "a4g_batch_splits")
        return {"nsplit": ns.value, "tuned_ms": {int(cand[i]): float(cost[i]) for i in range(2) if cand[i] > 0}}

    def launches(self):
        """Library kernels per run and the GEMM launches among them."""
        k, p = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().a4g_batch_launches(self._h, ctypes.byref(k), ctypes.byref(p)), "a4g_batch_launches")
        return {"kernels_per_run": k.value, "gemm_parts": p.value}

    FORMS = {1: "one SM per 128x128 tile", 2: "CTA pair per 256x128 tile", 3: "one SM per 128x256 tile",
             4: "CTA pair per 256x256 tile", 5: "one SM per 128x128 tile, direct FP64 store",
             6: "CTA pair per 256x128 tile, direct FP64 store"}

    def form(self):
        """The tensor-core GEMM form in use and the autotuner's score (ms) per form."""
        f = ctypes.c_int(0)
        n = len(self.FORMS)
        ms = (ctypes.c_float * n)()
        _check(lib().a4g_batch_form(self._h, ctypes.byref(f), ms, n), "a4g_batch_form")
        return {"form": f.value, "name": self.FORMS.get(f.value),
                "tuned_ms": {self.FORMS[i + 1]: float(ms[i]) for i in range(n) if ms[i] >= 0}}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().a4g_batch_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
