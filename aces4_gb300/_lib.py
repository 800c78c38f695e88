"""Loader of the in-tree C-ABI library (fails loudly when it is missing)."""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libaces4gb300.so")
_lib = None

c_int_p = ctypes.POINTER(ctypes.c_int)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_void_p = ctypes.c_void_p


def build(verbose: bool = False) -> str:
    from . import buildlib as _b

    return _b.build(verbose=verbose)


# (name, restype, argtypes) of every exported entry point; argtypes None means
# "plain ctypes conversion" for the by-pointer Fortran-style drop-ins.
SIGNATURES = {
    # tensor_ops_c_prototypes.h drop-ins
    "tensor_size_by_shape_": (ctypes.c_longlong, None),
    "get_contraction_ptrn_": (None, None),
    "tensor_block_init__": (None, None),
    "tensor_block_scale__": (None, None),
    "tensor_block_norm2__": (ctypes.c_double, None),
    "tensor_block_slice__": (None, None),
    "tensor_block_insert__": (None, None),
    "tensor_block_add__": (None, None),
    "tensor_block_copy__": (None, None),
    "tensor_block_contract__": (None, None),
    # gpu_super_instructions.h drop-ins
    "_init_gpu": (None, None),
    "_gpu_axpy": (None, [c_void_p, c_void_p, ctypes.c_double, ctypes.c_int]),
    "_gpu_double_memset": (None, [c_void_p, ctypes.c_double, ctypes.c_int]),
    "_gpu_selfmultiply": (None, [c_void_p, ctypes.c_double, ctypes.c_int]),
    "_gpu_contract": (None, None),
    "_gpu_permute": (None, None),
    "_gpu_host_to_device": (None, [c_void_p, c_void_p, ctypes.c_int]),
    "_gpu_allocate": (c_void_p, [ctypes.c_int]),
    "_gpu_device_to_host": (None, [c_void_p, c_void_p, ctypes.c_int]),
    "_gpu_device_to_device": (None, [c_void_p, c_void_p, ctypes.c_int]),
    "_gpu_free": (None, [c_void_p]),
    # super instruction
    "energy_denominator_rhf": (None, None),
    "a4g_set_predefined_int_array": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, c_void_p]),
    # a4g device API
    "a4g_last_error": (ctypes.c_char_p, []),
    "a4g_version": (ctypes.c_char_p, []),
    "a4g_init": (ctypes.c_int, [ctypes.c_int]),
    "a4g_sync": (ctypes.c_int, [c_void_p]),
    "a4g_default_stream": (c_void_p, []),
    "a4g_contract": (ctypes.c_int, None),
    "a4g_contract_labels": (ctypes.c_int, None),
    "a4g_permute": (ctypes.c_int, None),
    "a4g_fill": (ctypes.c_int, [c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p]),
    "a4g_scale": (ctypes.c_int, [c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p]),
    "a4g_scale_copy": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p]),
    "a4g_increment": (ctypes.c_int, [c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p]),
    "a4g_add_scaled": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, ctypes.c_double, c_void_p]),
    "a4g_add_sub": (ctypes.c_int, None),
    "a4g_add_sub_noalloc": (ctypes.c_int, None),
    "a4g_norm2": (ctypes.c_int, [c_void_p, ctypes.c_int64, c_double_p, c_void_p]),
    "a4g_slice": (ctypes.c_int, None),
    "a4g_insert": (ctypes.c_int, None),
    "a4g_energy_denominator": (ctypes.c_int, None),
    "a4g_energy_contract": (ctypes.c_int, None),
    "a4g_batch_splits": (ctypes.c_int, None),
    "a4g_selftest_wait_timeout": (ctypes.c_int, None),
    "a4g_selftest_round": (ctypes.c_int, [ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "a4g_selftest_div": (ctypes.c_int, [ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "a4g_clear_error": (None, []),
    "a4g_update_t2": (ctypes.c_int, None),
    "a4g_batch_launches": (ctypes.c_int, None),
    "a4g_batch_create": (ctypes.c_int, None),
    "a4g_batch_run": (ctypes.c_int, [c_void_p, c_void_p]),
    "a4g_batch_run_graph": (ctypes.c_int, [c_void_p, c_void_p]),
    "a4g_batch_run_timed": (ctypes.c_int, [c_void_p, c_void_p]),
    "a4g_batch_timings": (ctypes.c_int, None),
    "a4g_batch_info": (ctypes.c_int, None),
    "a4g_batch_form": (ctypes.c_int, None),
    "a4g_batch_destroy": (None, [c_void_p]),
    "a4g_batch_rebind": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, c_void_p]),
    "a4g_batch_hold": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_int, c_void_p]),
    "a4g_batch_tuning": (ctypes.c_int, None),
    "a4g_batch_error_bound": (ctypes.c_int, [c_void_p, ctypes.c_double, c_double_p, c_void_p]),
    "a4g_tune_cache_clear": (None, []),
    "a4g_blocks_create": (ctypes.c_int, [c_void_p, ctypes.c_size_t]),
    "a4g_blocks_destroy": (None, [c_void_p]),
    "a4g_blocks_on_device": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, ctypes.c_int, c_void_p, c_void_p]),
    "a4g_blocks_on_host": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int, c_void_p]),
    "a4g_blocks_flush": (ctypes.c_int, [c_void_p, c_void_p]),
    "a4g_blocks_forget": (ctypes.c_int, [c_void_p, c_void_p]),
    "a4g_blocks_stats": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "a4g_blocks_attach": (ctypes.c_int, [c_void_p]),
    "a4g_tune_cache_save": (ctypes.c_int, [ctypes.c_char_p]),
    "a4g_tune_cache_load": (ctypes.c_int, [ctypes.c_char_p]),
    "a4g_fused_create": (ctypes.c_int, None),
    "a4g_fused_run": (ctypes.c_int, [c_void_p, c_void_p, c_void_p]),
    "a4g_fused_rebind": (ctypes.c_int, None),
    "a4g_host_direct": (ctypes.c_int, [ctypes.c_int]),
    "a4g_fused_info": (ctypes.c_int, None),
    "a4g_fused_form": (ctypes.c_int, [c_void_p]),
    "a4g_fused_destroy": (None, [c_void_p]),
}


def lib() -> ctypes.CDLL:
    """The loaded library.  Raises if it has not been built: the package has
    no fallback implementation."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"aces4_gb300 CUDA library missing at {LIB_PATH}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            if args is not None:
                fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return (lib().a4g_last_error() or b"").decode()


def header_symbols(header: str) -> list[str]:
    """Function names declared in include/aces4_gb300.h (for the export check)."""
    import re

    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M)
    return sorted({n for n in names if n not in ("defined",) and not n.isupper()})
