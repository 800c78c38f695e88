"""aces4_gb300: GB300 (sm_103a) implementation of the ACES4 SIP block-contraction path.

The product is the C-ABI shared library ``aces4_gb300/_build/libaces4gb300.so``
(declared in ``include/aces4_gb300.h``).  This package is a thin Python mirror
of the reference's operator interface on top of it:

* ``ref``     — the reference-named drop-in entry points on HOST numpy buffers
                (``tensor_block_contract__`` and friends, same ierr values);
* ``device``  — the device-resident ``a4g_*`` API on CUDA buffers (torch
                tensors or raw device pointers), including the batched
                pardo-step contraction and its split-precision form.

Loading never initialises CUDA.  On a machine with a GPU every call runs the
CUDA kernels; there is no CPU fallback — a missing library raises.
"""
from ._lib import LIB_PATH, build, lib  # noqa: F401
from . import ref, device  # noqa: F401

__all__ = ["lib", "build", "LIB_PATH", "ref", "device"]
