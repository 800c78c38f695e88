"""Which tcgen05 MMA kinds the sm_103a toolchain accepts (CPU only, compile
step).  The split-precision contraction runs its slices as BF16 on
`tcgen05.mma kind::f16`; an INT8 variant would need `kind::i8`, which ptxas
rejects for sm_103a (GB300) while accepting it for sm_100a.  So the INT8
split variant cannot use this GPU's tensor-core MMA, and the library has
none."""
import os
import shutil
import subprocess

import pytest

PROBE = r"""
#include <cstdint>
__global__ void probe(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int n) {
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i)
      asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                   "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
                   :: "r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(i));
}
"""


def _compile(tmp_path, kind, arch):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / f"probe_{kind}_{arch}.cu"
    src.write_text(PROBE.replace("KIND", kind))
    return subprocess.run([nvcc, "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c", str(src), "-o",
                           str(tmp_path / f"probe_{kind}_{arch}.o")], capture_output=True, text=True)


def test_kind_f16_compiles_for_sm103a(tmp_path):
    r = _compile(tmp_path, "f16", "103a")
    assert r.returncode == 0, r.stderr


def test_kind_i8_rejected_for_sm103a(tmp_path):
    r = _compile(tmp_path, "i8", "103a")
    assert r.returncode != 0
    assert "not supported on .target 'sm_103a'" in r.stderr
    assert _compile(tmp_path, "i8", "100a").returncode == 0  # the kind itself exists (sm_100a)
