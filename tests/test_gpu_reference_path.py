"""The reference's legacy GPU contraction (gpu_super_instructions.cu:369-586:
its own reorder kernels, compiled from the reference source for sm_103a,
driven by the host steps restated in oracle/ref_gpu.cpp) against the CPU
oracle and against the library's `_gpu_contract` replacement on the same
device blocks: a ladder block pair and a ring pair with both operands
permuted.  FP64 throughout (cuBLAS DGEMM there, DMMA here): 1e-12 relative.
Skipped where the cubin was not built (it needs the reference tree)."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    if not oracle.ref_gpu_available():
        pytest.skip("reference GPU cubin not built (no reference tree)")
    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


@pytest.mark.parametrize("case", ["ladder", "ring"])
def test_reference_gpu_path_matches_oracle_and_library(a4, case):
    import torch

    rng = np.random.default_rng(5 if case == "ladder" else 6)
    if case == "ladder":  # R(a,b,i,j) = V(a,b,c,d) T(c,d,i,j)
        dl, ll, rl = [1, 2, 3, 4], [1, 2, 5, 6], [5, 6, 3, 4]
        le, re, de = [12, 12, 12, 12], [12, 12, 5, 5], [12, 12, 5, 5]
    else:  # R(a,i,b,j) = V(a,k,c,i) T(c,b,k,j)
        dl, ll, rl = [1, 2, 3, 4], [1, 5, 6, 2], [6, 3, 5, 4]
        le, re, de = [24, 20, 31, 20], [31, 27, 20, 20], [24, 20, 27, 20]
    L = rng.uniform(-1, 1, int(np.prod(le)))
    R = rng.normal(0.0, 0.1, int(np.prod(re)))
    ierr, want = oracle.contract_labels(dl, ll, rl, L, le, R, re, de)
    assert ierr == 0
    tl, tr = torch.tensor(L, device="cuda"), torch.tensor(R, device="cuda")
    ty = torch.full((int(np.prod(de)),), float("nan"), dtype=torch.float64, device="cuda")
    oracle.ref_gpu_contract(ty.data_ptr(), de, dl, tl.data_ptr(), le, ll, tr.data_ptr(), re, rl)
    got = ty.cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    tz = torch.full_like(ty, float("nan"))
    a4.device.gpu_contract(tz, de, dl, tl, le, ll, tr, re, rl)
    a4.device.sync()
    assert np.linalg.norm(tz.cpu().numpy() - got) <= 1e-12 * np.linalg.norm(want)
