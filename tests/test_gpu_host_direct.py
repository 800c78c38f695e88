"""Drop-ins on host blocks with the kernels running on the host memory in
place (the GPU reads and writes pageable host memory through the host's page
tables) against the same calls with the blocks staged through device memory:
the results must be the same bits, including a transpose whose output is its
own input (aliased, staged through a device temporary) and a scalar result.
Skipped where the GPU cannot access host memory."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    import aces4_gb300

    aces4_gb300.build()
    if aces4_gb300.ref.host_direct(True) != 0:
        pytest.skip("the GPU cannot access pageable host memory here")
    yield aces4_gb300.ref
    aces4_gb300.ref.host_direct(True)


def _both(ref, fn):
    out = []
    for mode in (True, False):
        assert ref.host_direct(mode) == 0
        out.append(fn())
    ref.host_direct(True)
    return out


def test_contract_in_place_equals_staged(ref):
    rng = np.random.default_rng(3)
    dl, ll, rl = [1, 2, 3, 4], [1, 5, 6, 2], [6, 3, 5, 4]  # ring: both operands permuted
    le, re, de = [24, 20, 31, 20], [31, 27, 20, 20], [24, 20, 27, 20]
    L = rng.uniform(-1, 1, int(np.prod(le)))
    R = rng.normal(0.0, 0.1, int(np.prod(re)))
    ierr, ptrn = ref.get_contraction_ptrn(4, 4, 4, dl + ll + rl)
    assert ierr == 0

    def run():
        D = np.full(int(np.prod(de)), np.nan)
        assert ref.tensor_block_contract(ptrn, L, le, R, re, D, de) == 0
        return D

    a, b = _both(ref, run)
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    ierr, want = oracle.contract_labels(dl, ll, rl, L, le, R, re, de)
    assert np.linalg.norm(a - want) <= 1e-12 * np.linalg.norm(want)

    # full contraction to a scalar (rank-0 destination written in place)
    def run_scalar():
        D = np.full(1, np.nan)
        ierr, p0 = ref.get_contraction_ptrn(0, 4, 4, [1, 2, 3, 4, 1, 2, 3, 4])
        assert ierr == 0
        assert ref.tensor_block_contract(p0, L, le, L, le, D, []) == 0
        return D

    s1, s2 = _both(ref, run_scalar)
    assert s1[0] == s2[0] and abs(s1[0] - float(L @ L)) <= 1e-12 * abs(float(L @ L))


def test_copy_add_norm_in_place_equal_staged(ref):
    rng = np.random.default_rng(4)
    ext = [16, 24, 12]
    x = rng.standard_normal(int(np.prod(ext)))
    y = rng.standard_normal(int(np.prod(ext)))

    def run():
        ierr, t = ref.tensor_block_copy(ext, [2, 3, 1], x.copy())
        assert ierr == 0
        z = x.copy()  # aliased: the output block is the input block
        ierr, z2 = ref.tensor_block_copy(ext, [1, 2, 3], z, out=z)
        assert ierr == 0
        w = y.copy()
        assert ref.tensor_block_add(ext, w, x, 0.5) == 0
        nrm, ierr = ref.tensor_block_norm2(w, ext)
        assert ierr == 0
        return t, z2, w, nrm

    (t1, z1, w1, n1), (t2, z2, w2, n2) = _both(ref, run)
    for a, b in ((t1, t2), (z1, z2), (w1, w2)):
        assert np.array_equal(a.view(np.int64), b.view(np.int64))
    assert n1 == n2
    assert np.array_equal(z1, x)


def test_energy_denominator_in_place_equals_staged(ref):
    rng = np.random.default_rng(5)
    segs = [5, 7, 6]
    norb = sum(segs)
    e = np.concatenate([rng.uniform(-2.0, -0.5, 5), rng.uniform(0.2, 5.0, 13)])
    fock = np.diag(e).ravel(order="F").copy()
    assert ref.set_predefined_int_array("moa_seg_ranges", segs) == 0
    iv, ext = [2, 1, 3, 1], [7, 5, 6, 5]
    t = rng.standard_normal(int(np.prod(ext)))

    def run():
        d = t.copy()
        assert ref.energy_denominator_rhf(iv, ext, d, [norb, norb], fock) == 0
        return d

    a, b = _both(ref, run)
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
