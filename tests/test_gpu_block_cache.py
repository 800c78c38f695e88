"""Device-resident blocks behind the drop-in entry points (a4g_blocks_*), the
GPU side of the reference's BlockManager lazy copies
(src/sip/dynamic_data/block_manager.cpp:291-446).

An interpreter-style sequence on host blocks (contract, permute, add, scale,
norm) with the cache attached must copy each operand to the device once
(resident operands cross the host link no more), keep results on the device
until the host asks for them, and give the same bits as the same sequence
without the cache (where every call copies in and out) and match the
oracle.  Eviction under a small capacity writes newer device copies back.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def a4():
    import aces4_gb300

    aces4_gb300.build()
    aces4_gb300.device.init(0)
    return aces4_gb300


def test_resident_operands_do_not_cross_the_link(a4):
    ref = a4.ref
    rng = np.random.default_rng(3)
    le, re, de = [12, 12, 12, 12], [12, 12, 5, 5], [12, 12, 5, 5]
    d, l, r = [1, 2, 3, 4], [1, 2, 5, 6], [5, 6, 3, 4]
    ierr, ptrn = ref.get_contraction_ptrn(4, 4, 4, d + l + r)
    assert ierr == 0
    V = rng.uniform(-1, 1, int(np.prod(le))) / 48
    T = rng.normal(0, 0.1, int(np.prod(re)))
    n = int(np.prod(de))

    def run(cache):
        R, P, Q = np.zeros(n), np.zeros(n), np.zeros(n)
        stats = []
        if cache:
            cache.attach()
        assert ref.tensor_block_contract(ptrn, V, le, T, re, R, de) == 0
        stats.append(cache.stats() if cache else None)
        ierr, _ = ref.tensor_block_copy(de, [2, 1, 3, 4], R, out=P)
        assert ierr == 0
        stats.append(cache.stats() if cache else None)
        assert ref.tensor_block_add(de, P, P, 0.5) == 0  # P += 0.5 P (operand and result alike)
        assert ref.tensor_block_scale(P, de, 3.0) == 0
        nrm = ref.tensor_block_norm2(P, de)
        stats.append(cache.stats() if cache else None)
        assert ref.tensor_block_contract(ptrn, V, le, T, re, Q, de) == 0  # V, T resident: no copy in
        stats.append(cache.stats() if cache else None)
        if cache:
            cache.detach()
        return R, P, Q, nrm, stats

    R0, P0, Q0, n0, _ = run(None)
    c = ref.BlockCache(1 << 30)
    R1, P1, Q1, n1, st = run(c)
    blk = n * 8
    vt = V.nbytes + T.nbytes
    assert st[0]["h2d_bytes"] == vt and st[0]["d2h_bytes"] == 0  # R overwritten on the device: nothing copied
    assert st[1]["h2d_bytes"] == vt  # R resident, P overwritten
    assert st[2]["h2d_bytes"] == vt and st[2]["d2h_bytes"] == 0
    assert st[3]["h2d_bytes"] == vt  # the second contraction reuses V and T on the device
    # results are on the device only until the host asks for them
    assert not np.any(R1) and not np.any(P1)
    c.on_host(R1)
    c.on_host(P1)
    c.on_host(Q1)
    assert c.stats()["d2h_bytes"] == 3 * blk
    np.testing.assert_array_equal(R1, R0)
    np.testing.assert_array_equal(P1, P0)
    np.testing.assert_array_equal(Q1, Q0)
    assert n1 == n0
    want = oracle.contract_blas(ptrn, V, le, T, re, de)
    assert np.linalg.norm(R1 - want) <= 1e-12 * np.linalg.norm(want)
    # the host changes V: marked newer on the host, the next use copies it in
    c.attach()
    c.on_host(V, ref.UPDATE)
    V *= 2.0
    assert ref.tensor_block_contract(ptrn, V, le, T, re, R1, de) == 0
    c.detach()
    assert c.stats()["h2d_bytes"] == vt + V.nbytes
    c.on_host(R1)
    np.testing.assert_array_equal(R1, 2.0 * R0)
    c.close()


def test_eviction_writes_back(a4):
    ref = a4.ref
    rng = np.random.default_rng(4)
    ext = [40, 40, 40]
    n = 40 ** 3
    blocks = [rng.standard_normal(n) for _ in range(6)]
    want = [b * 2.0 for b in blocks]
    c = ref.BlockCache(3 * n * 8)  # room for three blocks
    c.attach()
    for b in blocks:
        assert ref.tensor_block_scale(b, ext, 2.0) == 0
    c.detach()
    s = c.stats()
    assert s["evictions"] == 3 and s["d2h_bytes"] == 3 * n * 8 and s["resident_bytes"] == 3 * n * 8
    for b, w in zip(blocks[:3], want[:3]):
        np.testing.assert_array_equal(b, w)  # evicted: written back
    assert not np.array_equal(blocks[5], want[5])  # still only on the device
    c.flush()
    for b, w in zip(blocks, want):
        np.testing.assert_array_equal(b, w)
    c.close()


def test_block_cache_rejections(a4):
    ref = a4.ref
    x = np.zeros(1000)
    c = ref.BlockCache(1 << 20)
    c.on_device(x[:500])
    with pytest.raises(RuntimeError):  # overlaps a registered block
        c.on_device(x[400:900])
    c.on_device(x[:500], ref.UPDATE)
    c.on_host(x[:500], ref.READ)
    c.forget(x[:500])
    c.on_device(x[400:900])  # no overlap once forgotten
    c.close()
