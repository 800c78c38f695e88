"""CPU-only checks of the C-ABI library: it builds, loads without touching
CUDA, and exports every entry point that include/aces4_gb300.h declares."""
import ctypes
import os

import pytest

import aces4_gb300
from aces4_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "aces4_gb300.h")


@pytest.fixture(scope="module")
def so():
    path = aces4_gb300.build()
    return ctypes.CDLL(path)


def test_header_symbols_exported(so):
    names = _lib.header_symbols(HEADER)
    # the reference-named drop-ins must all be there
    for must in ["tensor_block_contract__", "get_contraction_ptrn_", "tensor_block_copy__",
                 "tensor_block_add__", "tensor_block_scale__", "tensor_block_init__",
                 "tensor_block_norm2__", "tensor_block_slice__", "tensor_block_insert__",
                 "_gpu_contract", "_gpu_permute", "_gpu_axpy", "energy_denominator_rhf"]:
        assert must in names
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_python_signature_table_matches_header():
    names = set(_lib.header_symbols(HEADER))
    assert names == set(_lib.SIGNATURES), (names ^ set(_lib.SIGNATURES))


def test_host_only_entries_without_gpu(so):
    # integer work that the reference does on the host needs no device
    ierr = ctypes.c_int(-7)
    out = (ctypes.c_int * 8)()
    aces = (ctypes.c_int * 12)(1, 2, 3, 4, 1, 2, 5, 6, 5, 6, 3, 4)
    four = ctypes.c_int(4)
    so.get_contraction_ptrn_(ctypes.byref(four), ctypes.byref(four), ctypes.byref(four), aces, out,
                             ctypes.byref(ierr))
    assert ierr.value == 0 and list(out) == [1, 2, -1, -2, -3, -4, 3, 4]
    so.tensor_size_by_shape_.restype = ctypes.c_longlong
    dims = (ctypes.c_int * 3)(3, 4, 5)
    n = so.tensor_size_by_shape_(ctypes.byref(ctypes.c_int(3)), dims, ctypes.byref(ierr))
    assert n == 60 and ierr.value == 0


def test_library_has_no_oracle_dependency(so):
    # the product never links the CPU oracle
    assert not hasattr(so, "a4o_tensor_block_contract")


def test_interpreter_style_caller_compiles_and_links(tmp_path):
    """A C++ caller that declares the drop-ins exactly as the reference's
    tensor_ops_c_prototypes.h does (scalars by reference) builds and links
    against the library (it runs in the GPU suite)."""
    import shutil

    if not shutil.which("g++"):
        pytest.skip("no g++")
    from tests import c_abi_helper

    exe = c_abi_helper.build(str(tmp_path))
    assert os.path.exists(exe)
    c_abi_helper.write_cases(str(tmp_path / "cases.txt"))
    assert (tmp_path / "cases.txt").stat().st_size > 0


def test_header_compiles_as_c_and_cpp():
    """The ABI header is plain C (a Fortran bind(c) or C host can include it)
    and also compiles as C++."""
    import shutil
    import subprocess

    for comp, lang, std in (("gcc", "c", "-std=c99"), ("g++", "c++", "-std=c++11")):
        if not shutil.which(comp):
            pytest.skip(f"no {comp}")
        r = subprocess.run([comp, "-fsyntax-only", "-Wall", "-Werror", "-x", lang, std, HEADER],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_tune_cache_file_round_trip(so, tmp_path):
    """The tuning cache's text file loads and saves without a GPU; a file of
    another format is rejected with A4G_ERR_ARG and leaves the cache as it was."""
    so.a4g_tune_cache_save.argtypes = [ctypes.c_char_p]
    so.a4g_tune_cache_load.argtypes = [ctypes.c_char_p]
    so.a4g_tune_cache_clear()
    src = tmp_path / "in.txt"
    src.write_text("a4g-tune 1\n"
                   "00000000deadbeef 3 19 19 38 16.9 17.2 39.3 39.9 19.8 16.9 -1 -1\n"
                   "0123456789abcdef 4 1 0 0 -1 -1 53 54 29.4 24.4 25 25.3\n")
    assert so.a4g_tune_cache_load(str(src).encode()) == 0
    out = tmp_path / "out.txt"
    assert so.a4g_tune_cache_save(str(out).encode()) == 0
    lines = out.read_text().splitlines()
    assert lines[0] == "a4g-tune 1"
    recs = sorted(l.split()[:3] for l in lines[1:])
    assert recs == [["00000000deadbeef", "3", "19"], ["0123456789abcdef", "4", "1"]]
    bad = tmp_path / "bad.txt"
    bad.write_text("something else\n")
    assert so.a4g_tune_cache_load(str(bad).encode()) == 1
    torn = tmp_path / "torn.txt"
    torn.write_text("a4g-tune 1\n00000000deadbeef 3 nineteen\n")
    assert so.a4g_tune_cache_load(str(torn).encode()) == 1
    so.a4g_tune_cache_clear()
    assert so.a4g_tune_cache_save(str(out).encode()) == 0
    assert out.read_text().splitlines() == ["a4g-tune 1"]


def _lib_ptrn(so, dr, lr, rr, aces):
    ierr = ctypes.c_int(-7)
    out = (ctypes.c_int * max(1, lr + rr))()
    arr = (ctypes.c_int * max(1, len(aces)))(*aces)
    so.get_contraction_ptrn_(ctypes.byref(ctypes.c_int(dr)), ctypes.byref(ctypes.c_int(lr)),
                             ctypes.byref(ctypes.c_int(rr)), arr, out, ctypes.byref(ierr))
    return ierr.value, list(out)[: lr + rr]


def test_pattern_golden_and_oracle_agree_with_library(so):
    """The library's get_contraction_ptrn_ (a transliteration of the
    reference's sort-based routine) against the fixtures and, on 20000 random
    label lists of ranks 0..6, against the oracle's counting restatement."""
    import random

    from oracle import oracle
    from tests import kat

    for c in kat.cases():
        if c["kind"] != "pattern" or min(c["drank"], c["lrank"], c["rrank"]) < 0:
            continue
        ierr, my = _lib_ptrn(so, c["drank"], c["lrank"], c["rrank"], c["aces"])
        assert ierr == c["ierr"], c["name"]
        if ierr == 0:
            assert my == c["my_ptrn"], c["name"]
    rng = random.Random(1142)
    seen = set()
    for _ in range(20000):
        dr, lr, rr = rng.randint(0, 6), rng.randint(0, 6), rng.randint(0, 6)
        if (dr + lr + rr) % 2 and rng.random() < 0.8:
            rr = max(0, rr - 1) if rr else rr + 1
        aces = [rng.randint(1, max(1, (dr + lr + rr) // 2 + rng.randint(0, 2))) for _ in range(dr + lr + rr)]
        i1, m1 = _lib_ptrn(so, dr, lr, rr, aces)
        i2, m2 = oracle.get_contraction_ptrn(dr, lr, rr, aces)
        assert i1 == i2, (dr, lr, rr, aces, i1, i2)
        if i1 == 0:
            assert m1 == m2[: lr + rr], (dr, lr, rr, aces)
        seen.add(i1)
    assert seen >= {0, 2, 3, 4, 5, 6}
