"""Builds tests/c_abi/interpreter_calls.cpp against the library and writes
its input cases from the reference known-answer fixtures."""
import os
import subprocess

import numpy as np

from tests import kat

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c_abi", "interpreter_calls.cpp")


def build(out_dir):
    import aces4_gb300

    lib = aces4_gb300.build()
    exe = os.path.join(out_dir, "interpreter_calls")
    cmd = ["g++", "-O2", "-std=c++17", SRC, "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _w(f, xs, fmt):
    f.write(f"{len(xs)} " + " ".join(fmt(x) for x in xs) + "\n")


def write_cases(path):
    from oracle import oracle

    with open(path, "w") as f:
        cases = []
        for name in ("contraction_small_test", "contraction_small_test2"):
            c = kat.case(name)
            L = kat.fill(c["l_fill"], kat.size(c["l_ext"]))
            R = kat.fill(c["r_fill"], kat.size(c["r_ext"]))
            cases.append(("contract", c, L, R))
        f.write(f"{len(cases) + 2}\n")
        for _, c, L, R in cases:
            f.write("contract\n")
            for key in ("d_labels", "l_labels", "r_labels", "d_ext", "l_ext", "r_ext"):
                _w(f, c[key], str)
            for arr in (L, R, np.asarray(c["expected"], dtype=np.float64)):
                _w(f, arr, lambda x: repr(float(x)))
        c = kat.case("transpose_tmp")
        S = kat.fill(c["s_fill"], kat.size(c["s_ext"]))
        f.write("copy\n")
        _w(f, c["s_ext"], str)
        _w(f, [1] + kat.perm_from_labels(c["d_labels"], c["s_labels"]), str)
        _w(f, S, lambda x: repr(float(x)))
        _w(f, np.asarray(c["expected"], dtype=np.float64), lambda x: repr(float(x)))
        # d += 1.0 * s on the sum_op operands (the 1e-13 unit-factor rule keeps it a plain add)
        c = kat.case("sum_op")
        A = kat.fill(c["a_fill"], kat.size(c["ext"]))
        C = kat.fill(c["c_fill"], kat.size(c["ext"]))
        want = A.copy()
        assert oracle.tensor_block_add(c["ext"], want, C, 1.0) == 0
        f.write("add\n")
        _w(f, c["ext"], str)
        f.write("1.0\n")
        for arr in (A, C, want):
            _w(f, arr, lambda x: repr(float(x)))
