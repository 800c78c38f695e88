"""The interpreter-style C++ caller (tests/c_abi/interpreter_calls.cpp) run
against the library on the reference's known-answer cases: contraction
through get_contraction_ptrn_ + tensor_block_contract__, permuted copy
through tensor_block_copy__, tensor_block_add__ -- bit for bit."""
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_interpreter_style_caller_runs_kats(tmp_path):
    from tests import c_abi_helper

    exe = c_abi_helper.build(str(tmp_path))
    cases = tmp_path / "cases.txt"
    c_abi_helper.write_cases(str(cases))
    r = subprocess.run([exe, str(cases)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" ok ") == 4, r.stdout
