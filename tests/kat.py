"""Shared helpers for the reference known-answer fixtures (tests/golden)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat_reference_tests.json")


def cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


def case(name):
    for c in cases():
        if c["name"] == name:
            return c
    raise KeyError(name)


def fill(spec, n):
    from oracle import oracle

    kind, start = spec
    return oracle.fill_block_cyclic(n, start) if kind == "cyclic" else oracle.fill_block_sequential(n, start)


def perm_from_labels(d_labels, s_labels):
    """permute_rhs_to_lhs (src/sip/worker/interpreter.cpp:2049-2084): source
    dimension j goes to destination dimension i where the labels match;
    returned 1-based (O2N, no sign slot)."""
    out = [0] * len(s_labels)
    for i, lab in enumerate(d_labels):
        out[s_labels.index(lab)] = i + 1
    return out


def size(ext):
    return int(np.prod(ext)) if len(ext) else 1
