"""The restated oracle (built on every machine) against the committed golden
fixtures generated from the reference's own kernels."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from tests.ref_cases import CASES, run_case
import os

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_cases.npz"))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def check_against_golden(name, snaps):
    kinds = list(GOLD[name + "/kinds"])
    ns = list(GOLD[name + "/n"])
    shas = list(GOLD[name + "/sha"])
    assert [s[0] for s in snaps] == kinds
    for s, n, h in zip(snaps, ns, shas):
        if s[0] in ("init", "step", "seed"):
            assert s[1] == n, s[0]
            assert digest(s[2]) == h, s[0]
        else:
            assert digest(s[1]) == h, s[0]


@pytest.mark.parametrize("name", sorted(CASES))
def test_restated_oracle_matches_golden(name):
    check_against_golden(name, run_case(name, lambda v, d: O.RefOracle(v, d)))
