"""The grouping autotuner: per shape class the first split runs the sort
grouping, the second the hash grouping, and later ones use the faster; the
state after every split equals the oracle's whichever grouping ran."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


def test_autotuner_decides_and_matches_oracle(dual):
    """(1-bit splits take the partner lookup and no grouping; a 2-bit
    Hadamard is grouped, so it is the autotuned operator here.)"""
    assert ps.get_group_strategy() == "autotune"
    dual.reg("a", U, 6)
    dual.reg("b", U, 16)
    rng = np.random.default_rng(12)
    quarter = 5000  # complete groups on bits 0-1 of a: the Hadamard keeps the entry count (one shape class)
    a0 = rng.integers(0, 64, quarter) & ~3
    b = rng.permutation(1 << 16)[:quarter]
    regs = np.concatenate([np.stack([a0 | j, b], axis=1) for j in range(4)]).astype(np.uint64)
    n = len(regs)
    amps = rng.normal(size=n) + 1j * rng.normal(size=n)
    dual.start(regs, amps / np.linalg.norm(amps))
    ran = []
    for i in range(4):
        _native.profile_reset()
        _native.profile_enable(True)
        dual.apply(ps.Hadamard_Int("a", 2))
        _native.profile_enable(False)
        names = _native.profile_read()
        ran.append("sort" if any(k.startswith("radix") or k == "group_heads" for k in names) else "hash")
        dual.compare()
        dual.apply(ps.Add_ConstUInt_InPlace("b", 1))  # key change: no cached ranges
    assert ran[0] == "sort" and ran[1] == "hash"
    assert ran[2] == ran[3]
    classes, decided = ps.autotune_classes()
    assert classes >= 1 and decided >= 1
