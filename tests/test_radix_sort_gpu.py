"""Sort grouping at sizes where the onesweep radix sort runs hundreds of
2048-key tiles, against the oracle: 32-bit and 64-bit sort keys, every digit
pass live, ragged last tiles, and keys concentrated in a few digits (long
equal-digit runs inside a tile). SPARQ_RADIX_ITEMS=16, SPARQ_RADIX_RANK=1 and
SPARQ_RADIX_MODE=1 run the same cases on the 4096-key tiles, the atomic-OR
ranking and the reduce-then-scan passes."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


@pytest.fixture
def sort_grouping():
    ps.set_group_strategy("sort")
    yield
    ps.set_group_strategy("autotune")


def _unique_rows(rng, n, widths, skew=False):
    cols = []
    for w in widths:
        if skew and w > 8:
            # most keys share their high bits: few digits per pass above the lowest
            c = rng.integers(0, 1 << 8, n, dtype=np.uint64) | (rng.integers(0, 3, n, dtype=np.uint64) << np.uint64(w - 2))
        else:
            c = rng.integers(0, 1 << w, n, dtype=np.uint64) if w < 64 else rng.integers(0, 2 ** 63, n, dtype=np.uint64)
        cols.append(c)
    regs = np.unique(np.stack(cols, axis=1), axis=0)
    return regs[rng.permutation(len(regs))]


@pytest.mark.parametrize("n, widths, skew", [
    (40_001, [1, 20, 8], False),     # 28 key bits: 32-bit keys
    (300_007, [1, 22, 9], False),    # 31 key bits: 32-bit keys, 4 passes
    (300_007, [1, 30, 20], True),    # skewed digits
    (700_001, [1, 40, 22], False),   # 62 key bits: 64-bit keys, 8 passes
])
def test_sort_grouping_vs_oracle(dual, sort_grouping, n, widths, skew):
    for name, w in zip(("q", "r", "c"), widths):
        dual.reg(name, ps.Boolean if w == 1 else U, w)
    rng = np.random.default_rng(n + widths[1])
    regs = _unique_rows(rng, n, widths, skew)
    # pair the first half with partners that differ only in q, so that the
    # split has two-member groups as well as singletons
    half = len(regs) // 2
    partners = regs[:half].copy()
    partners[:, 0] ^= np.uint64(1)
    regs = np.unique(np.concatenate([regs, partners]), axis=0)
    regs = regs[rng.permutation(len(regs))]
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))
    dual.apply(ps.Hadamard_Bool("q"))
    dual.compare(exact_amp=True)
    dual.apply(ps.Hadamard_Bool("q").conditioned_by_bit("c", 1))
    dual.compare(exact_amp=True)
