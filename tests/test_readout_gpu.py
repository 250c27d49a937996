"""Read-out by post-selection: PartialTraceSelect and PartialTraceSelectRange
(partial_trace.cpp:148-225) against the oracle: the same entries kept in the
same order (keys bit-exact), amplitudes scaled by the returned 1/sqrt(p)
(within 1e-12: the engine sums p in a tree, the reference in order)."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


def _state(dual, rng, n=50000):
    dual.reg("m", U, 10)
    dual.reg("x", U, 3)
    dual.reg("y", ps.Boolean, 1)
    regs = np.stack([rng.integers(0, 1024, n), rng.integers(0, 8, n), rng.integers(0, 2, n)], axis=1)
    _, first = np.unique(regs, axis=0, return_index=True)
    regs = regs[np.sort(first)].astype(np.uint64)
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))


@pytest.mark.parametrize("sel", [{"x": 3, "y": 1}, {"x": 0}, {"y": 0}])
def test_partial_trace_select(dual, sel):
    _state(dual, np.random.default_rng(len(sel)))
    op = ps.PartialTraceSelect(sel)
    f = op(dual.gpu)
    fo = dual.O.apply(dual.ora, op.spec())
    assert f == pytest.approx(fo, rel=1e-14)
    dual.compare(rel=1e-12)
    assert abs(dual.gpu.norm_sq() - 1.0) < 1e-12


def test_partial_trace_select_range_and_empty(dual):
    _state(dual, np.random.default_rng(9))
    op = ps.PartialTraceSelectRange("m", (100, 355))
    f = op(dual.gpu)
    fo = dual.O.apply(dual.ora, op.spec())
    assert f == pytest.approx(fo, rel=1e-14)
    dual.compare(rel=1e-12)
    none = ps.PartialTraceSelect({"m": 1000})
    assert none(dual.gpu) == float("inf") and dual.gpu.size() == 0
    assert dual.O.apply(dual.ora, none.spec()) == float("inf")
    assert ps.PartialTraceSelect({})(dual.gpu) == 0.0
