"""Cached group ranges: a Hadamard on the same bits as the split that produced
the state takes that split's output ranges as its groups (no grouping pass).
Each case runs a split, something or nothing in between, and a second split,
against the oracle (which always groups from scratch), and checks from the
engine's kernel list whether the grouping pass ran."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger
GROUPING_KERNELS = ("hash_insert", "bucket_members", "radix_onesweep", "radix_histogram", "group_stats", "group_small")


def _grouping_ran(fn) -> bool:
    _native.profile_reset()
    _native.profile_enable(True)
    try:
        fn()
    finally:
        _native.profile_enable(False)
    names = _native.profile_read()
    return any(name.startswith(k) for name in names for k in GROUPING_KERNELS)


def _start(dual, rng, n, n_entries):
    dual.reg("a", U, 14)
    dual.reg("b", U, 10)
    dual.reg("c", U, 6)
    # distinct (b, c) per entry: every first-split group is a singleton
    i = np.arange(n_entries)
    regs = np.stack([rng.integers(0, 1 << 14, n_entries), i % (1 << 10), i // (1 << 10)], axis=1)
    amps = rng.normal(size=n_entries) + 1j * rng.normal(size=n_entries)
    amps /= np.linalg.norm(amps)
    dual.start(regs.astype(np.uint64), amps)


@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
@pytest.mark.parametrize("sizing", ["auto", "exact"])
@pytest.mark.parametrize("n", [12, 5])
def test_split_then_merge_reuses_ranges(dual, n, sizing, arith):
    ps.set_fwht_arithmetic(arith)
    ps.set_output_sizing(sizing)
    dual.relaxed = arith == "exact-sum"
    rng = np.random.default_rng(7 + n)
    _start(dual, rng, n, 1000 if n == 12 else 20000)
    H = ps.Hadamard_Int("a", n)
    assert _grouping_ran(lambda: dual.apply(H))
    dual.compare(exact_amp=True)
    assert not _grouping_ran(lambda: dual.apply(H))  # merge back on the cached ranges
    dual.compare(exact_amp=True)
    # and once more: the merge output's ranges serve the next split too
    assert not _grouping_ran(lambda: dual.apply(H))
    dual.compare(exact_amp=True)
    ps.set_output_sizing("auto")


@pytest.mark.parametrize("between,reuse", [
    ("phase", True),        # amplitudes only
    ("x_b", False),         # key bits outside the target change
    ("x_a_low", False),     # key word written (conservatively dropped)
    ("clear_zero", False),  # entries move
    ("other_target", False),
    ("conditioned", False),
])
def test_ranges_dropped_when_keys_change(dual, between, reuse):
    rng = np.random.default_rng(99)
    _start(dual, rng, 6, 5000)
    H = ps.Hadamard_Int("a", 6)
    dual.apply(H)
    second = H
    if between == "phase":
        dual.apply(ps.Phase_Bool("a", 1, 0.3))
    elif between == "x_b":
        dual.apply(ps.Add_ConstUInt_InPlace("b", 3))
    elif between == "x_a_low":
        dual.apply(ps.X_Bool("a", 0))
    elif between == "clear_zero":
        dual.apply(ps.ClearZero(1e-9))
    elif between == "other_target":
        second = ps.Hadamard_Int("c", 6)
    elif between == "conditioned":
        second = ps.Hadamard_Int("a", 6).conditioned_by_bit("c", 0)
    assert _grouping_ran(lambda: dual.apply(second)) == (not reuse)
    dual.compare(exact_amp=True)


def test_upload_drops_ranges(dual):
    rng = np.random.default_rng(5)
    _start(dual, rng, 6, 2000)
    H = ps.Hadamard_Int("a", 6)
    dual.apply(H)
    regs, amps = dual.gpu.download()
    dual.start(regs[:, : len(ps.System.active_ids())], amps)  # same content, re-uploaded
    assert _grouping_ran(lambda: dual.apply(H))
    dual.compare(exact_amp=True)
