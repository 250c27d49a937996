"""Bounded device waits: a wait that runs out gives up, raises the device
error word and lets its block finish, and the host reports
SQ_ERR_DEVICE_TIMEOUT; the library stays usable afterwards. The wait is made
to run out on purpose by a look-back whose predecessor tile is never
published (sq_selftest_wait_timeout), with a short poll limit, so that no
kernel waits longer than a fraction of a millisecond."""
from __future__ import annotations

from ctypes import byref, c_uint32

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native

pytestmark = pytest.mark.gpu
U = ps.UnsignedInteger


def _limit():
    v = c_uint32()
    _native.call("sq_get_wait_limit", byref(v))
    return v.value


@pytest.mark.parametrize("polls", [1, 1000, 1 << 16])
def test_lookback_wait_runs_out_and_is_reported(dual, polls):
    rc = _native.lib().sq_selftest_wait_timeout(polls)
    assert rc == _native.SQ_ERR_DEVICE_TIMEOUT, _native.lib().sq_last_error()
    assert b"bounded" in _native.lib().sq_last_error()
    assert _limit() == 0  # the default limit is back
    # the error word was cleared and the context still works: a split and a
    # prune across many look-back tiles, against the oracle
    dual.reg("a", U, 6)
    dual.reg("b", U, 20)
    rng = np.random.default_rng(polls)
    pick = rng.choice(1 << 26, 50_000, replace=False)
    regs = np.stack([pick & 63, pick >> 6], axis=1).astype(np.uint64)
    amps = rng.normal(size=50_000) + 1j * rng.normal(size=50_000)
    dual.start(regs, amps / np.linalg.norm(amps))
    dual.apply(ps.Hadamard_Int("a", 6))
    dual.apply(ps.ClearZero(1e-9))
    dual.compare(exact_amp=True)
    ps.synchronize()


def test_wait_limit_knob_and_invalid_polls():
    try:
        _native.call("sq_set_wait_limit", 1 << 18)
        assert _limit() == 1 << 18
        st = ps.SparseState()
        ps.System.add_register("a", U, 16)
        st.upload(np.arange(1 << 16, dtype=np.uint64)[:, None], np.full(1 << 16, 2.0 ** -8, dtype=np.complex128))
        ps.ClearZero()(st)  # 32 look-back tiles, far inside the limit
        assert st.size() == 1 << 16
    finally:
        _native.call("sq_set_wait_limit", 0)
    assert _limit() == 0
    assert _native.lib().sq_selftest_wait_timeout(0) == _native.SQ_ERR_INVALID
