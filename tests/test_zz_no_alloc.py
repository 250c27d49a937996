"""sq_clear_zero_noalloc: ClearZero for callers that may not have the library
allocate device memory (code that owns every device buffer through its own
pool, or loops where an implicit cudaMalloc is not allowed). It must give the
same survivors, in the same order, as the state-level sq_clear_zero, on two
calls in a row (the second call must not see the first call's leftover
scratch). The caller owns every array here: torch allocates the inputs and
outputs, the library allocates nothing for the call.

This file sorts last so that a run stopping at the first failure has already
run every other test."""
from __future__ import annotations

import ctypes
from ctypes import byref, c_uint64, c_void_p

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native

pytestmark = pytest.mark.gpu


def _state(rng, n):
    ps.System.add_register("a", ps.UnsignedInteger, 40)
    ps.System.add_register("b", ps.UnsignedInteger, 40)  # second key word
    regs = np.stack([rng.permutation(1 << 20)[:n] << 20 | np.arange(n), rng.integers(0, 1 << 40, n)], axis=1)
    regs = regs.astype(np.uint64)
    amps = rng.normal(size=n) + 1j * rng.normal(size=n)
    amps[rng.random(n) < 0.35] *= 1e-9  # |a|^2 ~ 1e-18: pruned at eps 1e-14
    amps[rng.random(n) < 0.10] *= 1e-3  # |a|^2 ~ 1e-6: pruned only at the larger eps
    return regs, amps


def _run_noalloc(torch, keys_dev, amps_dev, k, n, eps, check_alloc=True):
    out_keys = [torch.empty(n, dtype=torch.int64, device="cuda") for _ in range(k)]
    out_amps = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    kin = (c_void_p * k)(*keys_dev)
    kout = (c_void_p * k)(*[t.data_ptr() for t in out_keys])
    n_out = c_uint64()
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    allocs0, free0 = _allocations(), torch.cuda.mem_get_info()[0]
    rc = _native.lib().sq_clear_zero_noalloc(kin, c_void_p(amps_dev), k, n, eps, kout, c_void_p(out_amps.data_ptr()),
                                             byref(n_out), c_void_p(stream))
    assert rc == 0, _native.lib().sq_last_error()
    if check_alloc:
        # the promise itself: the call made no device allocation
        assert _allocations() == allocs0
        assert torch.cuda.mem_get_info()[0] == free0
    m = n_out.value
    keys = np.stack([t[:m].cpu().numpy().view(np.uint64) for t in out_keys])
    amps = out_amps[: 2 * m].cpu().numpy()
    return keys, amps


def _allocations():
    c = c_uint64()
    _native.call("sq_device_allocation_count", byref(c))
    return c.value


def _reference_clear_zero(regs, amps, eps):
    st = ps.SparseState()
    st.upload(regs, amps)
    ps.ClearZero(eps)(st)
    k = ps.System.key_words()
    n = st.size()
    keys = np.zeros(k * n, dtype=np.uint64)
    out = np.zeros(2 * n, dtype=np.float64)
    _native.call("sq_state_download_packed", st._h, keys.ctypes.data_as(c_void_p), out.ctypes.data_as(c_void_p))
    return keys.reshape(k, n), out


def test_clear_zero_noalloc_matches_clear_zero_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2026)
    n = 300_000
    regs, amps = _state(rng, n)
    k = ps.System.key_words()
    assert k == 2
    src = ps.SparseState()
    src.upload(regs, amps)
    key_ptrs, amp_ptr = src.device_arrays()
    # The first call on a device is its set-up: it looks up the static array's
    # device address, and CUDA's lazy loading places the library's device code
    # and that array in device memory on first use, so the driver's memory use
    # grows once here (by its allocation granularity, 2 MiB). The library makes
    # no allocation of its own even then.
    _run_noalloc(torch, key_ptrs, amp_ptr, k, n, 1e-14, check_alloc=False)
    # two calls in a row through the C ABI, different thresholds
    for eps in (1e-14, 1e-5):
        got_keys, got_amps = _run_noalloc(torch, key_ptrs, amp_ptr, k, n, eps)
        want_keys, want_amps = _reference_clear_zero(regs, amps, eps)
        assert got_keys.shape == want_keys.shape
        assert np.array_equal(got_keys, want_keys)          # same survivors, same order
        assert np.array_equal(got_amps, want_amps)          # bit-exact amplitudes
        assert 0 < got_keys.shape[1] < n


def test_clear_zero_noalloc_rejects_overlapping_outputs():
    """Blocks write survivors while other blocks still read: an output array
    that overlaps an input is refused before anything runs."""
    torch = pytest.importorskip("torch")
    ps.System.add_register("a", ps.UnsignedInteger, 20)
    n = 10_000
    keys = torch.zeros(2 * n, dtype=torch.int64, device="cuda")
    amps = torch.zeros(4 * n, dtype=torch.float64, device="cuda")
    n_out = c_uint64()
    lib = _native.lib()
    kin = (c_void_p * 1)(keys.data_ptr())
    kout_ok = (c_void_p * 1)(keys.data_ptr() + 8 * n)
    # amplitudes in place
    rc = lib.sq_clear_zero_noalloc(kin, c_void_p(amps.data_ptr()), 1, n, 1e-14, kout_ok, c_void_p(amps.data_ptr()),
                                   byref(n_out), None)
    assert rc == _native.SQ_ERR_INVALID and b"overlaps" in lib.sq_last_error()
    # key words shifted by one entry into the input
    kout_bad = (c_void_p * 1)(keys.data_ptr() + 8)
    rc = lib.sq_clear_zero_noalloc(kin, c_void_p(amps.data_ptr()), 1, n, 1e-14, kout_bad,
                                   c_void_p(amps.data_ptr() + 16 * n), byref(n_out), None)
    assert rc == _native.SQ_ERR_INVALID
    # disjoint arrays are accepted
    rc = lib.sq_clear_zero_noalloc(kin, c_void_p(amps.data_ptr()), 1, n, 1e-14, kout_ok,
                                   c_void_p(amps.data_ptr() + 16 * n), byref(n_out), None)
    assert rc == 0 and n_out.value == 0  # every amplitude is zero


def test_clear_zero_noalloc_rejects_oversize_and_handles_empty():
    lib = _native.lib()
    n_out = c_uint64(123)
    k = 1
    dummy = (c_void_p * 1)(None)
    rc = lib.sq_clear_zero_noalloc(dummy, None, k, (1 << 26) + 1, 1e-14, dummy, None, byref(n_out), None)
    assert rc == _native.SQ_ERR_CAPACITY
    assert b"2^26" in lib.sq_last_error()
    rc = lib.sq_clear_zero_noalloc(dummy, None, k, 0, 1e-14, dummy, None, byref(n_out), None)
    assert rc == 0 and n_out.value == 0
