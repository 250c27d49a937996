"""The asynchronous packed download: it returns the state as it was when the
download was issued, even when the next operation on the same state
rewrites every key (that operation waits for the copy on the device), and it
matches the synchronous download."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu


def _buffers(kind, k, n):
    """Pinned destinations (stored into by the download kernel) or pageable
    ones (copied by the copy engine)."""
    if kind == "pinned":
        import torch
        kt = torch.empty(k * n, dtype=torch.int64, pin_memory=True)
        at = torch.empty(2 * n, dtype=torch.float64, pin_memory=True)
        return (kt, at), kt.data_ptr(), at.data_ptr(), lambda: (kt.numpy().view(np.uint64), at.numpy())
    keys = np.zeros(k * n, dtype=np.uint64)
    amps = np.zeros(2 * n, dtype=np.float64)
    return (keys, amps), keys.ctypes.data, amps.ctypes.data, lambda: (keys, amps)


@pytest.fixture(params=["sm", "copy", "split"])
def engine(request):
    """Pinned destinations stored into by the download kernel, or copied by
    the copy engine."""
    ps.set_download_engine(request.param)
    yield request.param
    ps.set_download_engine("sm")


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
def test_async_download_is_ordered_before_later_writes(kind, engine):
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 20)
    b = ps.System.add_register("b", ps.Boolean, 1)
    st = ps.SparseState()
    ps.Hadamard_Int_Full(a)(st)  # 2^20 entries, 24 MB: the copy outlasts the next kernel
    n = st.size()
    k = ps.System.key_words()
    ref_keys = np.zeros(k * n, dtype=np.uint64)
    ref_amps = np.zeros(2 * n, dtype=np.float64)
    ps._native.call("sq_state_download_packed", st._h, ref_keys.ctypes.data, ref_amps.ctypes.data)
    keep, kp, ap, view = _buffers(kind, k, n)
    st.download_packed_async(kp, ap)
    ps.X_Bool(b, 0)(st)  # sets b in every entry's key
    ps.GlobalPhase(complex(0.0, 1.0))(st)  # rewrites every amplitude
    st.wait()
    keys, amps = view()
    assert np.array_equal(keys, ref_keys)
    assert np.array_equal(amps, ref_amps)
    regs, _ = st.download()
    assert np.all(regs[:, b] == 1)


def test_two_states_alternate(engine):
    """Downloads of two states in flight while both are rewritten."""
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 16)
    sts = [ps.SparseState(), ps.SparseState()]
    outs = []
    for i, s in enumerate(sts):
        ps.Hadamard_Int_Full(a)(s)
        ps.Add_ConstUInt_InPlace(a, i + 1)(s)
        n, k = s.size(), ps.System.key_words()
        keep, kp, ap, view = _buffers("pinned" if i == 0 else "pageable", k, n)
        s.download_packed_async(kp, ap)
        outs.append((keep, view))
    for s in sts:
        ps.Hadamard_Int_Full(a)(s)  # back to one entry: frees and rewrites the buffers
    ps.synchronize()
    for _, view in outs:
        keys, amps = view()
        assert np.array_equal(np.sort(keys & 0xFFFF), np.arange(1 << 16, dtype=np.uint64))
        assert np.allclose(amps[0::2], 1 / 256) and np.all(amps[1::2] == 0)
    assert [s.size() for s in sts] == [1, 1]


def test_download_engine_names():
    with pytest.raises(ValueError):
        ps.set_download_engine("dma")
    with pytest.raises(ps.SparQInvalid):
        ps._native.call("sq_set_download_engine", 7)


def test_upload_packed_from_pinned_memory():
    """Uploads from pinned memory are loaded by the SMs (mapped memory), other
    host memory goes by the copy engine: both give the same state."""
    import torch
    ps.System.clear()
    ps.System.add_register("a", ps.UnsignedInteger, 40)
    ps.System.add_register("b", ps.UnsignedInteger, 40)
    k = ps.System.key_words()
    n = 300_001  # odd: the 8-byte tail of a 16-byte vector copy
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 2 ** 63, k * n, dtype=np.int64)
    amps = rng.normal(size=2 * n)
    kt = torch.from_numpy(keys).pin_memory()
    at = torch.from_numpy(amps).pin_memory()
    outs = []
    for kp, ap in ((kt.data_ptr(), at.data_ptr()), (keys.ctypes.data, amps.ctypes.data)):
        st = ps.SparseState()
        ps._native.call("sq_state_upload_packed", st._h, n, kp, ap)
        rk = np.zeros(k * n, dtype=np.uint64)
        ra = np.zeros(2 * n, dtype=np.float64)
        ps._native.call("sq_state_download_packed", st._h, rk.ctypes.data, ra.ctypes.data)
        outs.append((rk, ra))
    assert np.array_equal(outs[0][0], keys.view(np.uint64)) and np.array_equal(outs[0][1], amps)
    assert np.array_equal(outs[1][0], outs[0][0]) and np.array_equal(outs[1][1], outs[0][1])
