"""The oracle's Hadamard_Partial on several positions (no reference test pins
it) against the transform it stands for: the dense state vector with H on
each chosen bit, computed with numpy. One position against the same dense
form, and the bit permutation behind the GPU form against its definition."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from oracle import oracle as O

U = ps.UnsignedInteger


def _dense(regs, amps, widths):
    v = np.zeros(1 << sum(widths), dtype=np.complex128)
    for row, a in zip(regs, amps):
        idx, sh = 0, 0
        for val, w in zip(row, widths):
            idx |= int(val) << sh
            sh += w
        v[idx] += a
    return v


def _h_on_bits(v, bits):
    n = int(np.log2(v.size))
    for b in bits:
        t = v.reshape(-1, 2, 1 << b)
        a0, a1 = t[:, 0, :].copy(), t[:, 1, :].copy()
        t[:, 0, :] = (a0 + a1) / np.sqrt(2)
        t[:, 1, :] = (a0 - a1) / np.sqrt(2)
        v = t.reshape(1 << n)
    return v


@pytest.mark.parametrize("positions", [[1], [0, 2], [1, 2, 3], [0, 1, 2, 3], [3, 0]])
def test_oracle_partial_matches_dense_transform(positions):
    widths = [4, 3]
    q = ps.System.add_register("q", U, 4)
    r = ps.System.add_register("r", U, 3)
    O.add_register(int(U), 4)
    O.add_register(int(U), 3)
    rng = np.random.default_rng(7 + len(positions))
    idx = rng.choice(1 << 7, 40, replace=False)
    regs = np.stack([idx & 15, idx >> 4], axis=1).astype(np.uint64)
    amps = rng.normal(size=40) + 1j * rng.normal(size=40)
    amps /= np.linalg.norm(amps)
    st = O.OracleState()
    st.set(regs, amps)
    O.apply(st, ps.Hadamard_Partial("q", positions).spec())
    got_regs, got_amps = st.get()
    want = _h_on_bits(_dense(regs, amps, widths), sorted(set(positions)))
    got = _dense(got_regs[:, [q, r]], got_amps, widths)
    assert np.max(np.abs(got - want)) < 1e-14
    # every entry kept is above the prune threshold; every dropped one below
    assert np.all(np.abs(got_amps) ** 2 >= 1e-14)
    assert np.count_nonzero(np.abs(want) ** 2 >= 1e-14) == len(got_amps)


def test_oracle_bit_gather_definition():
    ps.System.add_register("q", U, 9)
    O.add_register(int(U), 9)
    vals = np.arange(512, dtype=np.uint64)
    st = O.OracleState()
    st.set(vals[:, None], np.ones(512, dtype=np.complex128) / np.sqrt(512))
    mask = 0b100100110
    O.apply(st, ps.BitGather("q", mask).spec())
    got = st.get()[0][:, 0]
    lo = [b for b in range(9) if mask >> b & 1]
    hi = [b for b in range(9) if not mask >> b & 1]
    order = lo + hi
    want = np.array([sum(((int(v) >> old) & 1) << new for new, old in enumerate(order)) for v in vals], dtype=np.uint64)
    assert np.array_equal(got, want)
    O.apply(st, ps.BitGather("q", mask).spec(True))
    assert np.array_equal(st.get()[0][:, 0], vals)
