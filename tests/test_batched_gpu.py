"""Batched trajectories on the GPU vs the CPU oracle: a Hadamard whose digit
count each entry reads from a width register (one pass over many trajectories
of different widths), and per-trajectory Pauli X/Z noise inside the fused
elementwise kernel. The oracle runs the reference's own composition of the
batched Hadamard: Hadamard_Int(reg, h).conditioned_by_value(width_reg, h) for
every h (hadamard.cpp:18-132 with the condition test of
global_macros.h:104-284). Keys and amplitudes are compared bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


def batched_state(rng, n_traj, maxd, a_bits=10, b_bits=6, zero_width=True):
    """Trajectories t with widths w_t in [0 or 1, maxd]; per (t, b) a fixed
    high part of `a` and a random subset of the 2^w_t low values."""
    rows = []
    lo_w = 0 if zero_width else 1
    widths = rng.integers(lo_w, maxd + 1, n_traj)
    for t in range(n_traj):
        h = int(widths[t])
        for bval in rng.choice(1 << b_bits, int(rng.integers(1, 4)), replace=False):
            high = int(rng.integers(0, 1 << (a_bits - h)))
            k = int(rng.integers(1, (1 << h) + 1))
            for lo in rng.choice(1 << h, k, replace=False):
                rows.append((t, h, (high << h) | int(lo), int(bval)))
    regs = np.array(rows, dtype=np.uint64)
    amps = rng.normal(size=len(rows)) + 1j * rng.normal(size=len(rows))
    amps /= np.linalg.norm(amps)
    return regs, amps


@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
@pytest.mark.parametrize("maxd", [1, 3, 8])
def test_hadamard_int_batched(dual, maxd, arith):
    ps.set_fwht_arithmetic(arith)
    dual.relaxed = arith == "exact-sum"
    dual.reg("t", U, 10)
    dual.reg("w", U, 4)
    dual.reg("a", U, 10)
    dual.reg("b", U, 6)
    rng = np.random.default_rng(400 + maxd)
    regs, amps = batched_state(rng, 300, maxd)
    dual.start(regs, amps)
    op = ps.Hadamard_Int_Batched("a", "w", maxd)
    dual.apply(op)
    dual.compare(exact_amp=True)
    from sparqsim_gb300 import _native
    _native.profile_reset()
    _native.profile_enable(True)
    dual.apply(op)  # H.H merges every trajectory back, on the first split's cached group ranges
    _native.profile_enable(False)
    names = _native.profile_read()
    assert "hash_insert" not in names and "group_small" not in names
    dual.compare(exact_amp=True)


def test_hadamard_int_batched_conditioned(dual):
    dual.reg("t", U, 10)
    dual.reg("w", U, 4)
    dual.reg("a", U, 10)
    dual.reg("b", U, 6)
    rng = np.random.default_rng(410)
    regs, amps = batched_state(rng, 200, 5)
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Int_Batched("a", "w", 5).conditioned_by_bit("b", 0))
    dual.compare(exact_amp=True)


def test_hadamard_int_batched_rejects_wide_entries(dual):
    dual.reg("t", U, 4)
    dual.reg("w", U, 4)
    dual.reg("a", U, 10)
    regs = np.array([[0, 2, 1], [1, 5, 3]], dtype=np.uint64)
    amps = np.array([0.6, 0.8], dtype=np.complex128)
    dual.start(regs, amps)
    with pytest.raises(ps.SparQInvalid, match="max_digits"):
        ps.Hadamard_Int_Batched("a", "w", 3)(dual.gpu)
    with pytest.raises(ps.SparQInvalid):
        ps.Hadamard_Int_Batched("a", "w", 9)(dual.gpu)


def _noise_masks(rng, n_traj, widths, p):
    """Seeded Pauli X/Z masks: each register bit flips with probability p."""
    m = np.zeros((n_traj, 6), dtype=np.uint64)
    for j, w in enumerate(widths * 2):
        bits = rng.random((n_traj, w)) < p
        m[:, j] = (bits.astype(np.uint64) << np.arange(w, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
    return m


@pytest.mark.parametrize("p", [1e-3, 0.2])
def test_pauli_noise(dual, p):
    dual.reg("t", U, 13)  # trajectory ids past the table's 4096 are left alone
    dual.reg("a", U, 16)
    dual.reg("b", U, 16)
    dual.reg("c", U, 16)
    rng = np.random.default_rng(int(p * 1e4))
    n_traj = 4096
    masks = _noise_masks(rng, n_traj, [16, 16, 16], p)
    masks[0] = [1, 2, 3, 1, 2, 3]
    table = ps.NoiseTable(masks)
    dual.O.register_qram(table.table)
    n = 20000
    regs = np.stack([rng.integers(0, n_traj + 50, n)] + [rng.integers(0, 1 << 16, n) for _ in range(3)], axis=1)
    regs[:, 1] = np.arange(n)  # distinct keys
    amps = rng.normal(size=n) + 1j * rng.normal(size=n)
    dual.start(regs.astype(np.uint64), amps)
    dual.apply(ps.PauliNoise("t", ["a", "b", "c"], table))
    dual.compare(exact_amp=True)
    # fused with arithmetic, conditioned
    op = ps.Fused([ps.Add_UInt_UInt_InPlace("a", "b"),
                   ps.PauliNoise("t", ["a", "b", "c"], table).conditioned_by_bit("c", 3)])
    dual.apply(op)
    dual.compare(exact_amp=True)


def test_pauli_noise_rejects_wide_masks(dual):
    dual.reg("t", U, 4)
    dual.reg("a", U, 8)
    table = ps.NoiseTable(np.array([[1 << 9, 0, 0, 0, 0, 0]], dtype=np.uint64))
    with pytest.raises(ps.SparQInvalid):
        ps.PauliNoise("t", ["a", "a", "a"], table)
