"""QDA walks on the engine: operator-by-operator parity with the CPU oracle
for the first walk steps, the end-to-end fidelity of a small tridiagonal
solve (the reference's own tridiagonal walk test shape:
PySparQ/test/algorithms/test_qda_integration.py:499-600), the pieces the walk
adds (PlusOneAndOverflow, Rot_GeneralStatePrep, Hadamard on more than 12
bits), and the schedule on the CPU."""
from __future__ import annotations

import math

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import qda
from sparqsim_gb300.operators import stateprep_unitary

U = ps.UnsignedInteger


# ------------------------------------------------------------------ CPU
def test_schedule_and_rotation():
    assert qda.schedule_f(0.0, 10.0, 0.5) == pytest.approx(0.0, abs=1e-15)
    assert qda.schedule_f(1.0, 10.0, 0.5) == pytest.approx(1.0, abs=1e-12)
    assert qda.schedule_f(0.3, 1.0, 0.5) == 0.3
    vals = [qda.schedule_f(s, 20.0, 1.3) for s in np.linspace(0, 1, 50)]
    assert all(b >= a - 1e-15 for a, b in zip(vals, vals[1:]))
    for f in (0.0, 0.2, 0.7, 1.0):
        r = np.array(qda.rotation_R(f)).reshape(2, 2)
        assert np.allclose(r @ r.conj().T, np.eye(2), atol=1e-14)


def test_stateprep_unitary():
    rng = np.random.default_rng(4)
    for n in (2, 4, 8, 16):
        t = rng.normal(size=n) + 1j * rng.normal(size=n)
        u = stateprep_unitary(t)
        assert np.allclose(u.conj().T @ u, np.eye(n), atol=1e-13)
        assert np.allclose(u[:, 0], t / np.linalg.norm(t), atol=1e-13)
    u = stateprep_unitary([0.0, 1.0, 0.0, 0.0])  # zero first amplitude
    assert np.allclose(u[:, 0], [0, 1, 0, 0], atol=1e-15)


# ------------------------------------------------------------------ GPU
class DualRunner:
    """Drives the GPU state and the oracle side by side."""

    def __init__(self, dual):
        self.dual = dual
        self.state = dual.gpu

    def op(self, o, dag=False):
        self.dual.apply(o, dag)

    def split(self, first, name, size):
        return self.dual.split(first, name, size)

    def combine(self, first, second):
        self.dual.combine(first, second)


@pytest.mark.gpu
def test_plus_one_and_overflow(dual):
    dual.reg("m", U, 3)
    dual.reg("o", ps.Boolean, 1)
    dual.reg("c", U, 2)
    regs = np.array([[m, o, c] for m in range(8) for o in range(2) for c in range(4)], dtype=np.uint64)
    rng = np.random.default_rng(1)
    dual.start(regs, rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs)))
    op = ps.PlusOneAndOverflow("m", "o")
    dual.apply(op)
    dual.compare(exact_amp=True)
    dual.apply(op.conditioned_by_value("c", 2), dag=True)
    dual.compare(exact_amp=True)
    dual.apply(ps.PlusOneAndOverflow("m", "o"), dag=True)
    dual.compare(exact_amp=True)


@pytest.mark.gpu
def test_rot_general_state_prep(dual):
    dual.reg("a", U, 2)
    dual.reg("b", U, 5)
    dual.start()
    vec = [0.5, 0.1 + 0.2j, -0.3, 0.7j]
    op = ps.Rot_GeneralStatePrep("a", vec)
    dual.apply(op)
    dual.compare(exact_amp=True)
    regs, amps = dual.gpu.download()
    got = np.zeros(4, dtype=np.complex128)
    got[regs[:, 0].astype(int)] = amps
    v = np.array(vec) / np.linalg.norm(vec)
    assert np.allclose(got, v, atol=1e-14)
    dual.apply(op, dag=True)
    dual.compare(exact_amp=True)


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
@pytest.mark.parametrize("width", [13, 16])
def test_hadamard_wider_than_12(dual, width, arith):
    """Passes of up to 12 bits: within 1e-12 of the oracle's single pass."""
    ps.set_fwht_arithmetic(arith)
    dual.relaxed = True
    dual.reg("m", U, width)
    dual.reg("c", U, 3)
    rng = np.random.default_rng(width)
    n = 300
    regs = np.stack([rng.integers(0, 1 << width, n), rng.integers(0, 8, n)], axis=1).astype(np.uint64)
    _, idx = np.unique(regs, axis=0, return_index=True)
    regs = regs[np.sort(idx)]
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))
    dual.apply(ps.Hadamard_Int_Full("m"))
    dual.compare(exact_amp=True)


@pytest.mark.gpu
@pytest.mark.parametrize("beta", [0.7, -0.7])
def test_walk_parity_with_oracle(dual, beta):
    """The first walk steps, every operator applied to both sides."""
    n_bits = 3
    for name in qda.REGS:
        width = n_bits if name == "main_reg" else 4 if name == "anc_UA" else 1
        dual.reg(name, U if name in ("main_reg", "anc_UA") else ps.Boolean, width)
    dual.start()
    run = DualRunner(dual)
    run.op(ps.Hadamard_Int_Full("main_reg"))
    dual.compare(exact_amp=True)
    qda.walk_sequence(run, n_bits, 1.0, beta, kappa=5.0, p=0.5, steps=40, first=0, clear_zero=ps.ClearZero())
    dual.compare(exact_amp=True)
    assert dual.gpu.size() > 8


@pytest.mark.gpu
def test_tridiagonal_solve_fidelity():
    """alpha = beta = 1 on 2 qubits, p = 0.5, step_rate 0.2 (as the reference's
    tridiagonal walk test): the anc_1 = 1 sector holds A^-1 b."""
    x, prob, fid, kappa, steps = qda.solve_tridiagonal(2, 1.0, 1.0, p=0.5, step_rate=0.2)
    assert steps > 1000
    assert prob > 0.99, prob
    assert fid > 0.999, fid
