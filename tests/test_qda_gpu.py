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

    def add_register(self, name, type_, size):
        return self.dual.add_register(name, type_, size)

    def remove_register(self, reg):
        self.dual.remove_register(reg)


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


# ------------------------------------------------------------------ GetOutput and the Poiseuille benchmark
POISSON_ALPHA = 2.2666666666564934
_BENCH_REGS = (("main", U, 3), ("anc_UA", U, 4), ("anc_4", ps.Boolean, 1), ("anc_3", ps.Boolean, 1),
               ("anc_2", ps.Boolean, 1), ("anc_1", ps.Boolean, 1))


def _oracle_output(dual, go):
    from oracle import oracle as O
    return O.get_output(dual.ora, go.zero, go.idx, ps.System.size_of)


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
def test_get_output_along_a_walk(dual, arith):
    """GetOutput on the GPU against the oracle's restatement of
    qda_fundamental.cpp:123-166 after walk steps of the Poisson benchmark
    (n = 8, a 24-step schedule), with ClearZero and Normalize after each step
    as the benchmark driver does; the state is left unchanged by the read-out.
    Vectors within 1e-12 of the largest amplitude, probabilities within
    1e-12 relative. Normalize sums |a|^2 as a tree on the GPU and in order in
    the oracle, so the states agree within 1e-12 rather than bit for bit."""
    ps.set_fwht_arithmetic(arith)
    dual.relaxed = True
    for name, t, w in _BENCH_REGS:
        dual.reg(name, t, w)
    dual.start()
    run = DualRunner(dual)
    enc_b = qda.StatePrepHadamard("main")
    enc_b.apply(run)
    enc_A = qda.BlockEncodingTridiagonal("main", "anc_UA", POISSON_ALPHA, -1.0)
    go = qda.GetOutput("main", "anc_UA", "anc_4", "anc_3", "anc_2", "anc_1")
    steps = 24
    for i in range(steps):
        qda.WalkS(enc_A, enc_b, "main", "anc_UA", "anc_1", "anc_2", "anc_3", "anc_4", i / steps, 16.0,
                  1.3).apply(run)
        run.op(ps.ClearZero(1e-14))
        run.op(ps.Normalize())
        if i % 4 == 3:
            g, gp = go(dual.gpu)
            o, op_ = _oracle_output(dual, go)
            assert g.shape == (32,)
            assert gp == pytest.approx(op_, rel=1e-12, abs=1e-300)
            assert np.max(np.abs(g - o)) <= 1e-12 * max(np.max(np.abs(o)), 1e-300)
            dual.compare(exact_amp=True)


@pytest.mark.gpu
def test_get_output_edges(dual):
    """An already normalised selection is returned as it is (|p - 1| < 1e-14),
    a selection of nothing gives zeros and p = 0, and a register that is
    neither post-selected nor indexed is rejected (two entries could share a
    slot)."""
    dual.reg("m", U, 3)
    dual.reg("a", U, 2)
    dual.reg("c", U, 2)
    regs = np.array([[m, a, c] for m in range(8) for a in range(4) for c in range(4)], dtype=np.uint64)
    rng = np.random.default_rng(11)
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))
    for zero, idx in ((["a"], ["m", "c"]), (["a", "c"], ["m"]), ([], ["m", "a", "c"]), (["m"], ["c", "a"])):
        z = [ps.System.resolve(r) for r in zero]
        ix = [ps.System.resolve(r) for r in idx]
        g, gp = ps.get_output(dual.gpu, z, ix)
        from oracle import oracle as O
        o, op_ = O.get_output(dual.ora, z, ix, ps.System.size_of)
        assert gp == pytest.approx(op_, rel=1e-13)
        assert np.max(np.abs(g - o)) <= 1e-13
    # everything selected: p = 1 within 1e-14, returned unscaled
    g, gp = ps.get_output(dual.gpu, [], ["m", "a", "c"])
    assert abs(gp - 1.0) < 1e-14
    # nothing selected: keep c in [1, 3] first (both sides), then post-select c = 0
    dual.apply(ps.PartialTraceSelectRange("c", (1, 3)))
    dual.compare()
    g, gp = ps.get_output(dual.gpu, ["c"], ["m", "a"])
    assert gp == 0.0 and not np.any(g)
    with pytest.raises(ps.SparQInvalid):
        ps.get_output(dual.gpu, ["a"], ["m"])


def _poiseuille(tmp_path, *argv):
    import json

    from sparqsim_gb300 import poiseuille
    summary = poiseuille.run(poiseuille.parser().parse_args([*argv, "--outdir", str(tmp_path)]))
    rows = np.loadtxt(tmp_path / "residual_curve.csv", delimiter=",", skiprows=1, ndmin=2)
    assert json.loads((tmp_path / "qda_summary.json").read_text())["steps_executed"] == summary["steps_executed"]
    return summary, rows


@pytest.mark.gpu
def test_poiseuille_compressed_schedule_2_16(tmp_path):
    """n = 2^16, the schedule compressed to 40 steps, logged every 10 steps:
    res_dir 2.071000e-02 at all four log points in the reference's runs
    (docs/verification/v1d-qda-linsolver-a800.md:21,133-135), printed to 7
    digits, so within 6e-9."""
    summary, rows = _poiseuille(tmp_path, "--nqubit", "16", "--maxSteps", "40", "--logEvery", "10")
    assert rows.shape == (4, 5)
    assert list(rows[:, 0]) == [10, 20, 30, 40]
    assert np.all(np.abs(rows[:, 1] - 2.071000e-02) <= 6e-9), rows[:, 1]
    assert summary["step_budget"] == 40568 and summary["termination"] == "fixed_step_budget"


@pytest.mark.gpu
def test_poiseuille_dim256_rate_0_1(tmp_path):
    """n = 256, rate 0.1 (3688 steps), kappa 16: final res_dir 3.135e-2,
    fidelity 0.999438 and success probability 0.5969 in the reference's CUDA
    run (docs/verification/v1d-qda-linsolver-a800.md:138-140), with about
    17.5k entries at the peak (:50). res_dir is quoted truncated to four
    digits; the others to the digits printed there."""
    summary, rows = _poiseuille(tmp_path, "--nqubit", "8", "--steprate", "0.1", "--kappa", "16",
                                "--logEvery", "922")
    assert summary["steps_executed"] == 3688
    assert 3.135e-2 <= summary["final_res_dir"] < 3.136e-2, summary
    assert abs(summary["final_fidelity_vs_classical"] - 0.999438) <= 5e-7, summary
    assert abs(summary["final_success_prob"] - 0.5969) <= 5e-5, summary
    assert 17_400 <= summary["max_system_size"] <= 17_600, summary


@pytest.mark.gpu
def test_batched_walk_matches_plain_walks():
    """Two walks of the Poisson benchmark with different step budgets (60 and
    90) run side by side in one state, told apart by a 1-bit instance
    register, against the same walks run alone: per instance the same basis
    entries, and amplitudes (times sqrt 2, the instance superposition's
    factor) within 1e-12 after 12 steps. The batched run prunes at half the
    threshold, where each walk's |a|^2 is half its own."""
    n_bits, budgets, steps, eps0 = 4, [60, 90], 12, 1e-14
    alpha, kappa, p = POISSON_ALPHA, 16.0, 1.3

    def walk(budget_list, inst):
        ps.System.clear()
        st = ps.SparseState()
        run = qda.Runner(st)
        qda.declare_registers(run, n_bits)
        if inst:
            run.add_register("inst", U, 1)
            run.op(ps.Hadamard_Int_Full("inst"))
        run.op(ps.Hadamard_Int_Full("main_reg"))
        enc_A = qda.BlockEncodingTridiagonal("main_reg", "anc_UA", alpha, -1.0)
        enc_b = qda.StatePrepHadamard("main_reg")
        eps = eps0 / len(budget_list)
        for i in range(steps):
            s = [i / b for b in budget_list] if inst else i / budget_list[0]
            qda.WalkS(enc_A, enc_b, *qda.REGS, s, kappa, p, inst_reg="inst" if inst else None).apply(run)
            run.op(ps.ClearZero(eps))
            run.op(ps.Normalize())
        return st.download()

    eps_saved = ps.get_clearzero_default_eps()
    try:
        plain = [walk([b], False) for b in budgets]
        ps.set_clearzero_default_eps(eps0 / 2)  # the ClearZero calls inside the walk
        regs, amps = walk(budgets, True)
    finally:
        ps.set_clearzero_default_eps(eps_saved)
    ncol = len(qda.REGS)
    for t, (pr, pa) in enumerate(plain):
        sel = regs[:, ncol] == t
        br, ba = regs[sel][:, :ncol], amps[sel] * math.sqrt(2)
        assert len(ba) == len(pa) > 1 << n_bits
        o1, o2 = np.lexsort(pr[:, :ncol].T[::-1]), np.lexsort(br.T[::-1])
        assert np.array_equal(pr[o1, :ncol], br[o2])
        assert np.max(np.abs(pa[o1] - ba[o2])) <= 1e-12
