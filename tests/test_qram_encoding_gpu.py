"""QRAM block encodings (block_encoding_via_QRAM.h, state_preparation.h,
make_qram.h): the classical tree construction and the host angle words on the
CPU; on the GPU, the angle operators, State_Prep_via_QRAM, U_R and
Block_Encoding_via_QRAM against the oracle operator by operator (keys
bit-exact, amplitudes within 1e-12 of the largest: CondRot uses the device's
sincos), and what they prepare against the classical vectors and matrix."""
from __future__ import annotations

import math

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native
from sparqsim_gb300 import qram_encoding as Q
from sparqsim_gb300.operators import SQ_ANGLE_DIV_SQRT_ARCCOS, SQ_ANGLE_ROTATE, AngleTable

U = ps.UnsignedInteger
EXP, DS, RS = 20, 50, 51  # the reference's exponent, data and rational sizes (Experiments/GPUTime/qda_test.cu:13-15)


# ------------------------------------------------------------------ CPU
def _tree_as_written(dist, data_size):
    """make_vector_tree (make_qram.h:148-182) step by step, in Python ints."""
    dist = [int(x) for x in dist]
    temp_tree = list(dist)
    dist_sz = len(dist)
    while True:
        temp = []
        for i in range(0, dist_sz, 2):
            if i + 1 < dist_sz:
                if dist_sz == len(dist):
                    a = Q.get_complement(temp_tree[i], data_size)
                    b = Q.get_complement(temp_tree[i + 1], data_size)
                    temp.append((a * a + b * b) & Q.U64)
                else:
                    temp.append((temp_tree[i] + temp_tree[i + 1]) & Q.U64)
        temp_tree = temp + temp_tree
        dist_sz = (dist_sz + 1) // 2
        if dist_sz <= 1:
            break
    return temp_tree + [0]


@pytest.mark.parametrize("n", [2, 8, 64])
def test_make_vector_tree_matches_the_reference_loop(n):
    rng = np.random.default_rng(n)
    v = rng.normal(size=n)
    leaves = Q.scale_and_convert_vector(v, EXP, DS)
    assert np.array_equal(Q.make_vector_tree(leaves, DS), np.array(_tree_as_written(leaves, DS), dtype=np.uint64))
    # llround and two's complement
    assert [Q.get_complement(int(x), DS) for x in leaves] == [int(math.copysign(math.floor(abs(x) * 2 ** EXP + 0.5), x))
                                                              for x in v]


def test_matrix_leaves_are_column_major():
    A = np.arange(16, dtype=float).reshape(4, 4) / 16
    leaves = Q.scale_and_convert_vector(A, 4, 12)
    assert [Q.get_complement(int(x), 12) for x in leaves] == [int(round(x * 16)) for x in A.T.reshape(-1)]


def test_angle_words_are_the_c_library_formula():
    rng = np.random.default_rng(5)
    for _ in range(200):
        r = int(rng.integers(1, 1 << 50))
        l = int(rng.integers(0, r + 1))
        want = math.acos(math.sqrt(1.0 * l / r)) / math.pi / 2
        assert AngleTable.word(SQ_ANGLE_DIV_SQRT_ARCCOS, DS, DS, RS, l, r) == int(want * 2.0 ** RS)
        a, b = (int(x) for x in rng.integers(-(1 << 40), 1 << 40, 2))
        want = math.atan2(b, a) / math.pi / 2
        want = want + 1 if want < 0 else want
        w = AngleTable.word(SQ_ANGLE_ROTATE, DS, DS, RS, Q.make_complement(a, DS), Q.make_complement(b, DS))
        assert w == int(want * 2.0 ** RS)
    assert AngleTable.word(SQ_ANGLE_ROTATE, DS, DS, RS, 0, 5) == 1 << (RS - 2)           # 0.25
    assert AngleTable.word(SQ_ANGLE_ROTATE, DS, DS, RS, 0, (1 << DS) - 1) == 3 << (RS - 2)  # 0.75
    assert AngleTable.word(SQ_ANGLE_DIV_SQRT_ARCCOS, DS, DS, RS, 0, 0) == 0               # NaN -> 0


# ------------------------------------------------------------------ GPU
class DualRunner:
    def __init__(self, dual):
        self.dual, self.state = dual, dual.gpu

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


class CheckedRunner(DualRunner):
    """Compares with the oracle after every operator."""

    def op(self, o, dag=False):
        super().op(o, dag)
        self.dual.compare()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["div", "rot"])
def test_angle_operators(dual, kind):
    dual.reg("l", ps.SignedInteger, DS)
    dual.reg("r", ps.SignedInteger, DS)
    dual.reg("o", ps.Rational, RS)
    dual.reg("x", U, 6)
    rng = np.random.default_rng(9)
    n = 3000
    r = rng.integers(1, 1 << 49, n).astype(np.uint64)
    l = (rng.random(n) * r).astype(np.uint64) if kind == "div" else rng.integers(0, 1 << 50, n).astype(np.uint64)
    l[:5] = 0
    regs = np.stack([l, r, np.zeros(n, dtype=np.uint64), np.arange(n, dtype=np.uint64) % 64], axis=1)
    dual.start(regs, np.full(n, 1 / math.sqrt(n), dtype=np.complex128))
    k = SQ_ANGLE_DIV_SQRT_ARCCOS if kind == "div" else SQ_ANGLE_ROTATE
    cls = ps.Div_Sqrt_Arccos_UInt_UInt if kind == "div" else ps.GetRotateAngle_Int_Int
    table = AngleTable(k, DS, DS, RS, l, r)
    dual.apply(cls("l", "r", "o", table=table))
    dual.compare(exact_amp=True)
    dual.apply(cls("l", "r", "o", table=table).conditioned_by_bit("x", 2))
    dual.compare(exact_amp=True)
    dual.apply(cls("l", "r", "o"))  # no table: the pairs are read back and their angles computed
    dual.compare(exact_amp=True)
    # a pair the table does not hold is refused at the next synchronising call
    small = AngleTable(k, DS, DS, RS, l[:10], r[:10])
    cls("l", "r", "o", table=small)(dual.gpu)
    with pytest.raises(ps.SparQInvalid, match="angle"):
        ps.synchronize()


def _declare(dual, names_widths):
    for name, t, w in names_widths:
        dual.reg(name, t, w)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 3])
def test_state_prep_via_qram(dual, n):
    _declare(dual, [("main", U, n), ("flag", ps.Boolean, 1)])
    rng = np.random.default_rng(30 + n)
    b = rng.normal(size=1 << n)
    tree = Q.QRAMTree.for_vector(b, EXP, DS, RS)
    dual.O.register_qram(tree.qram)
    dual.start()
    run = CheckedRunner(dual)
    prep = Q.State_Prep_via_QRAM(tree, "main", DS, RS)
    prep.apply(run)
    regs, amps = dual.gpu.download()
    main = ps.System.resolve("main")
    got = np.zeros(1 << n, dtype=np.complex128)
    got[regs[:, main].astype(int)] = amps
    assert np.allclose(got, b / np.linalg.norm(b), atol=2.0 ** -(EXP - 4))
    prep.apply_dag(run)
    assert dual.gpu.size() == 1
    # conditioned: only the flag = 1 half is prepared
    run.op(ps.Hadamard_Bool("flag"))
    prep.conditioned_by_all_ones("flag").apply(run)
    assert dual.gpu.size() == 1 + (1 << n) - int(np.count_nonzero(np.abs(got) ** 2 < 1e-14))


@pytest.mark.gpu
def test_u_r_prepares_the_column_norms(dual):
    n = 2
    _declare(dual, [("main", U, n)])
    rng = np.random.default_rng(41)
    A = rng.normal(size=(1 << n, 1 << n))
    A /= np.linalg.norm(A)
    tree = Q.QRAMTree.for_matrix(A, EXP, DS, RS)
    dual.O.register_qram(tree.qram)
    dual.start()
    run = CheckedRunner(dual)
    ur = Q.U_R(tree, "main", DS, RS)
    ur.apply(run)
    regs, amps = dual.gpu.download()
    got = np.zeros(1 << n, dtype=np.complex128)
    got[regs[:, 0].astype(int)] = amps
    assert np.allclose(np.abs(got), np.linalg.norm(A, axis=0), atol=2.0 ** -(EXP - 4))
    ur.apply_dag(run)
    assert dual.gpu.size() == 1


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 3])
def test_block_encoding_via_qram(dual, n):
    """<i|_col <0|_row U_A |j>_col |0>_row = A_ij / ||A||_F for a symmetric A
    (the QDA matrices), every operator against the oracle for one column,
    the whole block for every column, and U_A^dag U_A = I."""
    _declare(dual, [("main", U, n), ("row", U, n)])
    N = 1 << n
    rng = np.random.default_rng(50 + n)
    B = rng.uniform(-1, 1, size=(N, N))
    A = (B + B.T) / 2 + N * np.eye(N)
    A /= np.linalg.norm(A)
    tree = Q.QRAMTree.for_matrix(A, EXP, DS, RS)
    dual.O.register_qram(tree.qram)
    enc = Q.Block_Encoding_via_QRAM(tree, "main", "row", DS, RS)
    main, row = ps.System.resolve("main"), ps.System.resolve("row")
    got = np.zeros((N, N))
    for j in range(N):
        regs = np.zeros((1, 2), dtype=np.uint64)
        regs[0, main] = j
        dual.start(regs, np.ones(1, dtype=np.complex128))
        run = CheckedRunner(dual) if j == 1 else DualRunner(dual)
        enc.apply(run)
        dual.compare()
        r, a = dual.gpu.download()
        sel = r[:, row] == 0
        got[r[sel, main].astype(int), j] = a[sel].real
        enc.apply_dag(run)
        dual.compare()
        r, a = dual.gpu.download()
        assert len(a) == 1 and int(r[0, main]) == j and abs(a[0] - 1) < 1e-9
    assert np.allclose(got, A, atol=2.0 ** -(EXP - 6)), np.max(np.abs(got - A))


@pytest.mark.gpu
def test_qda_walk_via_qram_against_oracle(dual):
    """Walk_s_via_QRAM (qda_via_QRAM.h:91-160): the QRAM state preparation of
    b, then walk steps with the QRAM block encoding of A inside H(s), against
    the oracle after every step."""
    A = Q.banded_spd(4, 1, 4.0, seed=3)
    b = np.random.default_rng(4).normal(size=4)
    solver = Q.QDAviaQRAM(A, b)
    dual.O.register_qram(solver.tree_A.qram)
    dual.O.register_qram(solver.tree_b.qram)
    dual.start()
    run = DualRunner(dual)
    solver.start(run)
    dual.compare()
    for i in range(3):
        solver.step(run, i, 64)
        dual.compare()
    assert dual.gpu.size() > 4


@pytest.mark.gpu
def test_qda_via_qram_solves_a_small_system():
    """A 4 x 4 banded SPD system solved by the walk through the QRAM
    encodings: the post-selected solution block against numpy's solve."""
    A = Q.banded_spd(4, 1, 1.5, seed=5)
    b = np.random.default_rng(6).normal(size=4)
    solver = Q.QDAviaQRAM(A, b)
    ps.System.clear()
    st = ps.SparseState()
    from sparqsim_gb300.qda import Runner
    run = Runner(st)
    solver.start(run)
    steps = int(0.2 * 2305 * solver.kappa)
    steps += steps % 2
    for i in range(steps):
        solver.step(run, i, steps)
    x, prob, fid = solver.read_out(st)
    print(f"QDA via QRAM, 4x4: kappa {solver.kappa:.2f}, {steps} steps, fidelity {fid:.6f}, p {prob:.3f}")
    assert fid > 0.98
