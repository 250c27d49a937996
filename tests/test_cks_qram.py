"""The CKS walk over a sparse matrix in QRAM (sparqsim_gb300.cks_qram):
the restated SparseMatrix word layout on the CPU; on the GPU, the sparse
oracles, T / T^dag and walk steps against the oracle operator by operator,
the LCU terms, and a small positive system solved end to end."""
from __future__ import annotations

import math

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import cks, cks_qram

U = ps.UnsignedInteger


def _positive_banded(n, half_bandwidth, diag, seed):
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for d in range(1, half_bandwidth + 1):
        v = rng.uniform(0.2, 1.0, n - d)
        A += np.diag(v, d) + np.diag(v, -d)
    return A + diag * np.eye(n)


# ------------------------------------------------------------------ CPU
def test_sparse_matrix_layout():
    A = _positive_banded(16, 2, 4.0, 1)
    m = cks_qram.SparseMatrix(A, 12)
    n, nn = m.n_row, m.nnz_col
    assert (n, nn) == (16, 8) and m.positive_only and m.is_symmetric  # 5 nonzeros per row -> 8 slots
    d = m.get_data()
    off = m.get_sparsity_offset()
    assert off == n * nn and d.size == 2 * n * nn
    for j in range(n):
        cols = np.nonzero(A[j])[0]
        row_cols = d[off + nn * j: off + nn * (j + 1)]
        assert list(row_cols[:len(cols)]) == list(cols)
        assert list(row_cols[len(cols):]) == [n + s for s in range(len(cols), nn)]
        assert np.all(np.diff(row_cols.astype(np.int64)) > 0)  # sorted: the binary search's precondition
        assert np.all(d[nn * j + len(cols): nn * (j + 1)] == 0)
    # the encoded matrix is the input within the quantisation
    assert np.allclose(m.dequantised() * m.amax, A, atol=m.amax / ((1 << 12) - 1))
    # a signed matrix: two's complement words, magnitudes read back
    S = A.copy()
    S[0, 1] = S[1, 0] = -0.5
    ms = cks_qram.SparseMatrix(S, 12)
    assert not ms.positive_only
    assert np.allclose(ms.dequantised() * ms.amax, S, atol=ms.amax / ((1 << 11) - 1))


def _slot_lists(M, nnz_col):
    """pysparq's slot lists of a matrix already scaled into (-1, 1): row j's
    nonzeros in ascending column order, then padding slots (column 0, value
    0), as PySparQ/pysparq/algorithms/cks_solver.py:329-341 lays them out."""
    values, sparsity = [], []
    for row in M:
        cols = list(np.nonzero(row)[0])
        for pos in range(nnz_col):
            sparsity.append(int(cols[pos]) if pos < len(cols) else 0)
            values.append(float(row[cols[pos]]) if pos < len(cols) else 0.0)
    return values, sparsity


@pytest.mark.parametrize("signed", [False, True])
def test_sparse_matrix_pysparq_form(signed):
    """ps.SparseMatrix(elements, sparsity, data_size, nnz_col, n_row,
    positive_only), the constructor the reference's Python CKS solver calls:
    the same words as the dense form, quantised against full scale 1.0."""
    A = _positive_banded(16, 2, 4.0, 3)
    if signed:
        A[2, 3] = A[3, 2] = -0.7
    M = A / np.linalg.norm(A, 2)
    vals, cols = _slot_lists(M, 5)
    m = ps.SparseMatrix(vals, cols, 14, 5, 16, not signed)
    assert isinstance(m, cks_qram.SparseMatrix)
    assert (m.n_row, m.nnz_col, m.data_size, m.positive_only, m.amax) == (16, 8, 14, not signed, 1.0)
    full = (1 << 14) - 1 if not signed else (1 << 13) - 1
    assert np.allclose(m.dequantised(), M, atol=1.0 / full)
    # the layout is the dense form's, only the full scale differs
    dense = cks_qram.SparseMatrix(M, 14, positive_only=not signed)
    off = m.get_sparsity_offset()
    assert off == dense.get_sparsity_offset() == 16 * 8
    assert m.sparsity == dense.sparsity == [int(v) for v in m.get_data()[off:]]
    assert m.elements == [int(v) for v in m.get_data()[:off]]
    nz = np.nonzero(M)
    enc = m.quantise_array(M[nz])
    slots = [8 * j + int(np.searchsorted(np.nonzero(M[j])[0], c)) for j, c in zip(*nz)]
    assert [m.elements[s] for s in slots] == [int(v) for v in enc]
    # malformed slot lists are refused
    with pytest.raises(ValueError):
        ps.SparseMatrix(vals[:-1], cols, 14, 5, 16, not signed)
    bad = list(cols)
    bad[1] = bad[0]  # row 0 names one column twice
    with pytest.raises(ValueError):
        ps.SparseMatrix(vals, bad, 14, 5, 16, not signed)
    with pytest.raises(ValueError):
        ps.SparseMatrix([2.0 * v for v in vals], cols, 14, 5, 16, not signed)


# ------------------------------------------------------------------ GPU
class DualRun:
    def __init__(self, dual):
        self.dual, self.checks, self.peak = dual, True, 0

    def op(self, o, dag=False):
        self.dual.apply(o, dag)

    def add_register(self, name, type_, width):
        return self.dual.add_register(name, type_, width)

    def remove_register(self, name):
        self.dual.remove_register(name)

    def check(self, o):
        o(self.dual.gpu)


def _walk(dual, A, ds=16, form="dense"):
    if form == "dense":
        mat = cks_qram.SparseMatrix(A, ds)
    else:  # pysparq's slot lists of A / ||A||_2, as the reference's Python solver builds them
        M = A / np.linalg.norm(A, 2)
        nnz = int(np.max(np.sum(M != 0, axis=1)))
        vals, cols = _slot_lists(M, nnz)
        mat = ps.SparseMatrix(vals, cols, ds, nnz, A.shape[0], bool(np.all(M >= 0)))
    w = cks_qram.QuantumWalkNSteps(mat)
    w.InitEnvironment(declare=dual.reg)
    dual.O.register_qram(w.qram)
    return mat, w


@pytest.mark.gpu
def test_sparse_oracles_parity(dual):
    """SparseMatrixOracle1 and SparseMatrixOracle2 both ways on a state of
    valid rows and slots, columns that are and are not in their rows, and
    out-of-range rows."""
    A = _positive_banded(16, 2, 4.0, 2)
    mat, w = _walk(dual, A)
    dual.reg("data", U, w.default_register_size)
    rng = np.random.default_rng(5)
    n = 2500
    ids = {r: ps.System.resolve(r) for r in (w.data_offset, w.sparse_offset, w.j, w.k, w.k_comp, "data")}
    regs = np.zeros((n, ps.System.register_count()), dtype=np.uint64)
    regs[:, ids[w.sparse_offset]] = mat.get_sparsity_offset()
    regs[:, ids[w.j]] = rng.integers(0, 18, n)
    regs[:, ids[w.k]] = rng.integers(0, 20, n)
    regs = np.unique(regs, axis=0)
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))
    run = DualRun(dual)
    o1 = cks_qram.SparseMatrixOracle1(w.qram, w.data_offset, w.j, w.k, "data", mat.nnz_col)
    o2 = cks_qram.SparseMatrixOracle2(w.qram, w.sparse_offset, w.j, w.k, w.k_comp, mat.nnz_col)
    o2.apply_dag(run)
    dual.compare(exact_amp=True)
    o1.apply(run)
    dual.compare(exact_amp=True)
    o1.apply(run)
    o2.apply(run)
    dual.compare(exact_amp=True)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["dense", "pysparq", "pysparq_signed"])
def test_walk_parity_with_oracle(dual, form):
    """Input preparation, FirstStep and two walk steps over a QRAM matrix at
    n = 8, every operator against the oracle: keys bit-exact, amplitudes
    within 1e-12 (CondRot takes sin and cos on the GPU). The matrix is built
    from a dense array, or from pysparq's slot lists (ps.SparseMatrix's
    constructor form), positive or with signed elements."""
    dual.relaxed = True
    A = _positive_banded(8, 1, 3.0, 3)
    if form == "pysparq_signed":
        A[1, 2] = A[2, 1] = -A[1, 2]
    mat, w = _walk(dual, A, form=form)
    assert mat.positive_only == (form != "pysparq_signed")
    dual.start()
    run = DualRun(dual)
    for o in w.init_ops():
        run.op(o)
    run.op(ps.Hadamard_Int(w.j, 3))
    run.op(ps.ClearZero())
    dual.compare(exact_amp=True)
    w.FirstStep(run)
    dual.compare()
    for _ in range(2):
        w.Step(run)
        dual.compare()
    assert dual.gpu.size() > 8


@pytest.mark.gpu
def test_small_positive_system_solved():
    """A 16 x 16 positive banded SPD system through the QRAM walk and the
    least-squares 1/x coefficients on the encoded matrix's spectrum (the
    walk encodes A / (max|A| nnz_col)): the post-selected solution against
    numpy's solve of the encoded matrix."""
    n = 16
    A = _positive_banded(n, 1, 3.0, 4)
    ps.System.clear()
    mat = cks_qram.SparseMatrix(A, 24)
    enc = mat.dequantised() / mat.nnz_col
    ev = np.linalg.eigvalsh(enc)
    kappa = 1.0 / ev[0]
    obj = cks_qram.LCU_Container_NoiseFree(mat, kappa, 0.01)
    obj.set_inverse_coefficients(cks.ChebyshevInverseCoefficients(ev[0] * (1 - 1e-12), ev[-1] * (1 + 1e-12), 256))
    run = obj.run
    run.op(ps.Hadamard_Int(obj.GetInputVecReg(), 4))
    run.op(ps.ClearZero())
    obj.quantum_walk_obj.FirstStep(run)
    while obj.Step():
        pass
    state, p_succ = obj.PartialTrace_Nondestructive()
    from sparqsim_gb300.cks_bench import read_out
    x = read_out(state, obj.GetInputVecReg(), n, False)
    ref = np.linalg.solve(enc, np.ones(n) / math.sqrt(n))
    fid = abs(np.vdot(x / np.linalg.norm(x), ref / np.linalg.norm(ref))) ** 2
    print(f"QRAM CKS n=16: kappa {kappa:.2f}, j0 {obj.j0}, fidelity {fid:.6f}, p {p_succ:.3e}, "
          f"peak {obj.max_system_size}")
    assert fid > 0.99
