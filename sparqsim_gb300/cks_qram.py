"""The CKS solver's quantum walk over a sparse matrix held in QRAM, on the
GB300 engine: the general (QRAM) form of the walk in
SparQ_Algorithm/include/hamiltonian_simulation.h, operator for operator:

- the sparse-matrix oracles SparseMatrixOracle1 (element of row j, sparse
  slot s: a QRAM load at data_offset + nnz_col * j + s, :983-1058) and
  SparseMatrixOracle2 (column <-> slot by a binary search of row j's sorted
  column list in QRAM, :1060-1172), with GetRowAddr / GetDataAddr and
  QuantumBinarySearch_Fast (src/hamiltonian_simulation.cpp:146-253);
- the walk rotation angle GetQWRotateAngle_Int_Int_Int (:321-385) and
  CondRot_Fixed_Bool;
- the state preparation T and its dagger (:1276-1446), the walk and its
  steps (QuantumWalkNSteps, :1551-1773) and the LCU accumulation
  sum_j c_j W^(2j+1)|b> (LCU_Container_NoiseFree, :1858-2066), whose
  bookkeeping is shared with the tridiagonal walk in `cks`.

The matrix type SparseMatrix belongs to the reference's absent submodule
(its header is not in the checkout); what the walk reads of it is restated
here from its uses: `data_size`, `n_row`, `nnz_col`, `positive_only`,
`get_sparsity_offset()` and `get_data()`, the QRAM words. Its word layout is
this module's: 2 n nnz_col words, the elements of row j at
[nnz_col j, nnz_col (j + 1)) (its nonzeros in ascending column order, then
zeros) and the same rows' columns at get_sparsity_offset() = n nnz_col
onwards (ascending; a row's unused slots hold n + s, distinct and above every
column, so that the search stays sorted). Elements are quantised to
data_size bits against the largest magnitude: v = round(|a| / max|a| *
(2^ds - 1)) when positive_only, else the signed round(a / max|a| *
(2^(ds-1) - 1)) in two's complement, which is what the walk angle reads back
(ratio = |v| / Amax).
"""
from __future__ import annotations

import math

import numpy as np

from . import cks, core
from .core import QRAMCircuit_qutrit, SparseState, System
from .operators import (AddRegister, ClearZero, CondRot_Fixed_Bool, GetDataAddr, GetRowAddr, Hadamard_Int,
                        Init_Unsafe, QRAMLoad, QuantumBinarySearch_Fast, RemoveRegister, Swap_General_General,
                        ZeroConditionalPhaseFlip, Add_AnyInt_AnyInt_InPlace)


# ------------------------------------------------------------------ the matrix in QRAM words
class SparseMatrix(cks.SparseMatrix):
    """A sparse n x n matrix (n a power of two; a dense array or a
    scipy.sparse matrix) as the QRAM words the walk reads, with at most
    nnz_col nonzeros per row (nnz_col the next power of two of the densest
    row).

    pysparq's constructor form is accepted too (PySparQ/pysparq/_core.pyi
    SparseMatrix, as PySparQ/pysparq/algorithms/cks_solver.py:278 and :344
    call it): SparseMatrix(elements, sparsity, data_size, nnz_col, n_row,
    positive_only), row j's slots at [nnz_col j, nnz_col (j + 1)) of both
    lists, values already scaled into (-1, 1) and quantised against full
    scale 1.0; slots whose value is 0 are padding."""

    def __init__(self, A, data_size: int, *args, positive_only: bool | None = None):
        import scipy.sparse as sp
        full_scale = None
        if len(args) == 4:  # pysparq form: (elements, sparsity, data_size, nnz_col, n_row, positive_only)
            A, positive_only = self._from_slot_lists(A, data_size, args[1], args[2]), bool(args[3])
            data_size, full_scale = int(args[0]), 1.0
        elif len(args) == 1:
            positive_only = args[0]
        elif args:
            raise TypeError("SparseMatrix(A, data_size[, positive_only]) or "
                            "SparseMatrix(elements, sparsity, data_size, nnz_col, n_row, positive_only)")
        C = sp.csr_matrix(A, dtype=np.float64)
        C.eliminate_zeros()
        C.sort_indices()
        n = C.shape[0]
        if C.shape != (n, n) or n < 2 or n & (n - 1):
            raise ValueError("SparseMatrix: a square matrix of power-of-two order")
        self.csr = C
        self.n_row = n
        self.data_size = int(data_size)
        vals = C.data
        self.positive_only = bool(np.all(vals >= 0)) if positive_only is None else bool(positive_only)
        self.is_symmetric = bool(abs(C - C.T).sum() == 0)
        counts = np.diff(C.indptr)
        dens = max(1, int(counts.max()) if counts.size else 1)
        self.nnz_col = 1 << max(0, (dens - 1).bit_length())
        if n + self.nnz_col > (1 << self.data_size):
            raise ValueError("SparseMatrix: column indices do not fit data_size bits")
        if full_scale is not None:
            if vals.size and float(np.max(np.abs(vals))) > full_scale:
                raise ValueError("SparseMatrix: elements must lie in [-1, 1] in the slot-list form")
            self.amax = full_scale
        else:
            self.amax = float(np.max(np.abs(vals))) if vals.size else 1.0
        nn = self.nnz_col
        off = n * nn
        # slot s of row j: the s-th nonzero in ascending column order, then padding
        row_of = np.repeat(np.arange(n), counts)
        slot_of = np.arange(vals.size) - np.repeat(C.indptr[:-1], counts)
        pos = nn * row_of + slot_of
        data = np.zeros(2 * n * nn, dtype=np.uint64)
        data[pos] = self.quantise_array(vals)
        cols = np.tile(np.arange(n, n + nn, dtype=np.uint64), n)  # padding: n + s
        cols[pos] = C.indices.astype(np.uint64)
        data[off:] = cols
        self._data = data
        self._angle_tables: dict = {}

    @staticmethod
    def _from_slot_lists(elements, sparsity, nnz_col, n_row):
        """The n_row x n_row matrix of pysparq's slot lists (padding slots,
        value 0, dropped; a column named twice in a row is an error)."""
        import scipy.sparse as sp
        nn, n = int(nnz_col), int(n_row)
        vals = np.asarray(elements, dtype=np.float64)
        cols = np.asarray(sparsity, dtype=np.int64)
        if nn < 1 or n < 1 or vals.shape != (n * nn,) or cols.shape != (n * nn,):
            raise ValueError("SparseMatrix: elements and sparsity need n_row * nnz_col slots each")
        rows = np.repeat(np.arange(n), nn)
        keep = vals != 0
        if np.any((cols[keep] < 0) | (cols[keep] >= n)):
            raise ValueError("SparseMatrix: a column index is outside the matrix")
        pairs = rows[keep] * n + cols[keep]
        if np.unique(pairs).size != pairs.size:
            raise ValueError("SparseMatrix: a row names the same column twice")
        return sp.csr_matrix((vals[keep], (rows[keep], cols[keep])), shape=(n, n))

    @property
    def elements(self) -> list:
        """The quantised element words, nnz_col per row (pysparq's `elements`)."""
        return [int(v) for v in self._data[: self.get_sparsity_offset()]]

    @property
    def sparsity(self) -> list:
        """The column words, nnz_col per row (pysparq's `sparsity`)."""
        return [int(v) for v in self._data[self.get_sparsity_offset():]]

    def quantise_array(self, a) -> np.ndarray:
        ds = self.data_size
        a = np.asarray(a, dtype=np.float64)
        if self.positive_only:
            return np.round(np.abs(a) / self.amax * ((1 << ds) - 1)).astype(np.uint64)
        v = np.round(a / self.amax * ((1 << (ds - 1)) - 1)).astype(np.int64)
        return (v.astype(np.uint64)) & np.uint64((1 << ds) - 1)

    def dequantised(self) -> np.ndarray:
        """The matrix the walk encodes, entry by entry as the angle reads it
        (|v| / Amax, the signs of a signed matrix kept)."""
        n, nn, ds = self.n_row, self.nnz_col, self.data_size
        amax_enc = (1 << ds) - 1 if self.positive_only else (1 << (ds - 1)) - 1
        out = np.zeros((n, n))
        off = n * nn
        for j in range(n):
            for s in range(nn):
                c = int(self._data[off + nn * j + s])
                if c >= n:
                    continue
                v = int(self._data[nn * j + s])
                if not self.positive_only and v >> (ds - 1) & 1:
                    v -= 1 << ds
                out[j, c] = v / amax_enc
        return out

    def get_sparsity_offset(self) -> int:
        return self.n_row * self.nnz_col

    def get_data(self) -> np.ndarray:
        return self._data

    def oracle_values(self):
        """(dense length, sorted values above it): the values a data register
        can hold after the element oracle, every word of the QRAM."""
        dense = self.n_row + self.nnz_col
        extra = np.unique(self._data[self._data >= np.uint64(dense)])
        return dense, [int(v) for v in extra]


# ------------------------------------------------------------------ oracles
class SparseMatrixOracle1:
    """|offset>|j>|s>|z> -> |offset>|j>|s>|z ^ a_(j, s)> (hamiltonian_simulation.h:983-1058)."""

    def __init__(self, qram, reg_offset, reg_row, reg_col_id, reg_output, row_size: int):
        self.qram, self.offset, self.row, self.col, self.out = qram, reg_offset, reg_row, reg_col_id, reg_output
        self.row_size = int(row_size)

    def apply(self, run):
        run.add_register("data_addr", core.UnsignedInteger, self.qram.address_size)
        run.op(GetDataAddr(self.offset, self.row, self.col, self.row_size, "data_addr"))
        run.op(QRAMLoad(self.qram, "data_addr", self.out))
        run.op(GetDataAddr(self.offset, self.row, self.col, self.row_size, "data_addr"))
        run.remove_register("data_addr")

    apply_dag = apply


class SparseMatrixOracle2:
    """|offset>|j>|k>|0> -> |offset>|j>|s_k>|0>: row j's column k to its
    sparse slot (forward) and back (dag), by the binary search of the row's
    column list (hamiltonian_simulation.h:1060-1172)."""

    def __init__(self, qram, reg_sparse_offset, reg_row, reg_col, reg_search_result, row_size: int):
        self.qram, self.offset, self.row = qram, reg_sparse_offset, reg_row
        self.col, self.sr, self.row_size = reg_col, reg_search_result, int(row_size)

    def _row_addr(self):
        return GetRowAddr(self.offset, self.row, self.row_size, "row_addr")

    def apply(self, run):
        run.add_register("row_addr", core.UnsignedInteger, self.qram.address_size)
        run.op(self._row_addr())
        run.op(QuantumBinarySearch_Fast(self.qram, "row_addr", self.row_size, self.col, self.sr))
        run.op(QRAMLoad(self.qram, self.sr, self.col))
        run.op(Swap_General_General(self.col, self.sr))
        run.op(Add_AnyInt_AnyInt_InPlace(self.col, "row_addr"), dag=True)
        run.op(self._row_addr())
        run.remove_register("row_addr")

    def apply_dag(self, run):
        run.add_register("row_addr", core.UnsignedInteger, self.qram.address_size)
        run.op(self._row_addr())
        run.op(Add_AnyInt_AnyInt_InPlace(self.col, "row_addr"))
        run.op(Swap_General_General(self.col, self.sr))
        run.op(QRAMLoad(self.qram, self.sr, self.col))
        run.op(QuantumBinarySearch_Fast(self.qram, "row_addr", self.row_size, self.col, self.sr))
        run.op(self._row_addr())
        run.remove_register("row_addr")


# ------------------------------------------------------------------ T and the walk
class T:
    """The walk's state preparation and its dagger, op for op as
    hamiltonian_simulation.h:1276-1446 (the dagger is the reference's
    sequence, with its ClearZero calls and checks)."""

    def __init__(self, qram, reg_data_offset, reg_sparse_offset, reg_j, reg_b1, reg_k, reg_b2, reg_search_result,
                 nnz_col: int, data_size: int, mat: SparseMatrix):
        self.qram = qram
        self.data_offset, self.sparse_offset = reg_data_offset, reg_sparse_offset
        self.j, self.b1, self.k, self.b2, self.sr = reg_j, reg_b1, reg_k, reg_b2, reg_search_result
        self.nnz_col, self.data_size, self.mat = int(nnz_col), int(data_size), mat

    def _o1(self, run):
        SparseMatrixOracle1(self.qram, self.data_offset, self.j, self.k, "data", self.nnz_col).apply(run)

    def _o2(self, run, dag=False):
        o = SparseMatrixOracle2(self.qram, self.sparse_offset, self.j, self.k, self.sr, self.nnz_col)
        (o.apply_dag if dag else o.apply)(run)

    def _angle(self):
        return cks.GetQWRotateAngle_Int_Int_Int("data", self.j, self.k, "rotation", self.mat)

    def apply(self, run):
        run.add_register("data", core.UnsignedInteger, self.data_size)
        run.op(Hadamard_Int(self.k, int(math.log2(self.nnz_col))))
        self._o1(run)
        self._o2(run, dag=True)
        run.add_register("rotation", core.Rational, 32)
        run.op(self._angle())
        run.op(CondRot_Fixed_Bool("rotation", self.b2))
        run.op(self._angle())
        run.remove_register("rotation")
        self._o2(run)
        self._o1(run)
        run.remove_register("data")
        self._o2(run, dag=True)
        run.check(cks.CheckNan())

    def apply_dag(self, run):
        run.add_register("data", core.UnsignedInteger, self.data_size)
        self._o2(run)
        run.check(cks.CheckNan())
        self._o1(run)
        self._o2(run)
        run.add_register("rotation", core.Rational, 32)
        run.op(self._angle())
        run.op(CondRot_Fixed_Bool("rotation", self.b2), dag=True)
        run.op(self._angle())
        run.remove_register("rotation")
        run.op(ClearZero())
        self._o2(run, dag=True)
        run.check(cks.CheckNormalization())
        self._o1(run)
        run.op(Hadamard_Int(self.k, int(math.log2(self.nnz_col))))
        run.op(ClearZero())
        run.remove_register("data")


class QuantumWalkNSteps(cks.QuantumWalkNSteps_Tridiagonal):
    """Registers, initial state and steps of the QRAM walk
    (hamiltonian_simulation.h:1551-1773): every register
    max(log2(QRAM words), data_size) bits wide, sparse_offset set to the
    sparsity offset."""

    def __init__(self, mat: SparseMatrix):
        self.mat = mat
        data = mat.get_data()
        self.addr_size = int(math.log2(data.size))
        self.data_size, self.n_row, self.nnz_col = mat.data_size, mat.n_row, mat.nnz_col
        self.offset = mat.get_sparsity_offset()
        self.default_register_size = max(self.addr_size, self.data_size)
        self.qram = QRAMCircuit_qutrit(self.addr_size, self.data_size, data)

    def InitEnvironment(self, declare=None):
        declare = declare or System.add_register
        w = self.default_register_size
        declare(self.data_offset, core.UnsignedInteger, w)
        declare(self.sparse_offset, core.UnsignedInteger, w)
        declare(self.j, core.UnsignedInteger, w)
        declare(self.b1, core.Boolean, 1)
        declare(self.k, core.UnsignedInteger, w)
        declare(self.b2, core.Boolean, 1)
        declare(self.j_comp, core.UnsignedInteger, w)
        declare(self.k_comp, core.UnsignedInteger, w)

    def _T(self):
        return T(self.qram, self.data_offset, self.sparse_offset, self.j, self.b1, self.k, self.b2, self.k_comp,
                 self.nnz_col, self.default_register_size, self.mat)


class LCU_Container_NoiseFree(cks.LCU_Container_NoiseFree_Tridiagonal):
    """sum_j c_j W^(2j+1)|b> over the QRAM walk (hamiltonian_simulation.h:
    1858-2066): b = kappa^2 log(kappa / eps), j0 = sqrt(b log(4 b / eps))
    (or the inverse coefficients' J); the bookkeeping is the tridiagonal
    container's."""

    def __init__(self, mat: SparseMatrix, kappa: float, eps: float, checks: bool = True):
        self.quantum_walk_obj = QuantumWalkNSteps(mat)
        self.kappa, self.eps = float(kappa), float(eps)
        self.b = int(self.kappa * self.kappa * (math.log(self.kappa) - math.log(self.eps)))
        self.chebyshev_obj = cks.ChebyshevPolynomialCoefficient(self.b)
        self.j0 = int(math.sqrt(self.b * (math.log(4 * self.b) - math.log(self.eps))))
        self.j = 0
        self.a = 0.0
        self.inv_coef = None
        self.quantum_walk_obj.InitEnvironment()
        self.step_state = self.quantum_walk_obj.CreateSys()
        self.current_state = SparseState()
        self.run = cks.Runner(self.step_state, checks)


def banded_symmetric(n: int, half_bandwidth: int, kappa: float, seed: int = 20261204):
    """A symmetric banded matrix (scipy.sparse CSR) with off-diagonals uniform
    in [-1, 1] and the diagonal set for lambda_max / lambda_min = kappa:
    extreme eigenvalues in FP64 up to n = 4096, Gershgorin bounds of the
    off-diagonal part above (the workload of the QRAM CKS leg)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    diags, offs = [], []
    for d in range(1, half_bandwidth + 1):
        v = rng.uniform(-1.0, 1.0, n - d)
        diags += [v, v]
        offs += [d, -d]
    B = sp.diags(diags, offs, shape=(n, n), format="csr")
    if n <= 4096:
        ev = np.linalg.eigvalsh(B.toarray())
        lo, hi = float(ev[0]), float(ev[-1])
    else:
        r = float(np.max(np.abs(B).sum(axis=1)))
        lo, hi = -r, r
    shift = (hi - kappa * lo) / (kappa - 1.0)
    return (B + shift * sp.identity(n, format="csr")).tocsr()
