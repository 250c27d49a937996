"""QRAM block encodings and state preparation on the GB300 engine.

The classical side (SparQ_Algorithm/include/BlockEncoding/make_qram.h):
a matrix or vector is scaled by 2^exponent, rounded and stored as data_size-bit
two's complement (scaleAndConvertVector; a matrix column by column), and a
binary tree is built over it (make_vector_tree): the parents of the leaves hold
the sum of the squares of their two children's signed values, every higher
node the sum of its children, in heap order (level k starts at 2^k - 1), one
trailing zero word. The tree is the QRAM memory.

The quantum side, operator for operator as the reference writes it (the
circuits are the algorithm, so their steps have to be alike; the code is this
package's own):

- U_R (block_encoding_via_QRAM.h:39-193): |0>_col -> sum_j ||a_j|| |j>, a
  descent of the top levels of the tree with one conditional rotation per
  column bit, arccos(sqrt(child / parent)) from Div_Sqrt_Arccos_UInt_UInt;
- U_L (:195-396): |j>_col |0>_row -> |j> |a_j / ||a_j||>, the descent of
  column j's subtree, the last level by GetRotateAngle_Int_Int (signs);
- Block_Encoding_via_QRAM (:398-483): U_A = SWAP(row, col) U_R^dag(col)
  U_L(row, col), so <i|_col <0|_row U_A |j>_col |0>_row = A_ij / ||A||_F
  (the quantisation aside);
- State_Prep_via_QRAM (SparQ_Algorithm/include/state_preparation.h:36-250):
  |0> -> sum_i b_i |i> / ||b|| from the vector's tree.

Every angle a descent computes is the angle of a (child, parent) pair (or of
the two leaves under a leaf parent) of the tree, so a QRAMTree builds the
angle tables for all of its pairs once; the rotations then take the C
library's angle bits, exactly as the reference's CPU loop does.

Conditions on these composites apply to every operator inside them; the
register bookkeeping (AddRegister, SplitRegister, ...) acts on all entries,
which is what the reference's SPLIT_BY_CONDITIONS / MERGE_BY_CONDITIONS
blocks amount to as long as the inside writes no condition register. One
difference in timing remains: the ClearZero calls inside prune every entry,
where the reference's prune only the part of the state the block processes
(entries below the threshold set aside by the conditions are pruned at the
next ClearZero after the block instead).
"""
from __future__ import annotations

import math

import numpy as np

from . import core
from .core import QRAMCircuit_qutrit, System
from .operators import (SQ_ANGLE_DIV_SQRT_ARCCOS, SQ_ANGLE_ROTATE, Add_ConstUInt_InPlace,
                        Add_Mult_UInt_ConstUInt_InPlace, Add_UInt_UInt_InPlace, AngleTable, BaseOperator,
                        ClearZero, CondRot_Fixed_Bool, Div_Sqrt_Arccos_UInt_UInt, ElementwiseOperator,
                        GetRotateAngle_Int_Int, Mult_UInt_ConstUInt, QRAMLoad, ShiftLeft_InPlace,
                        ShiftRight_InPlace, Swap_General_General, X_Bool)
from .qda import Composite, _with

U64 = (1 << 64) - 1


# ------------------------------------------------------------------ classical side (make_qram.h)
def make_complement(v: int, size: int) -> int:
    """The size-bit two's complement of v."""
    return v & ((1 << size) - 1) if size < 64 else v & U64


def get_complement(v: int, size: int) -> int:
    v &= (1 << size) - 1
    return v - (1 << size) if v >> (size - 1) & 1 else v


def scale_and_convert_vector(values, exponent: int, data_size: int, from_matrix: bool = False) -> np.ndarray:
    """scaleAndConvertVector (make_qram.h:58-80): round(x * 2^exponent) as
    data_size-bit two's complement; a matrix (2-D, or a flattened square
    when `from_matrix`) is taken column by column (get_column_flatten)."""
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 2:
        v = v.T.reshape(-1)
    elif from_matrix:
        n = int(round(math.sqrt(v.size)))
        if n * n != v.size:
            raise ValueError("not a flattened square matrix")
        v = v.reshape(n, n).T.reshape(-1)
    scale = 2.0 ** exponent
    # std::llround: halves away from zero
    q = np.where(v * scale >= 0, np.floor(v * scale + 0.5), np.ceil(v * scale - 0.5)).astype(np.int64)
    return (q.astype(np.uint64) & np.uint64((1 << data_size) - 1 if data_size < 64 else U64))


def make_vector_tree(dist, data_size: int) -> np.ndarray:
    """make_vector_tree (make_qram.h:148-182) for a power-of-two number of
    leaves: [root, level 1, ..., leaves, 0] in heap order; the leaves' parents
    hold the sum of the squares of the leaves' signed values, the nodes above
    the sums of their children (uint64, wrapping as the reference's)."""
    d = np.ascontiguousarray(np.asarray(dist, dtype=np.uint64))
    n = d.size
    if n < 2 or n & (n - 1):
        raise ValueError("make_vector_tree: a power of two (>= 2) of leaves")
    sign = np.uint64(1 << (data_size - 1))
    signed = ((d ^ sign) - sign).view(np.int64) if data_size < 64 else d.view(np.int64)
    sq = (signed * signed).view(np.uint64)  # products wrap like the reference's int64 arithmetic
    levels = [d]
    cur = sq[0::2] + sq[1::2]
    levels.append(cur)
    while cur.size > 1:
        cur = cur[0::2] + cur[1::2]
        levels.append(cur)
    return np.concatenate(levels[::-1] + [np.zeros(1, dtype=np.uint64)])


class QRAMTree:
    """A loading tree in QRAM, with the angle tables of every pair of words a
    descent can read. A descent loads data_parent = tree[a] and data_child =
    tree[2a + 1] (Div_Sqrt_Arccos_UInt_UInt), or at its last level tree[a']
    and tree[2a + 2] with a' = rotl(a) ^ 1 (GetRotateAngle_Int_Int), all
    addresses modulo 2^address_size. On the intended input (an empty row
    register) a is a parent on the descent; on others (the walk applies the
    encoding to every branch that passes its conditions) a can be any
    address, so the tables hold the pairs of every a."""

    def __init__(self, tree, depth: int, data_size: int, rational_size: int):
        self.tree = np.ascontiguousarray(np.asarray(tree, dtype=np.uint64))
        self.depth, self.data_size, self.rational_size = int(depth), int(data_size), int(rational_size)
        if self.tree.size != 1 << (self.depth + 1):
            raise ValueError("QRAMTree: a tree of 2^(depth + 1) words (make_vector_tree's output)")
        self.address_size = self.depth + 1
        self.qram = QRAMCircuit_qutrit(self.address_size, self.data_size, self.tree)
        t, M, w = self.tree, self.tree.size, self.address_size
        a = np.arange(M, dtype=np.int64)
        rotl = ((a << 1) | (a >> (w - 1))) & (M - 1)
        div = np.unique(np.stack([t[(2 * a + 1) % M], t[a]], axis=1), axis=0)
        rot = np.unique(np.stack([t[rotl ^ 1], t[(2 * a + 2) % M]], axis=1), axis=0)
        ds, rs = self.data_size, self.rational_size
        self.div_table = AngleTable(SQ_ANGLE_DIV_SQRT_ARCCOS, ds, ds, rs, div[:, 0], div[:, 1])
        self.rot_table = AngleTable(SQ_ANGLE_ROTATE, ds, ds, rs, rot[:, 0], rot[:, 1])

    @classmethod
    def for_matrix(cls, A, exponent: int, data_size: int, rational_size: int) -> "QRAMTree":
        """The tree of an n x n matrix (n a power of two), columns first: the
        QRAM of Block_Encoding_via_QRAM (address size 2 log2 n + 1)."""
        A = np.asarray(A, dtype=np.float64)
        n = A.shape[0]
        leaves = scale_and_convert_vector(A, exponent, data_size)
        return cls(make_vector_tree(leaves, data_size), 2 * int(round(math.log2(n))), data_size, rational_size)

    @classmethod
    def for_vector(cls, b, exponent: int, data_size: int, rational_size: int) -> "QRAMTree":
        """The tree of a vector: the QRAM of State_Prep_via_QRAM (address size
        log2 n + 1)."""
        b = np.asarray(b, dtype=np.float64).reshape(-1)
        leaves = scale_and_convert_vector(b, exponent, data_size)
        return cls(make_vector_tree(leaves, data_size), int(round(math.log2(b.size))), data_size, rational_size)

    def div(self, lhs, rhs, out):
        return Div_Sqrt_Arccos_UInt_UInt(lhs, rhs, out, table=self.div_table)

    def rot(self, lhs, rhs, out):
        return GetRotateAngle_Int_Int(lhs, rhs, out, table=self.rot_table)


# ------------------------------------------------------------------ quantum side
def _pow2(k: int) -> int:
    return 1 << k


class _Program(BaseOperator):
    """Consecutive elementwise operators of a descent as one launch of the
    fused elementwise kernel. Each entry maps on its own under every one of
    them, so the sequence applied entry by entry is the sequence applied
    operator by operator. The instructions are built when the operator is
    queued (register types can change between two queued operators)."""

    has_dag = False

    def __init__(self, items):
        super().__init__()
        self.items = items  # [(operator, dagger)], in order
        self.instrs = [o.instr(d and not o.self_adjoint) for o, d in items]

    def spec(self, dag: bool = False):
        if dag:
            raise NotImplementedError("a fused program is applied forward only")
        return ("prog", list(self.instrs))


class _QRAMComposite(Composite):
    """The descents queue their elementwise operators and apply each run of
    them as one fused program; anything else (a split of amplitudes, a
    register change, ClearZero) applies the queue first."""

    def __init__(self):
        super().__init__()
        self._queue = []

    def conditioned(self, outer):
        o = super().conditioned(outer)
        o._queue = []
        return o

    def _do(self, run, op, dag=False, outer=None):
        o = _with(op, outer if outer is not None else self)
        if isinstance(o, ElementwiseOperator):
            self._queue.append((o, dag))
        else:
            self._flush(run)
            run.op(o, dag)

    def _flush(self, run):
        if self._queue:
            prog = _Program(self._queue)
            self._queue = []
            run.op(prog)

    def _set_boolean(self, reg):
        System.set_register_type(reg, core.Boolean)

    def _add(self, run, name, type_, size):
        self._flush(run)
        return run.add_register(name, type_, size)

    def _remove(self, run, reg):
        self._flush(run)
        run.remove_register(reg)

    def _split(self, run, first, name, size):
        self._flush(run)
        return run.split(first, name, size)

    def _combine(self, run, first, second):
        self._flush(run)
        run.combine(first, second)

    def _clear(self, run):
        self._flush(run)
        run.op(ClearZero())


class U_R(_QRAMComposite):
    """Column-norm state preparation U_R|0>_col = sum_j ||a_j|| |j>
    (block_encoding_via_QRAM.h:39-193)."""

    def __init__(self, tree: QRAMTree, column_index, data_size: int, rational_size: int):
        super().__init__()
        self.tree, self.col = tree, column_index
        self.addr_size = System.size_of(column_index)
        self.data_size, self.rational_size = int(data_size), int(rational_size)

    def _open(self, run):
        n, ds, rs = self.addr_size, self.data_size, self.rational_size
        self._add(run, "addr_child", core.UnsignedInteger, n + 1)
        self._add(run, "data_parent", core.SignedInteger, ds)
        self._add(run, "data_child", core.SignedInteger, ds)
        self._add(run, "temp_bit", core.Boolean, 1)
        self._add(run, "div_result", core.Rational, rs)

    def _close(self, run):
        for r in ("data_parent", "addr_child", "data_child", "temp_bit", "div_result"):
            self._remove(run, r)
        self._clear(run)

    def _rotate(self, run, dag: bool):
        q, tr, d, col = self.tree.qram, self.tree, self._do, self.col
        d(run, QRAMLoad(q, col, "data_parent") if not dag else QRAMLoad(q, "addr_child", "data_child"))
        d(run, QRAMLoad(q, "addr_child", "data_child") if not dag else QRAMLoad(q, col, "data_parent"))
        d(run, tr.div("data_child", "data_parent", "div_result"))
        self._set_boolean("rotation")
        d(run, CondRot_Fixed_Bool("div_result", "rotation"), dag=dag)
        self._clear(run)
        d(run, tr.div("data_child", "data_parent", "div_result"))
        d(run, QRAMLoad(q, "addr_child", "data_child") if not dag else QRAMLoad(q, col, "data_parent"))
        d(run, QRAMLoad(q, col, "data_parent") if not dag else QRAMLoad(q, "addr_child", "data_child"))

    def apply(self, run):
        n, col, d = self.addr_size, self.col, self._do
        self._open(run)
        for k in range(n):
            self._split(run, col, "rotation", 1)
            self._combine(run, col, "temp_bit")
            d(run, ShiftRight_InPlace(col, 1))
            d(run, Add_ConstUInt_InPlace(col, _pow2(k) - 1))
            d(run, Mult_UInt_ConstUInt(col, 2, "addr_child"))
            d(run, X_Bool("addr_child", 0))
            self._rotate(run, False)
            d(run, X_Bool("addr_child", 0))
            d(run, Mult_UInt_ConstUInt(col, 2, "addr_child"))
            d(run, Add_ConstUInt_InPlace(col, _pow2(n) - _pow2(k) + 1))
            d(run, ShiftLeft_InPlace(col, 1))
            self._split(run, col, "temp_bit", 1)
            self._combine(run, col, "rotation")
            d(run, ShiftLeft_InPlace(col, 1))
        d(run, ShiftRight_InPlace(col, 1))
        self._close(run)

    def apply_dag(self, run):
        n, col, d = self.addr_size, self.col, self._do
        self._open(run)
        d(run, ShiftLeft_InPlace(col, 1))
        for k in range(n):
            d(run, ShiftRight_InPlace(col, 1))
            self._split(run, col, "rotation", 1)
            self._combine(run, col, "temp_bit")
            d(run, ShiftRight_InPlace(col, 1))
            d(run, Add_ConstUInt_InPlace(col, _pow2(n - 1 - k) - 1))
            d(run, Mult_UInt_ConstUInt(col, 2, "addr_child"))
            d(run, X_Bool("addr_child", 0))
            self._rotate(run, True)
            d(run, X_Bool("addr_child", 0))
            d(run, Mult_UInt_ConstUInt(col, 2, "addr_child"))
            d(run, Add_ConstUInt_InPlace(col, _pow2(n) - _pow2(n - 1 - k) + 1))
            d(run, ShiftLeft_InPlace(col, 1))
            self._split(run, col, "temp_bit", 1)
            self._combine(run, col, "rotation")
        self._close(run)


class _TreeDescent(_QRAMComposite):
    """The descent shared by U_L and State_Prep_via_QRAM: one level per bit of
    `work` (split off as 'rotation'), the parent address formed in
    addr_parent, the child at 2 parent + 1; the last level reads the two
    leaves and rotates by GetRotateAngle_Int_Int."""

    def _level(self, run, k: int, last: bool, dag: bool, addr_terms):
        q, tr, d, work = self.tree.qram, self.tree, self._do, self.work
        self._split(run, work, "rotation", 1)
        self._set_boolean("rotation")
        d(run, Add_ConstUInt_InPlace("addr_parent", _pow2(k) - 1))
        addr_terms(run, False)
        d(run, Add_UInt_UInt_InPlace(work, "addr_parent"))
        d(run, Mult_UInt_ConstUInt("addr_parent", 2, "addr_child"))
        d(run, X_Bool("addr_child", 0))
        loads = [QRAMLoad(q, "addr_parent", "data_parent"), QRAMLoad(q, "addr_child", "data_child")]
        if dag:
            loads = loads[::-1]
        if not last:
            for o in loads:
                d(run, o)
            d(run, tr.div("data_child", "data_parent", "div_result"))
            d(run, CondRot_Fixed_Bool("div_result", "rotation"), dag=dag)
            if dag or self.prune_forward:
                self._clear(run)
            d(run, tr.div("data_child", "data_parent", "div_result"))
            for o in loads:
                d(run, o)
        else:
            d(run, ShiftLeft_InPlace("addr_parent", 1))
            d(run, X_Bool("addr_parent", 0))
            d(run, Add_ConstUInt_InPlace("addr_child", 1))
            for o in loads:
                d(run, o)
            d(run, tr.rot("data_parent", "data_child", "div_result"))
            d(run, CondRot_Fixed_Bool("div_result", "rotation"), dag=dag)
            if dag or self.prune_forward:
                self._clear(run)
            d(run, tr.rot("data_parent", "data_child", "div_result"))
            for o in loads:
                d(run, o)
            d(run, Add_ConstUInt_InPlace("addr_child", 1), dag=True)
            d(run, X_Bool("addr_parent", 0))
            d(run, ShiftRight_InPlace("addr_parent", 1))
        d(run, X_Bool("addr_child", 0))
        d(run, Mult_UInt_ConstUInt("addr_parent", 2, "addr_child"))
        d(run, Add_UInt_UInt_InPlace(work, "addr_parent"), dag=True)
        addr_terms(run, True)
        d(run, Add_ConstUInt_InPlace("addr_parent", _pow2(k) - 1), dag=True)
        self._combine(run, work, "rotation")


class U_L(_TreeDescent):
    """U_L|j>_col|0>_row = |j>|a_j / ||a_j||> (block_encoding_via_QRAM.h:195-396)."""

    prune_forward = False  # the reference's forward U_L has no ClearZero between levels

    def __init__(self, tree: QRAMTree, row_index, column_index, data_size: int, rational_size: int):
        super().__init__()
        self.tree, self.work, self.col = tree, row_index, column_index
        self.addr_size = System.size_of(row_index)
        self.data_size, self.rational_size = int(data_size), int(rational_size)

    def _open(self, run):
        n, ds, rs = self.addr_size, self.data_size, self.rational_size
        self._add(run, "addr_parent", core.UnsignedInteger, 2 * n + 1)
        self._add(run, "addr_child", core.UnsignedInteger, 2 * n + 1)
        self._add(run, "data_parent", core.SignedInteger, ds)
        self._add(run, "data_child", core.SignedInteger, ds)
        self._add(run, "div_result", core.Rational, rs)

    def _close(self, run):
        for r in ("addr_parent", "data_parent", "addr_child", "data_child", "div_result"):
            self._remove(run, r)
        self._clear(run)

    def _col_term(self, k):
        def terms(run, undo):
            self._do(run, Add_Mult_UInt_ConstUInt_InPlace(self.col, _pow2(k - self.addr_size), "addr_parent"),
                     dag=undo)
        return terms

    def apply(self, run):
        n, d = self.addr_size, self._do
        self._open(run)
        for k in range(n, 2 * n):
            self._level(run, k, k == 2 * n - 1, False, self._col_term(k))
            d(run, ShiftLeft_InPlace(self.work, 1))
        d(run, ShiftRight_InPlace(self.work, 1))
        self._close(run)

    def apply_dag(self, run):
        n, d = self.addr_size, self._do
        self._open(run)
        d(run, ShiftLeft_InPlace(self.work, 1))
        for k in range(2 * n - 1, n - 1, -1):
            d(run, ShiftRight_InPlace(self.work, 1))
            self._level(run, k, k == 2 * n - 1, True, self._col_term(k))
        self._close(run)


class State_Prep_via_QRAM(_TreeDescent):
    """|0> -> sum_i b_i |i> / ||b|| on `work_qubit` from the vector's tree
    (state_preparation.h:36-250)."""

    prune_forward = True  # the reference's state preparation prunes after every rotation

    def __init__(self, tree: QRAMTree, work_qubit, data_size: int, rational_size: int):
        super().__init__()
        self.tree, self.work = tree, work_qubit
        self.addr_size = System.size_of(work_qubit)
        self.data_size, self.rational_size = int(data_size), int(rational_size)

    def _open(self, run):
        n, ds, rs = self.addr_size, self.data_size, self.rational_size
        self._add(run, "addr_parent", core.UnsignedInteger, n + 1)
        self._add(run, "addr_child", core.UnsignedInteger, n + 1)
        self._add(run, "data_parent", core.SignedInteger, ds)
        self._add(run, "data_child", core.SignedInteger, ds)
        self._add(run, "div_result", core.Rational, rs)

    _close = U_L._close

    @staticmethod
    def _no_terms(run, undo):
        pass

    def apply(self, run):
        n, d = self.addr_size, self._do
        self._open(run)
        for k in range(n):
            self._level(run, k, k == n - 1, False, self._no_terms)
            d(run, ShiftLeft_InPlace(self.work, 1))
        d(run, ShiftRight_InPlace(self.work, 1))
        self._close(run)

    def apply_dag(self, run):
        n, d = self.addr_size, self._do
        self._open(run)
        d(run, ShiftLeft_InPlace(self.work, 1))
        for k in range(n - 1, -1, -1):
            d(run, ShiftRight_InPlace(self.work, 1))
            self._level(run, k, k == n - 1, True, self._no_terms)
        self._close(run)


class Block_Encoding_via_QRAM(_QRAMComposite):
    """U_A = SWAP(row, col) U_R^dag(col) U_L(row, col)
    (block_encoding_via_QRAM.h:398-483): <i|_col <0|_row U_A |j>_col |0>_row
    = A_ij / ||A||_F, A as quantised in the tree."""

    def __init__(self, tree: QRAMTree, column_index, row_index, data_size: int, rational_size: int):
        super().__init__()
        self.tree, self.col, self.row = tree, column_index, row_index
        self.data_size, self.rational_size = int(data_size), int(rational_size)

    def _parts(self):
        ul = U_L(self.tree, self.row, self.col, self.data_size, self.rational_size).conditioned(self)
        ur = U_R(self.tree, self.col, self.data_size, self.rational_size).conditioned(self)
        return ul, ur

    def apply(self, run):
        ul, ur = self._parts()
        ul.apply(run)
        ur.apply_dag(run)
        self._do(run, Swap_General_General(self.row, self.col))
        self._flush(run)

    def apply_dag(self, run):
        ul, ur = self._parts()
        self._do(run, Swap_General_General(self.row, self.col))
        self._flush(run)
        ur.apply(run)
        ul.apply_dag(run)


# ------------------------------------------------------------------ QDA through the QRAM block encoding
REGS = ("main_reg", "anc_UA", "anc_1", "anc_2", "anc_3", "anc_4")


def declare_registers(run, n_bits: int):
    """main register and anc_UA (the block encoding's row register) of n bits,
    anc_1..anc_4 of one bit (Experiments/GPUTime/qda_test.cu:38-43)."""
    run.add_register("main_reg", core.UnsignedInteger, n_bits)
    run.add_register("anc_UA", core.UnsignedInteger, n_bits)
    for a in ("anc_1", "anc_2", "anc_3", "anc_4"):
        run.add_register(a, core.Boolean, 1)


def banded_spd(n: int, half_bandwidth: int = 4, kappa: float = 50.0, seed: int = 20261203) -> np.ndarray:
    """A symmetric banded matrix with off-diagonals uniform in [-1, 1] (half
    bandwidth `half_bandwidth`) and the diagonal set to one constant that puts
    lambda_max / lambda_min at `kappa` (extreme eigenvalues in FP64)."""
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for d in range(1, half_bandwidth + 1):
        v = rng.uniform(-1.0, 1.0, n - d)
        A += np.diag(v, d) + np.diag(v, -d)
    ev = np.linalg.eigvalsh(A)
    lo, hi = float(ev[0]), float(ev[-1])
    shift = (hi - kappa * lo) / (kappa - 1.0)  # (hi + c) / (lo + c) = kappa
    return A + shift * np.eye(n)


class QDAviaQRAM:
    """The QDA solve of A x = b through the QRAM block encoding of A and the
    QRAM state preparation of b (Walk_s_via_QRAM, qda_via_QRAM.h:91-160;
    the driver of Experiments/GPUTime/qda_test.cu:8-126): the matrix is
    scaled to unit Frobenius norm and quantised (exponent, data and rational
    sizes as there), the walk runs s = i / steps, each step followed by
    ClearZero and renormalisation, and the read-out post-selects the solution
    block. `kappa` is the walk's condition parameter (by default that of the
    encoded matrix A / ||A||_F, whose smallest singular value is
    lambda_min / ||A||_F)."""

    def __init__(self, A, b, exponent: int = 20, data_size: int = 50, rational_size: int = 51,
                 kappa: float | None = None, p: float = 1.3):
        A = np.asarray(A, dtype=np.float64)
        self.n_bits = int(round(math.log2(A.shape[0])))
        if A.shape != (1 << self.n_bits, 1 << self.n_bits):
            raise ValueError("QDAviaQRAM: a square matrix of power-of-two size")
        self.A_enc = A / np.linalg.norm(A)
        self.b = np.asarray(b, dtype=np.float64) / np.linalg.norm(b)
        self.exponent, self.data_size, self.rational_size = exponent, data_size, rational_size
        ev = np.linalg.eigvalsh(self.A_enc)
        self.kappa_matrix = float(ev[-1] / ev[0])
        self.kappa = float(kappa) if kappa is not None else float(1.0 / min(abs(ev[0]), abs(ev[-1])))
        self.p = float(p)
        self.tree_A = QRAMTree.for_matrix(self.A_enc, exponent, data_size, rational_size)
        self.tree_b = QRAMTree.for_vector(self.b, exponent, data_size, rational_size)

    def encodings(self):
        enc_A = Block_Encoding_via_QRAM(self.tree_A, "main_reg", "anc_UA", self.data_size, self.rational_size)
        enc_b = State_Prep_via_QRAM(self.tree_b, "main_reg", self.data_size, self.rational_size)
        return enc_A, enc_b

    def start(self, run):
        declare_registers(run, self.n_bits)
        _, enc_b = self.encodings()
        enc_b.apply(run)

    def step(self, run, i: int, steps: int):
        from .operators import Normalize
        from .qda import WalkS
        enc_A, enc_b = self.encodings()
        WalkS(enc_A, enc_b, *REGS, i / steps, self.kappa, self.p).apply(run)
        run.op(ClearZero())
        run.op(Normalize())

    def read_out(self, state):
        """(normalised solution block, its probability, fidelity with the FP64
        solution of A x = b)."""
        from .qda import GetOutput
        out, prob = GetOutput(*[REGS[i] for i in (0, 1, 5, 4, 3, 2)])(state)
        N = 1 << self.n_bits
        x = out[N:2 * N]
        nx = np.linalg.norm(x)
        x_ref = np.linalg.solve(self.A_enc, self.b)
        x_ref /= np.linalg.norm(x_ref)
        fid = float(abs(np.vdot(x / nx, x_ref)) ** 2) if nx > 0 else 0.0
        return x / max(nx, 1e-300), float(prob * nx * nx), fid
