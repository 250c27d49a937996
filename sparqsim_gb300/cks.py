"""CKS (Childs-Kothari-Somma) linear-system solver on the GB300 engine.

The Chebyshev-LCU quantum walk on a constant-diagonal tridiagonal matrix
A = tridiag(beta, alpha, beta) with arithmetic (QRAM-free) oracles, in the
circuit form of SparQ_Algorithm/include/hamiltonian_simulation_tridiagonal.h:

- the quantised positive-only matrix and its 4-slot row windows
  (TridiagonalSpec, make_tridiagonal_matrix_spec, :104-230);
- the element and slot<->column oracles (TridiagOracle1/2, :235-357;
  src/hamiltonian_tridiagonal.cpp), the parity phase D = diag((-1)^i)
  (:359-396), the walk rotation angle (GetQWRotateAngle_Int_Int_Int,
  hamiltonian_simulation.h:321-385) and CondRot_Fixed_Bool;
- the state preparation T and its dagger (T_Tridiagonal, :398-533), the walk
  (QuantumWalkNSteps_Tridiagonal, :535-684) and the LCU accumulation of
  sum_j c_j W^(2j+1) |b> (LCU_Container_NoiseFree_Tridiagonal, :686-852)
  through add_systems, with the stock (binomial / erfc) coefficients
  (hamiltonian_simulation.h:391-440, src/hamiltonian_simulation.cpp:40-100)
  or the least-squares 1/x coefficients (ChebyshevInverseCoefficients,
  :54-96).

Every per-entry step is an elementwise instruction on the GPU; Hadamard_Int
on the slot register and CondRot_Fixed_Bool are the split/merge operators;
add_systems is the GPU merge. The walk angle is a function of the element
value alone: its values are computed on the host with the C library's acos
(as the CPU reference does) and looked up on the GPU, so the angle bits are
the CPU's.

The oracles' tag registers (j_comp, k_comp) are declared 64 bits wide: the
reference reads them modulo 2^k_width but its slot->column oracle stores
row addresses into them unmasked, and a 64-bit register keeps every bit it
keeps (the comparisons, swaps and post-selection see the same values).
"""
from __future__ import annotations

import math

import numpy as np

from . import core
from .core import SparseState, StateStorageType, System
from .operators import (AddRegister, ClearZero, CondRot_Fixed_Bool, ElementwiseOperator, Hadamard_Int, Init_Unsafe,
                        PartialTraceSelect, PartialTraceSelectRange, RemoveRegister, SelfAdjointOperator,
                        Swap_General_General, ZeroConditionalPhaseFlip, _R, add_systems)

SLOT_COUNT = 4
STEP_CONSTANT = 2305


# ------------------------------------------------------------------ matrix
class TridiagonalSpec:
    """Quantised constant-diagonal tridiagonal matrix with 4-slot row windows
    (hamiltonian_simulation_tridiagonal.h:104-190)."""

    slot_count = SLOT_COUNT

    def __init__(self, n_row: int, data_size: int, alpha_enc: int, beta_enc: int):
        self.n_row, self.data_size = int(n_row), int(data_size)
        self.alpha_enc, self.beta_enc = int(alpha_enc), int(beta_enc)
        self.sparse_offset = self.n_row * SLOT_COUNT
        self.addr_mask = 2 * self.sparse_offset - 1
        self.k_width = max(int(math.log2(self.n_row)) + 1, self.data_size)

    def window_base(self, j: int) -> int:
        b = j - 1 if j > 0 else 0
        return min(b, self.n_row - SLOT_COUNT)

    def col_of(self, j: int, s: int) -> int:
        return self.window_base(j) + s

    def value_of(self, j: int, s: int) -> int:
        c = self.col_of(j, s)
        if c == j:
            return self.alpha_enc
        if c + 1 == j or c == j + 1:
            return self.beta_enc
        return 0

    def combined_mem(self, idx: int) -> int:
        idx &= self.addr_mask
        half = self.n_row * SLOT_COUNT
        if idx < half:
            return self.value_of(idx >> 2, idx & 3)
        t = idx - half
        return self.col_of(t >> 2, t & 3)

    def enc_word(self) -> int:
        if self.alpha_enc >> 32 or self.beta_enc >> 32:
            raise ValueError("quantised elements wider than 32 bits")
        return self.alpha_enc | (self.beta_enc << 32)


class SparseMatrix:
    """What the walk angle and the walk need of the reference's SparseMatrix:
    element width, slots per row, order, sign convention, and the values a
    data register can hold after the element oracle (element values, and
    window columns for out-of-range addresses)."""

    def __init__(self, spec: TridiagonalSpec):
        self.spec = spec
        self.data_size = spec.data_size
        self.nnz_col = SLOT_COUNT
        self.n_row = spec.n_row
        self.positive_only = True
        self._angle_tables: dict = {}

    def get_sparsity_offset(self) -> int:
        return self.n_row * self.nnz_col

    def oracle_values(self):
        """(dense length, sorted values above it): every word of the combined
        table is a window column (< n) or an element value."""
        dense = self.n_row
        extra = sorted({v for v in (0, self.spec.alpha_enc, self.spec.beta_enc) if v >= dense})
        return dense, extra

    def angle_table(self, out_width: int):
        """Lookup table of the walk angle for every value oracle_values() holds."""
        from ._native import call
        tab = self._angle_tables.get(out_width)
        if tab is None:
            import ctypes
            dense, extra = self.oracle_values()
            vals = np.concatenate([np.arange(dense, dtype=np.uint64), np.array(extra, dtype=np.uint64)])
            words = np.zeros(vals.size, dtype=np.uint64)
            call("sq_qw_rotate_angle_words", vals.ctypes.data_as(ctypes.c_void_p), vals.size, self.data_size,
                 1 if self.positive_only else 0, out_width, words.ctypes.data_as(ctypes.c_void_p))
            tab = LookupTable(words[:dense], vals[dense:], words[dense:])
            self._angle_tables[out_width] = tab
        return tab


def make_tridiagonal_matrix_spec(alpha: float, beta: float, n: int, ds: int):
    """(SparseMatrix, TridiagonalSpec) of tridiag(beta, alpha, beta) scaled by
    1 / (|alpha| + 2 |beta|) and quantised to ds bits, magnitudes only
    (hamiltonian_simulation_tridiagonal.h:192-230); n a power of two >= 8."""
    if n < 8 or n & (n - 1):
        raise ValueError("n must be a power of two >= 8")
    lam_max = abs(alpha) + 2.0 * abs(beta)
    scale = 1.0 / lam_max
    alpha_enc = math.floor(abs(alpha) * scale * float(1 << ds))
    beta_enc = math.floor(abs(beta) * scale * float(1 << ds))
    spec = TridiagonalSpec(n, ds, alpha_enc, beta_enc)
    return SparseMatrix(spec), spec


def walk_spectrum(spec: TridiagonalSpec):
    """The exact spectral interval of the quantised walk matrix, widened by
    1e-12 on each side (CKSPoiseuilleBench.cu:176-182)."""
    n = spec.n_row
    ccos = math.cos(math.pi / float(n + 1))
    denom = float(1 << spec.data_size) * 4.0
    lam1 = (float(spec.alpha_enc) + 2.0 * float(spec.beta_enc) * ccos) / denom
    lamn = (float(spec.alpha_enc) - 2.0 * float(spec.beta_enc) * ccos) / denom
    return min(lam1, lamn) * (1.0 - 1e-12), max(lam1, lamn) * (1.0 + 1e-12)


# ------------------------------------------------------------------ coefficients
class ChebyshevPolynomialCoefficient:
    """The stock LCU coefficients c_j of sum_j c_j T_(2j+1)
    (src/hamiltonian_simulation.cpp:40-100): 2 erfc((j + 1/2) / sqrt(b)) for
    b > 100, else 4 sum_{i=j+1..b} C(2b, b+i) / 4^b; odd j negative."""

    def __init__(self, b: int):
        self.b = int(b)

    def C(self, big: int, small: int) -> float:
        ret = 1.0
        flag = True
        pow2_b = math.pow(2, self.b)
        for i in range(small):
            ret /= (small - i)
            ret *= (big - i)
            if flag and ret > pow2_b:
                flag = False
                ret /= pow2_b
        if flag:
            ret /= pow2_b
        return ret / pow2_b

    def coef(self, j: int) -> float:
        if self.b > 100:
            return math.erfc((j + 0.5) / math.sqrt(self.b)) * 2
        ret = 0.0
        for i in range(j + 1, self.b + 1):
            ret += self.C(2 * self.b, self.b + i)
        return ret * 4

    @staticmethod
    def sign(j: int) -> bool:
        return bool(j & 1)

    @staticmethod
    def step(j: int) -> int:
        return 2 * j + 1


class ChebyshevInverseCoefficients:
    """1/x ~ sum_{j<=J} d_j T_(2j+1)(x) on [m, M] by collocation least squares
    on the Lobatto grid x_i = (M+m)/2 + (M-m)/2 cos(pi i / ngrid)
    (hamiltonian_simulation_tridiagonal.h:54-96). The system is numerically
    rank-deficient; singular values below min(rows, cols) * eps of the largest
    are dropped (the truncation of the reference's SVD solve), and the minimum
    norm solution is taken. a = sum |d_j|."""

    def __init__(self, m: float, M: float, J: int, ngrid: int = 4096):
        self.J = int(J)
        th = math.pi * np.arange(ngrid + 1, dtype=np.float64) / float(ngrid)
        x = 0.5 * (M + m) + 0.5 * (M - m) * np.cos(th)
        T = np.empty((ngrid + 1, 2 * J + 2))
        T[:, 0] = 1.0
        T[:, 1] = x
        for k in range(2, 2 * J + 2):
            T[:, k] = 2.0 * x * T[:, k - 1] - T[:, k - 2]
        V = T[:, 1::2]
        y = 1.0 / x
        rcond = float(min(V.shape)) * np.finfo(np.float64).eps
        self.coef = np.linalg.lstsq(V, y, rcond=rcond)[0]
        self.a = float(np.sum(np.abs(self.coef)))


# ------------------------------------------------------------------ operators
class LookupTable:
    """A classical function table on the GPU (sq_lookup_create): f(v) =
    dense[v] for v < len(dense), words[i] for v == keys[i]."""

    def __init__(self, dense, keys, words):
        import ctypes

        from ._native import call
        d = np.ascontiguousarray(dense, dtype=np.uint64)
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        w = np.ascontiguousarray(words, dtype=np.uint64)
        h = ctypes.c_void_p()
        call("sq_lookup_create", d.ctypes.data_as(ctypes.c_void_p), d.size, k.ctypes.data_as(ctypes.c_void_p),
             w.ctypes.data_as(ctypes.c_void_p), k.size, ctypes.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            try:
                from ._native import call
                call("sq_qram_destroy", h)
            except Exception:
                pass
            self._h = None


class LookupXor(ElementwiseOperator, SelfAdjointOperator):
    """out ^= f(in) for a LookupTable f."""

    opcode = "LOOKUP_XOR"

    def __init__(self, table: LookupTable, reg_in, reg_out):
        super().__init__()
        self.table, self.reg_in, self.reg_out = table, _R(reg_in), _R(reg_out)

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1] = self.reg_in, self.reg_out
        ins.qram = self.table._h.value


class TridiagOracle1(ElementwiseOperator, SelfAdjointOperator):
    """out ^= mem(offset + 4 j + slot) (hamiltonian_tridiagonal.cpp:16-33)."""

    opcode = "TRIDIAG_ELEMENT"

    def __init__(self, reg_offset, reg_row, reg_slot, reg_out, spec: TridiagonalSpec):
        super().__init__()
        self.regs = [_R(reg_offset), _R(reg_row), _R(reg_slot), _R(reg_out)]
        self.tspec = spec

    def _fill(self, ins, dag):
        for i, r in enumerate(self.regs):
            ins.reg[i] = r
        ins.imm[0] = self.tspec.n_row
        ins.imm[1] = self.tspec.enc_word()


class TridiagOracle2(ElementwiseOperator):
    """Column -> slot (forward) and slot -> column (dag) on (k, k_comp)
    (hamiltonian_tridiagonal.cpp:35-83)."""

    opcode = "TRIDIAG_SLOT_COLUMN"

    def __init__(self, reg_offset, reg_row, reg_k, reg_sr, spec: TridiagonalSpec):
        super().__init__()
        self.regs = [_R(reg_offset), _R(reg_row), _R(reg_k), _R(reg_sr)]
        self.tspec = spec

    def _fill(self, ins, dag):
        for i, r in enumerate(self.regs):
            ins.reg[i] = r
        ins.imm[0] = self.tspec.n_row
        ins.imm[1] = self.tspec.enc_word()
        ins.imm[2] = self.tspec.k_width


class TridiagParityPhase(ElementwiseOperator, SelfAdjointOperator):
    """amp = -amp where the register is odd (hamiltonian_tridiagonal.cpp:88-105)."""

    opcode = "PARITY_PHASE"

    def __init__(self, reg):
        super().__init__()
        self.reg = _R(reg)

    def _fill(self, ins, dag):
        ins.reg[0] = self.reg


class GetQWRotateAngle_Int_Int_Int(SelfAdjointOperator):
    """out ^= Rational(acos(sqrt(v / Amax)) / 2 pi), v the element in `data`
    (src/hamiltonian_simulation.cpp:257-291). On the GPU the angle comes from
    the matrix's lookup table; spec() gives the oracle the direct formula."""

    def __init__(self, data, row, col, out, mat: SparseMatrix):
        super().__init__()
        self.data_id, self.row_id, self.col_id, self.out_id = _R(data), _R(row), _R(col), _R(out)
        self.mat = mat

    def _lookup(self):
        op = LookupXor(self.mat.angle_table(System.size_of(self.out_id)), self.data_id, self.out_id)
        self.copy_control_conditions_to(op)
        return op

    def __call__(self, state: SparseState) -> None:
        self._lookup()(state)

    def dag(self, state: SparseState) -> None:
        self._lookup()(state)

    def spec(self, dag=False):
        return ("qw_rotate_angle", self.data_id, self.out_id, self.mat.data_size, self.mat.positive_only,
                self._cond())


class CheckNormalization(SelfAdjointOperator):
    """Raises unless | |psi|^2 - 1 | <= threshold (debugger.h:78-114)."""

    def __init__(self, threshold: float = 1e-5):
        super().__init__()
        self.threshold = float(threshold)

    def __call__(self, state: SparseState) -> None:
        s = state.norm_sq()
        if not abs(s - 1.0) <= self.threshold:
            raise RuntimeError(f"state not normalised: |psi|^2 = {s!r}")

    dag = __call__


class CheckNan(SelfAdjointOperator):
    """Raises if an amplitude is NaN (debugger.h:153-176); a NaN makes the
    norm NaN."""

    def __call__(self, state: SparseState) -> None:
        if math.isnan(state.norm_sq()):
            raise RuntimeError("NaN amplitude in the state")

    dag = __call__


# ------------------------------------------------------------------ walk
class Runner:
    """Applies operators and register changes to one GPU state; `peak` is the
    largest entry count after any operator (System::max_system_size)."""

    def __init__(self, state: SparseState, checks: bool = True):
        self.state, self.checks = state, checks
        self.peak = state.size()

    def op(self, o, dag: bool = False):
        (o.dag if dag else o)(self.state)
        self.peak = max(self.peak, self.state.size())

    def add_register(self, name: str, type_, width: int):
        return AddRegister(name, type_, width)(self.state)

    def remove_register(self, name: str):
        RemoveRegister(name)(self.state)

    def check(self, o):
        if self.checks:
            o(self.state)


class T_Tridiagonal:
    """State preparation T of the walk and its dagger, op for op as
    hamiltonian_simulation_tridiagonal.h:398-533 (the dagger is the
    reference's sequence, which includes its ClearZero calls)."""

    def __init__(self, reg_data_offset, reg_sparse_offset, reg_j, reg_b1, reg_k, reg_b2, reg_search_result,
                 data_size: int, mat: SparseMatrix, spec: TridiagonalSpec):
        self.data_offset, self.sparse_offset = reg_data_offset, reg_sparse_offset
        self.j, self.b1, self.k, self.b2, self.sr = reg_j, reg_b1, reg_k, reg_b2, reg_search_result
        self.data_size, self.mat, self.spec = int(data_size), mat, spec

    def _o1(self):
        return TridiagOracle1(self.data_offset, self.j, self.k, "data", self.spec)

    def _o2(self):
        return TridiagOracle2(self.sparse_offset, self.j, self.k, self.sr, self.spec)

    def _angle(self):
        return GetQWRotateAngle_Int_Int_Int("data", self.j, self.k, "rotation", self.mat)

    def apply(self, run):
        run.add_register("data", core.UnsignedInteger, self.data_size)
        run.op(Hadamard_Int(self.k, int(math.log2(SLOT_COUNT))))
        run.op(self._o1())
        run.op(self._o2(), dag=True)
        run.add_register("rotation", core.Rational, 32)
        run.op(self._angle())
        run.op(CondRot_Fixed_Bool("rotation", self.b2))
        run.op(self._angle())
        run.remove_register("rotation")
        run.op(self._o2())
        run.op(self._o1())
        run.remove_register("data")
        run.op(self._o2(), dag=True)
        run.check(CheckNan())

    def apply_dag(self, run):
        run.add_register("data", core.UnsignedInteger, self.data_size)
        run.op(self._o2())
        run.check(CheckNan())
        run.op(self._o1())
        run.op(self._o2())
        run.add_register("rotation", core.Rational, 32)
        run.op(self._angle())
        run.op(CondRot_Fixed_Bool("rotation", self.b2), dag=True)
        run.op(self._angle())
        run.remove_register("rotation")
        run.op(ClearZero())
        run.op(self._o2(), dag=True)
        run.check(CheckNormalization())
        run.op(self._o1())
        run.op(Hadamard_Int(self.k, int(math.log2(SLOT_COUNT))))
        run.op(ClearZero())
        run.remove_register("data")


class QuantumWalkNSteps_Tridiagonal:
    """Registers, initial state and steps of the walk
    (hamiltonian_simulation_tridiagonal.h:535-684)."""

    data_offset = "data_offset"
    sparse_offset = "sparse_offset"
    j = "row_id"
    b1 = "reg_b1"
    k = "col_id"
    b2 = "reg_b2"
    j_comp = "j_comp"
    k_comp = "k_comp"

    def __init__(self, mat: SparseMatrix, spec: TridiagonalSpec):
        self.mat, self.spec = mat, spec
        self.data_size, self.n_row, self.nnz_col = mat.data_size, mat.n_row, mat.nnz_col
        self.offset = mat.get_sparsity_offset()
        self.default_register_size = max(int(math.log2(mat.n_row)) + 1, self.data_size)

    def GetVecInputReg(self) -> str:
        return self.j

    def get_init_size(self) -> int:
        return int(math.log2(self.mat.n_row))

    def InitEnvironment(self, declare=None):
        """Declares the walk registers; j_comp and k_comp 64 bits wide (see
        the module notes). `declare(name, type, width)` defaults to
        System.add_register."""
        declare = declare or System.add_register
        w = self.default_register_size
        declare(self.data_offset, core.UnsignedInteger, w)
        declare(self.sparse_offset, core.UnsignedInteger, w)
        declare(self.j, core.UnsignedInteger, w)
        declare(self.b1, core.Boolean, 1)
        declare(self.k, core.UnsignedInteger, w)
        declare(self.b2, core.Boolean, 1)
        declare(self.j_comp, core.UnsignedInteger, 64)
        declare(self.k_comp, core.UnsignedInteger, 64)

    def init_ops(self):
        """The initial state's preparation from |0>: sparse_offset = 4n."""
        return [Init_Unsafe(self.sparse_offset, self.offset)]

    def CreateSys(self) -> SparseState:
        st = SparseState()
        for o in self.init_ops():
            o(st)
        return st

    def _T(self):
        return T_Tridiagonal(self.data_offset, self.sparse_offset, self.j, self.b1, self.k, self.b2, self.k_comp,
                             self.default_register_size, self.mat, self.spec)

    def _swaps(self, run):
        run.op(Swap_General_General(self.j, self.k))
        run.op(Swap_General_General(self.b1, self.b2))
        run.op(Swap_General_General(self.j_comp, self.k_comp))

    def FirstStep(self, run):
        self._T().apply(run)
        self._swaps(run)
        self._T().apply_dag(run)

    def StepImplOneStep(self, run):
        run.op(ZeroConditionalPhaseFlip([self.j_comp, self.k_comp, self.b1, self.k, self.b2]))
        self._T().apply(run)
        run.check(CheckNan())
        self._swaps(run)
        self._T().apply_dag(run)
        run.check(CheckNan())

    def Step(self, run):
        self.StepImplOneStep(run)
        self.StepImplOneStep(run)


class LCU_Container_NoiseFree_Tridiagonal:
    """sum_j c_j W^(2j+1) |b>, accumulated term by term with add_systems
    (hamiltonian_simulation_tridiagonal.h:686-852): b = kappa^2 log(kappa /
    eps), j0 = sqrt(b log(4b / eps)) (or the inverse coefficients' J)."""

    def __init__(self, mat: SparseMatrix, spec: TridiagonalSpec, kappa: float, eps: float,
                 checks: bool = True):
        self.quantum_walk_obj = QuantumWalkNSteps_Tridiagonal(mat, spec)
        self.kappa, self.eps = float(kappa), float(eps)
        self.b = int(self.kappa * self.kappa * (math.log(self.kappa) - math.log(self.eps)))
        self.chebyshev_obj = ChebyshevPolynomialCoefficient(self.b)
        self.j0 = int(math.sqrt(self.b * (math.log(4 * self.b) - math.log(self.eps))))
        self.j = 0
        self.a = 0.0
        self.inv_coef = None
        self.quantum_walk_obj.InitEnvironment()
        self.step_state = self.quantum_walk_obj.CreateSys()
        self.current_state = SparseState()
        self.run = Runner(self.step_state, checks)

    def set_inverse_coefficients(self, coef: ChebyshevInverseCoefficients | None):
        self.inv_coef = coef
        self.j0 = coef.J if coef is not None else int(
            math.sqrt(self.b * (math.log(4.0 * self.b) - math.log(self.eps))))

    def GetInputVecReg(self) -> str:
        return self.quantum_walk_obj.GetVecInputReg()

    def ExternalInput_V2(self, op):
        op(self.step_state)
        ClearZero()(self.step_state)
        self.quantum_walk_obj.FirstStep(self.run)

    def Step(self) -> bool:
        if self.j > self.j0:
            return False
        if self.j != 0:
            self.quantum_walk_obj.Step(self.run)
        if self.inv_coef is not None:
            c = abs(float(self.inv_coef.coef[self.j]))
            sgn = float(self.inv_coef.coef[self.j]) < 0.0
        else:
            c = self.chebyshev_obj.coef(self.j)
            sgn = self.chebyshev_obj.sign(self.j)
        self.a += c
        self.Add(self.step_state, c, sgn)
        self.j += 1
        return True

    @property
    def max_system_size(self) -> int:
        """The largest walk state (the accumulator is not counted, as in the
        reference's System::max_system_size)."""
        return self.run.peak

    def Add(self, new_state: SparseState, coef: float, sign: bool):
        add_systems(self.current_state, new_state, -coef if sign else coef)

    def _impl_partial_trace(self, state: SparseState) -> float:
        w = self.quantum_walk_obj
        ret = PartialTraceSelect({w.b1: 0, w.k: 0, w.b2: 0, w.j_comp: 0, w.k_comp: 0,
                                  w.sparse_offset: w.offset, w.data_offset: 0})(state)
        ret *= PartialTraceSelectRange(w.j, (0, w.n_row - 1))(state)
        return 1.0 / ret / ret / self.a / self.a

    def PartialTrace(self) -> float:
        return self._impl_partial_trace(self.current_state)

    def PartialTrace_Nondestructive(self):
        state = SparseState(self.current_state)
        return state, self._impl_partial_trace(state)
