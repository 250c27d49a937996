"""Operators with the pysparq names and constructor arguments, executed by
the GB300 engine.

Each operator is a value object built from register names or ids (resolved
at construction, like the reference constructors) and applied with
``op(state)`` / ``op.dag(state)``. ``spec(dag)`` describes the operation as
plain data; the engine call is chosen from it, and the same description is
what a test checker consumes.

Reference files (SparQ/src unless noted): quantum_arithmetic.cpp, qram.cpp,
basic_gates.cpp, parallel_phase_operations.cpp, hadamard.cpp, condrot.cpp,
system_operations.cpp, dark_magic.cpp; Python names from PySparQ/core.cpp.
"""
from __future__ import annotations

import cmath
import ctypes
import math
from ctypes import byref, c_double, c_uint32

from ._native import OP, SQ_ERR_BAD_RESULT, SQ_ERR_INVALID, SQ_MAX_PROGRAM, SparQError, SparQInvalid, SqInstr, call
from .core import Controllable, QRAMCircuit_qutrit, SparseState, StateStorageType, System

PI = math.pi
U64 = 0xFFFFFFFFFFFFFFFF


def _R(x) -> int:
    return System.resolve(x)


def _run(state: SparseState, spec) -> None:
    kind = spec[0]
    h = state._h
    if kind == "prog":
        instrs = spec[1]
        for i in range(0, len(instrs), SQ_MAX_PROGRAM):
            chunk = instrs[i:i + SQ_MAX_PROGRAM]
            arr = (SqInstr * len(chunk))(*chunk)
            call("sq_apply_program", h, arr, len(chunk))
    elif kind == "hadamard_int":
        call("sq_hadamard_int", h, spec[1], spec[2], byref(spec[3]))
    elif kind == "hadamard_int_batched":
        call("sq_hadamard_int_batched", h, spec[1], spec[2], spec[3], byref(spec[4]))
    elif kind == "hadamard_int_full":
        call("sq_hadamard_int_full", h, spec[1], byref(spec[2]))
    elif kind == "hadamard_bool":
        call("sq_hadamard_bool", h, spec[1], byref(spec[2]))
    elif kind == "rot_bool":
        m = (c_double * 8)(*spec[3])
        call("sq_rot_bool", h, spec[1], spec[2], m, byref(spec[4]), 0)
    elif kind == "condrot":
        call("sq_condrot_rational_bool_cond", h, spec[1], spec[2], 1 if spec[3] else 0, byref(spec[4]))
    elif kind == "condrot_general":
        tab = spec[3]
        call("sq_condrot_general_bool_cond", h, spec[1], spec[2], tab.ctypes.data_as(ctypes.POINTER(c_double)),
             tab.size // 8, byref(spec[4]))
    elif kind == "rot_general_unitary":
        mat = spec[2]
        call("sq_rot_general_unitary", h, spec[1], mat.ctypes.data_as(ctypes.POINTER(c_double)), spec[3],
             byref(spec[4]), 1 if spec[5] else 0)
    elif kind == "hadamard_partial":
        pos = (c_uint32 * len(spec[2]))(*spec[2])
        call("sq_hadamard_partial", h, spec[1], pos, len(spec[2]), byref(spec[3]))
    elif kind == "clear_zero":
        call("sq_clear_zero", h, spec[1])
    elif kind == "normalize":
        call("sq_normalize", h, None)
    else:
        raise ValueError(f"unknown operation {kind}")


class BaseOperator(Controllable):
    """op(state) / op.dag(state) (basic_components.h:748-800)."""

    self_adjoint = False
    has_dag = True

    def __init__(self):
        self._init_controls()

    def spec(self, dag: bool = False):
        raise NotImplementedError

    def __call__(self, state: SparseState) -> None:
        _run(state, self.spec(False))

    def dag(self, state: SparseState) -> None:
        if not self.has_dag:
            raise NotImplementedError("Dagger is not implemented.")
        _run(state, self.spec(not self.self_adjoint))


class SelfAdjointOperator(BaseOperator):
    self_adjoint = True


# ---------------------------------------------------------------------- elementwise
class ElementwiseOperator(BaseOperator):
    """An operator that maps each entry on its own: one instruction of the
    fused elementwise kernel."""

    opcode = "NOP"

    def _fill(self, ins: SqInstr, dag: bool) -> None:
        pass

    def instr(self, dag: bool = False) -> SqInstr:
        ins = SqInstr()
        ins.op = OP[self.opcode]
        ins.dag = 1 if dag else 0
        ins.cond = self._cond()
        self._fill(ins, dag)
        return ins

    def spec(self, dag: bool = False):
        return ("prog", [self.instr(dag)])


def _set_regs(ins, *regs):
    for i, r in enumerate(regs):
        ins.reg[i] = r


class _Regs(ElementwiseOperator):
    """Operators whose operands are only registers, stored in reg slots."""

    def __init__(self, *regs):
        super().__init__()
        self.regs = [_R(r) for r in regs]

    def _fill(self, ins, dag):
        _set_regs(ins, *self.regs)


# XOR-out (self-adjoint) three-register arithmetic: res ^= f(lhs, rhs)
def _xor3(name, opcode, doc):
    cls = type(name, (_Regs, SelfAdjointOperator), {"opcode": opcode, "__doc__": doc})
    return cls


Add_UInt_UInt = _xor3("Add_UInt_UInt", "ADD_UINT_UINT", "res ^= (lhs + rhs) mod 2^|res| (quantum_arithmetic.cpp:287-306)")
Sub_UInt_UInt = _xor3("Sub_UInt_UInt", "SUB_UINT_UINT", "res ^= (lhs - rhs) mod 2^|res| (:490-509)")
Mul_UInt_UInt = _xor3("Mul_UInt_UInt", "MUL_UINT_UINT", "res ^= (lhs * rhs) mod 2^|res| (:556-575)")
Div_UInt_UInt = _xor3("Div_UInt_UInt", "DIV_UINT_UINT", "res ^= lhs / rhs (0 when rhs == 0) (:577-600)")
And_UInt_UInt = _xor3("And_UInt_UInt", "AND_UINT_UINT", "res ^= lhs & rhs (:646-665)")
Or_UInt_UInt = _xor3("Or_UInt_UInt", "OR_UINT_UINT", "res ^= lhs | rhs (:667-686)")
Xor_UInt_UInt = _xor3("Xor_UInt_UInt", "XOR_UINT_UINT", "res ^= lhs ^ rhs (:688-707)")
Less_SInt_SInt = _xor3("Less_SInt_SInt", "LESS_SINT_SINT", "flag ^= sext(lhs) < sext(rhs) (:709-729)")
Less_UInt_UInt = _xor3("Less_UInt_UInt", "LESS_UINT_UINT", "flag ^= lhs < rhs (:961-980)")
GetMid_UInt_UInt = _xor3("GetMid_UInt_UInt", "GETMID_UINT_UINT", "mid ^= (l + r) / 2 (:1001-1020)")

Neg_UInt = _xor3("Neg_UInt", "NEG_UINT", "res ^= -reg mod 2^|res| (:511-530)")
Abs_SInt = _xor3("Abs_SInt", "ABS_SINT", "res ^= |sext(reg)| (:532-554)")
Sqrt_UInt = _xor3("Sqrt_UInt", "SQRT_UINT", "res ^= isqrt(reg) (:602-620)")
IsZero_UInt = _xor3("IsZero_UInt", "ISZERO_UINT", "flag ^= (reg == 0) (:819-837)")
Negative_SInt = _xor3("Negative_SInt", "NEGATIVE_SINT", "flag ^= sext(reg) < 0 (:839-857)")

Carry_UInt_UInt = _xor3("Carry_UInt_UInt", "CARRY_UINT_UINT", "flag ^= carry of lhs + rhs at width(res) (:731-754)")
Overflow_SInt_SInt = _xor3("Overflow_SInt_SInt", "OVERFLOW_SINT_SINT", "flag ^= signed overflow at width(res) (:756-785)")
MulOverflow_UInt_UInt = _xor3("MulOverflow_UInt_UInt", "MULOVERFLOW_UINT_UINT", "flag ^= lhs*rhs >= 2^width(res) (:787-817)")
Select_Bool_UInt_UInt = _xor3("Select_Bool_UInt_UInt", "SELECT_BOOL", "res ^= cond&1 ? lhs : rhs (:623-644)")
Compare_UInt_UInt = _xor3("Compare_UInt_UInt", "COMPARE_UINT_UINT", "equal ^= 1 if l == r else less ^= l < r (:932-959)")
Assign = _xor3("Assign", "ASSIGN", "r2 ^= r1 (:909-930)")
Swap_General_General = _xor3("Swap_General_General", "SWAP_GENERAL", "swap(r1, r2) (:982-999)")


class _InPlace2(_Regs):
    """Two-register in-place ops with an inverse: dag flips the sign."""


class Add_UInt_UInt_InPlace(_InPlace2):
    """rhs = (rhs + lhs) mod 2^|rhs|; dag subtracts (quantum_arithmetic.cpp:308-349)."""

    opcode = "ADD_UINT_UINT_INPLACE"


class Add_AnyInt_AnyInt_InPlace(_InPlace2):
    """lhs = (lhs + ext(rhs)) mod 2^|lhs|, rhs sign-extended if SignedInteger (:860-907)."""

    opcode = "ADD_ANYINT_INPLACE"


class FlipBools(_Regs, SelfAdjointOperator):
    """reg = ~reg mod 2^|reg| (quantum_arithmetic.cpp:11-30)."""

    opcode = "FLIP_BOOLS"


class _RegConst(ElementwiseOperator):
    def __init__(self, reg, const):
        super().__init__()
        self.reg = _R(reg)
        self.const = int(const) & U64

    def _fill(self, ins, dag):
        ins.reg[0] = self.reg
        ins.imm[0] = self.const


class Add_ConstUInt_InPlace(_RegConst):
    """reg = (reg + c) mod 2^|reg|; dag subtracts (:371-411)."""

    opcode = "ADD_CONST_INPLACE"


class ShiftLeft_InPlace(_RegConst):
    """Cyclic left rotation by `digit` within the register (:63-92); dag rotates right."""

    opcode = "SHIFT_LEFT"


class ShiftRight_InPlace(_RegConst):
    """Cyclic right rotation (:95-121); dag rotates left."""

    opcode = "SHIFT_RIGHT"


class _LhsConstRes(ElementwiseOperator):
    def __init__(self, lhs, const, res):
        super().__init__()
        self.lhs, self.const, self.res = _R(lhs), int(const) & U64, _R(res)

    def _fill(self, ins, dag):
        ins.reg[0] = self.lhs
        ins.reg[2] = self.res
        ins.imm[0] = self.const


class Add_UInt_ConstUInt(_LhsConstRes, SelfAdjointOperator):
    """res ^= (lhs + c) mod 2^|res| (:351-369)."""

    opcode = "ADD_UINT_CONST"


class Mult_UInt_ConstUInt(_LhsConstRes, SelfAdjointOperator):
    """res = (res ^ lhs*c) mod 2^|res| (:137-155)."""

    opcode = "MULT_UINT_CONST"


class Add_Mult_UInt_ConstUInt_InPlace(_LhsConstRes):
    """res = (res + c*lhs) mod 2^|res|; dag subtracts (:157-196)."""

    opcode = "ADD_MULT_UINT_CONST"


class Mod_Mult_UInt_ConstUInt_InPlace(ElementwiseOperator):
    """reg = reg * a^(2^x) mod N; dag multiplies by the modular inverse (:200-285)."""

    opcode = "MOD_MULT_CONST"

    def __init__(self, reg, a, x, N):
        super().__init__()
        self.reg, self.a, self.x, self.N = _R(reg), int(a), int(x), int(N)
        if math.gcd(self.a, self.N) > 1:
            raise ValueError("a and N must be coprime")
        op = self.a % self.N
        for _ in range(self.x):
            op = ((op * op) & U64) % self.N
        self.opnum = op

    def _inverse(self) -> int:
        t, nt, r, nr = 0, 1, self.N, self.opnum
        while nr != 0:
            q = r // nr
            t, nt = nt, t - q * nt
            r, nr = nr, r - q * nr
        return t % self.N if r == 1 else 1

    def _fill(self, ins, dag):
        ins.reg[0] = self.reg
        ins.imm[0] = self._inverse() if dag else self.opnum
        ins.imm[1] = self.N
        ins.dag = 0


class Swap_Bool_Bool(ElementwiseOperator, SelfAdjointOperator):
    """Swap bit digit1 of lhs with bit digit2 of rhs (:32-61)."""

    opcode = "SWAP_BOOL_BOOL"

    def __init__(self, lhs, digit1, rhs, digit2):
        super().__init__()
        self.lhs, self.d1, self.rhs, self.d2 = _R(lhs), int(digit1), _R(rhs), int(digit2)

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1] = self.lhs, self.rhs
        ins.imm[0], ins.imm[1] = self.d1, self.d2


class _Gate(ElementwiseOperator):
    def __init__(self, reg, digit=0):
        super().__init__()
        self.id = _R(reg)
        self.digit = int(digit)
        if self.digit >= System.size_of(self.id):
            raise ValueError("digit out of range of the register")

    def _fill(self, ins, dag):
        ins.reg[0] = self.id
        ins.imm[0] = self.digit


class X_Bool(_Gate, SelfAdjointOperator):
    """Flip bit `digit` of reg (basic_gates.cpp:383-401)."""

    opcode = "X_BOOL"


class Y_Bool(_Gate, SelfAdjointOperator):
    """Flip bit, amplitude *= +i / -i (basic_gates.cpp:418-441)."""

    opcode = "Y_BOOL"


class Phase_Bool(ElementwiseOperator):
    """amp *= e^{i lambda} where bit `digit` of reg is 1; dag uses e^{-i lambda}
    (basic_gates.cpp:11-54). Phase_Bool(reg, lambda) uses digit 0."""

    opcode = "PHASE_BOOL"

    def __init__(self, reg, digit, lam=None):
        super().__init__()
        if lam is None:
            digit, lam = 0, digit
        self.id, self.digit, self.lam = _R(reg), int(digit), float(lam)
        if self.digit >= System.size_of(self.id):
            raise ValueError("digit out of range of the register")

    def _fill(self, ins, dag):
        ins.reg[0] = self.id
        ins.imm[0] = self.digit
        ins.c[0] = math.cos(self.lam)
        ins.c[1] = -math.sin(self.lam) if dag else math.sin(self.lam)


class Z_Bool(Phase_Bool):
    def __init__(self, reg):
        super().__init__(reg, 0, PI)


class S_Bool(Phase_Bool):
    def __init__(self, reg):
        super().__init__(reg, 0, PI / 2)


class T_Bool(Phase_Bool):
    def __init__(self, reg):
        super().__init__(reg, 0, PI / 4)


class GlobalPhase(ElementwiseOperator):
    """amp *= c (conditionable); dag uses conj(c) (parallel_phase_operations.cpp:72-107)."""

    opcode = "GLOBAL_PHASE"

    def __init__(self, c):
        super().__init__()
        self.c = complex(c)

    def _fill(self, ins, dag):
        ins.c[0] = self.c.real
        ins.c[1] = -self.c.imag if dag else self.c.imag


def _regmask(regs) -> int:
    if isinstance(regs, (str, int)):
        regs = [regs]
    m = 0
    for r in regs:
        rid = _R(r)
        if rid >= 64:
            raise ValueError("register id >= 64")
        m |= 1 << rid
    return m


class Reflection_Bool(ElementwiseOperator, SelfAdjointOperator):
    """amp *= -1 unless (inverse XOR all-zero) (parallel_phase_operations.cpp:46-70)."""

    opcode = "REFLECTION_BOOL"

    def __init__(self, regs, inverse: bool = False):
        super().__init__()
        self.mask = _regmask(regs)
        self.inverse = bool(inverse)

    def _fill(self, ins, dag):
        ins.imm[0] = self.mask
        ins.imm[1] = 1 if self.inverse else 0


class ZeroConditionalPhaseFlip(ElementwiseOperator, SelfAdjointOperator):
    """amp *= -1 where every listed register is 0 (parallel_phase_operations.cpp:11-31)."""

    opcode = "ZERO_COND_PHASE_FLIP"

    def __init__(self, regs):
        super().__init__()
        self.mask = _regmask(regs)

    def _fill(self, ins, dag):
        ins.imm[0] = self.mask


class Init_Unsafe(ElementwiseOperator, SelfAdjointOperator):
    """Set reg = value in every entry (dark_magic.cpp:35-40)."""

    opcode = "INIT_UNSAFE"

    def __init__(self, reg, value):
        super().__init__()
        self.id, self.value = _R(reg), int(value) & U64

    def _fill(self, ins, dag):
        ins.reg[0] = self.id
        ins.imm[0] = self.value


class QRAMLoad(ElementwiseOperator, SelfAdjointOperator):
    """data ^= memory[addr mod 2^address_size] (qram.cpp:15-35, noise-free)."""

    opcode = "QRAM_LOAD"

    def __init__(self, qram: QRAMCircuit_qutrit, addr, data):
        super().__init__()
        if qram is None:
            raise ValueError("null QRAM")
        self.qram, self.register_addr, self.register_data = qram, _R(addr), _R(data)
        if self.register_addr == self.register_data:
            raise ValueError("QRAMLoad: address and data registers must differ")
        if System.type_of(self.register_addr) != StateStorageType.UnsignedInteger:
            raise ValueError("QRAMLoad: address register must be UnsignedInteger")

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1] = self.register_addr, self.register_data
        ins.qram = self.qram._h.value


QRAMLoadFast = QRAMLoad


class GetRowAddr(ElementwiseOperator, SelfAdjointOperator):
    """row_offset ^= offset + row_sz * row (hamiltonian_simulation.cpp:222-237);
    the sum is kept to the output register's width."""

    opcode = "ADDR_XOR"

    def __init__(self, reg_offset, reg_row, row_sz: int, reg_row_offset):
        super().__init__()
        self.offset_id, self.row_id, self.out_id = _R(reg_offset), _R(reg_row), _R(reg_row_offset)
        self.row_sz = int(row_sz)

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1], ins.reg[3] = self.offset_id, self.row_id, self.out_id
        ins.imm[0], ins.imm[1] = self.row_sz, 0


class GetDataAddr(ElementwiseOperator, SelfAdjointOperator):
    """data_offset ^= offset + row_sz * row + col_sparse
    (hamiltonian_simulation.cpp:239-253)."""

    opcode = "ADDR_XOR"

    def __init__(self, reg_offset, reg_row, reg_col_sparse, row_sz: int, reg_data_offset):
        super().__init__()
        self.offset_id, self.row_id, self.col_id = _R(reg_offset), _R(reg_row), _R(reg_col_sparse)
        self.out_id, self.row_sz = _R(reg_data_offset), int(row_sz)

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1], ins.reg[2], ins.reg[3] = self.offset_id, self.row_id, self.col_id, self.out_id
        ins.imm[0], ins.imm[1] = self.row_sz, 1


class QuantumBinarySearch_Fast(ElementwiseOperator, SelfAdjointOperator):
    """result ^= the address in [offset, offset + total_length) of the QRAM
    word equal to target, by floor(log2(total_length)) + 1 rounds of
    bisection, or 0 (hamiltonian_simulation.cpp:146-220)."""

    opcode = "QBS_XOR"

    def __init__(self, qram: QRAMCircuit_qutrit, reg_offset, total_length: int, reg_target, reg_result):
        super().__init__()
        if qram is None:
            raise ValueError("null QRAM")
        self.qram = qram
        self.offset_id, self.target_id, self.result_id = _R(reg_offset), _R(reg_target), _R(reg_result)
        self.total_length = int(total_length)
        self.max_step = int(math.log2(self.total_length)) + 1 if self.total_length > 0 else 1

    def _fill(self, ins, dag):
        ins.reg[0], ins.reg[1], ins.reg[2] = self.offset_id, self.target_id, self.result_id
        ins.imm[0], ins.imm[1] = self.total_length, self.max_step
        ins.qram = self.qram._h.value


class Fused(ElementwiseOperator):
    """A chain of elementwise operators applied in one pass over the state
    (one kernel launch per 32 instructions). dag applies the chain's inverse:
    the ops' adjoints in reverse order."""

    def __init__(self, ops):
        super().__init__()
        for op in ops:
            if not isinstance(op, ElementwiseOperator):
                raise TypeError(f"{type(op).__name__} is not elementwise")
        self.ops = list(ops)

    def spec(self, dag: bool = False):
        if not dag:
            return ("prog", [op.instr(False) for op in self.ops])
        return ("prog", [op.instr(not op.self_adjoint) for op in reversed(self.ops)])


# ---------------------------------------------------------------------- split / merge
class Hadamard_Int(SelfAdjointOperator):
    """H on the low n_digits bits of reg, grouped by all other bits; ClearZero
    after (hadamard.cpp:18-162)."""

    def __init__(self, reg, n_digits):
        super().__init__()
        self.id, self.n_digits = _R(reg), int(n_digits)

    def spec(self, dag=False):
        return ("hadamard_int", self.id, self.n_digits, self._cond())


class Hadamard_Int_Batched(SelfAdjointOperator):
    """Hadamard_Int on the low n bits of `reg`, n read per entry from
    `width_reg` (n <= max_digits <= 8): many trajectories of different widths
    transformed in one pass. Same result as Hadamard_Int(reg, h)
    .conditioned_by_value(width_reg, h) for every h."""

    def __init__(self, reg, width_reg, max_digits):
        super().__init__()
        self.id, self.width_id, self.max_digits = _R(reg), _R(width_reg), int(max_digits)

    def spec(self, dag=False):
        return ("hadamard_int_batched", self.id, self.width_id, self.max_digits, self._cond())


class NoiseTable:
    """Per-trajectory Pauli masks: masks[t] = (xa, xb, xc, za, zb, zc)."""

    def __init__(self, masks):
        import numpy as np
        m = np.ascontiguousarray(np.asarray(masks, dtype=np.uint64).reshape(-1, 6))
        self.n_traj = m.shape[0]
        words = m.reshape(-1)
        bits = max(1, int(np.ceil(np.log2(max(words.size, 2)))))
        padded = np.zeros(1 << bits, dtype=np.uint64)
        padded[: words.size] = words
        self.masks = m
        self.table = QRAMCircuit_qutrit(bits, 64, padded)


class PauliNoise(ElementwiseOperator):
    """Per-trajectory Pauli X then Z errors on three registers, selected by the
    trajectory register's value (batched noisy trajectories)."""

    opcode = "PAULI_NOISE"

    def __init__(self, traj_reg, regs, table: NoiseTable):
        super().__init__()
        if len(regs) != 3:
            raise ValueError("PauliNoise acts on three registers")
        self.traj = _R(traj_reg)
        self.regs = [_R(r) for r in regs]
        self.noise = table
        for j, r in enumerate(self.regs):
            w = System.size_of(r)
            lim = (1 << w) - 1 if w < 64 else (1 << 64) - 1
            if int(table.masks[:, j].max(initial=0)) > lim or int(table.masks[:, j + 3].max(initial=0)) > lim:
                raise SparQInvalid(SQ_ERR_INVALID, f"PauliNoise: a mask of register {r} is wider than its {w} bits")

    def _fill(self, ins, dag):
        ins.reg[0] = self.traj
        for i, r in enumerate(self.regs):
            ins.reg[i + 1] = r
        ins.imm[0] = self.noise.n_traj
        ins.qram = self.noise.table._h.value


class Hadamard_Int_Full(SelfAdjointOperator):
    """H on the whole register (hadamard.cpp:181-338)."""

    def __init__(self, reg):
        super().__init__()
        self.id = _R(reg)

    def spec(self, dag=False):
        return ("hadamard_int_full", self.id, self._cond())


class Hadamard_Bool(SelfAdjointOperator):
    """H on a 1-bit register (hadamard.cpp:340-439)."""

    def __init__(self, reg):
        super().__init__()
        self.out_id = _R(reg)
        if System.size_of(self.out_id) != 1:
            raise ValueError("Hadamard_Bool: size of output register must be 1")

    def spec(self, dag=False):
        return ("hadamard_bool", self.out_id, self._cond())


def _mat8(mat):
    m = [complex(x) for x in mat]
    if len(m) != 4:
        raise ValueError("2x2 matrix needs 4 elements (m00, m01, m10, m11)")
    out = []
    for z in m:
        out += [z.real, z.imag]
    return out


class Rot_Bool(BaseOperator):
    """2x2 unitary on bit `digit` of reg (basic_gates.cpp:74-357); dag applies
    the conjugate transpose. Rot_Bool(reg, mat) uses digit 0."""

    def __init__(self, reg, digit, mat=None):
        super().__init__()
        if mat is None:
            digit, mat = 0, digit
        self.id, self.digit, self.mat = _R(reg), int(digit), [complex(x) for x in mat]
        if self.digit >= System.size_of(self.id):
            raise ValueError("digit out of range of the register")

    def spec(self, dag=False):
        m = self.mat
        if dag:
            m = [m[0].conjugate(), m[2].conjugate(), m[1].conjugate(), m[3].conjugate()]
        return ("rot_bool", self.id, self.digit, _mat8(m), self._cond())


class RX_Bool(Rot_Bool):
    """RX(theta) (basic_gates.cpp:536-553)."""

    def __init__(self, reg, digit, angle=None):
        if angle is None:
            digit, angle = 0, digit
        c, s = math.cos(angle / 2), math.sin(angle / 2)
        super().__init__(reg, digit, [complex(c, 0), complex(0, -s), complex(0, -s), complex(c, 0)])


class RY_Bool(Rot_Bool):
    """RY(theta) (basic_gates.cpp:571-588)."""

    def __init__(self, reg, digit, angle=None):
        if angle is None:
            digit, angle = 0, digit
        c, s = math.cos(angle / 2), math.sin(angle / 2)
        super().__init__(reg, digit, [complex(c, 0), complex(-s, 0), complex(s, 0), complex(c, 0)])


class CondRot_Rational_Bool(BaseOperator):
    """Rotate the 1-bit `out` by 2*pi*in/2^|in| (condrot.cpp:12-152)."""

    def __init__(self, reg_in, reg_out):
        super().__init__()
        self.register_in, self.register_out = _R(reg_in), _R(reg_out)
        if (System.type_of(self.register_in) != StateStorageType.Rational
                or System.type_of(self.register_out) != StateStorageType.Boolean):
            raise ValueError("CondRot_Rational_Bool: input must be Rational and output Boolean")

    def spec(self, dag=False):
        return ("condrot", self.register_in, self.register_out, dag, self._cond())


CondRot_Fixed_Bool = CondRot_Rational_Bool


class CondRot_General_Bool(BaseOperator):
    """2x2 unitary func(v) on the 1-bit `out`, v = value of `in`
    (CondRot_General_Bool_Fast<F>, condrot.h:149-300). `func(v)` returns the
    four elements (m00, m01, m10, m11); it is evaluated on the host for every
    v < 2^width(in) and the table is uploaded. Conditions restrict it to the
    entries that satisfy them."""

    has_dag = False

    def __init__(self, reg_in, reg_out, func):
        super().__init__()
        import numpy as np
        self.in_id, self.out_id = _R(reg_in), _R(reg_out)
        if System.type_of(self.out_id) != StateStorageType.Boolean or System.size_of(self.out_id) != 1:
            raise ValueError("CondRot_General_Bool: output must be a 1-bit Boolean register")
        n = 1 << System.size_of(self.in_id)
        tab = np.zeros((n, 8), dtype=np.float64)
        for v in range(n):
            m = [complex(x) for x in func(v)]
            tab[v] = [m[0].real, m[0].imag, m[1].real, m[1].imag, m[2].real, m[2].imag, m[3].real, m[3].imag]
        self.table = np.ascontiguousarray(tab.reshape(-1))

    @classmethod
    def from_table(cls, reg_in, reg_out, mats):
        """From a list of 2^width(in) matrices (m00, m01, m10, m11); values of
        `in` past the list's end get the identity."""
        n = 1 << System.size_of(_R(reg_in))
        if len(mats) > n:
            raise ValueError("CondRot_General_Bool: more matrices than values of the input register")
        eye = (1, 0, 0, 1)
        return cls(reg_in, reg_out, lambda v: mats[v] if v < len(mats) else eye)

    def spec(self, dag=False):
        return ("condrot_general", self.in_id, self.out_id, self.table, self._cond())


class Rot_GeneralUnitary(BaseOperator):
    """Dense 2^k x 2^k unitary on a k-bit register (rot.cpp:353-477); dag
    applies the conjugate transpose."""

    def __init__(self, reg, mat):
        super().__init__()
        import numpy as np
        self.id = _R(reg)
        m = np.asarray(mat, dtype=np.complex128)
        dim = 1 << System.size_of(self.id)
        if m.shape != (dim, dim):
            raise ValueError("Matrix size does not match the register's size.")
        self.dim = dim
        self.mat = np.ascontiguousarray(m).view(np.float64).reshape(-1).copy()

    def spec(self, dag=False):
        return ("rot_general_unitary", self.id, self.mat, self.dim, self._cond(), dag)


def stateprep_unitary(target):
    """Unitary U with U e0 = target / |target| (rot.cpp:481-519): a complex
    Householder reflection I - 2 v v* / <v, v>, v = psi + phase(psi_0) e0, whose
    first column is multiplied by -phase(psi_0). psi is the target scaled by
    its largest component, then normalised."""
    import numpy as np
    t = np.asarray(target, dtype=np.complex128).reshape(-1)
    if t.size == 0:
        raise ValueError("Cannot prepare an empty vector.")
    if not (np.all(np.isfinite(t.real)) and np.all(np.isfinite(t.imag))):
        raise ValueError("State amplitudes must be finite.")
    scale = max(float(np.max(np.abs(t.real))), float(np.max(np.abs(t.imag))))
    if scale == 0:
        raise ValueError("Cannot prepare the zero vector.")
    v = t / scale
    norm_sq = 0.0
    for x in v:
        norm_sq += x.real * x.real + x.imag * x.imag
    v = v / math.sqrt(norm_sq)
    first_abs = abs(v[0])
    phase = complex(1.0, 0.0) if first_abs == 0 else v[0] / first_abs
    v = v.copy()
    v[0] += phase
    vns = 0.0
    for x in v:
        vns += x.real * x.real + x.imag * x.imag
    n = v.size
    u = np.empty((n, n), dtype=np.complex128)
    for i in range(n):
        for j in range(n):
            e = (1.0 if i == j else 0.0) - (2.0 / vns) * v[i] * v[j].conjugate()
            if j == 0:
                e *= -phase
            u[i, j] = e
    return u


class Rot_GeneralStatePrep(Rot_GeneralUnitary):
    """Prepare `vec` on a register from |0> (rot.cpp:528-564): the state-prep
    unitary above applied with Rot_GeneralUnitary; dag applies its inverse."""

    def __init__(self, reg, vec):
        import numpy as np
        dim = 1 << System.size_of(_R(reg))
        if len(vec) != dim:
            raise ValueError("Matrix size does not match the register's size.")
        super().__init__(reg, stateprep_unitary(np.asarray(vec, dtype=np.complex128)))
        self.vec = list(vec)


class PlusOneAndOverflow(ElementwiseOperator):
    """main = main + 1 mod 2^|main|, and on the wrap overflow = (overflow + 1) % 2;
    dag subtracts (SparQ_Algorithm/src/BlockEncoding/block_encoding_tridiagonal.cpp:20-83)."""

    opcode = "PLUS_ONE_OVERFLOW"

    def __init__(self, main_reg, overflow_reg):
        super().__init__()
        self.main, self.overflow = _R(main_reg), _R(overflow_reg)

    def _fill(self, ins, dag):
        ins.reg[0] = self.main
        ins.reg[1] = self.overflow


SQ_ANGLE_DIV_SQRT_ARCCOS, SQ_ANGLE_ROTATE = 0, 1


class AngleTable:
    """The rational angle words of Div_Sqrt_Arccos_UInt_UInt or
    GetRotateAngle_Int_Int for a set of (lhs, rhs) register pairs, computed
    on the host with the C library exactly as the reference's CPU loop does
    (quantum_arithmetic.cpp:413-432, 458-487) and looked up on the GPU
    (sq_angle_table_create), so that the angle bits in the keys are the
    CPU's."""

    def __init__(self, kind: int, lhs_width: int, rhs_width: int, out_width: int, lhs, rhs):
        import numpy as np
        l = np.ascontiguousarray(np.asarray(lhs, dtype=np.uint64).reshape(-1))
        r = np.ascontiguousarray(np.asarray(rhs, dtype=np.uint64).reshape(-1))
        if l.size != r.size:
            raise ValueError("AngleTable: lhs and rhs differ in length")
        self.kind, self.widths = int(kind), (int(lhs_width), int(rhs_width), int(out_width))
        self.pairs = int(l.size)
        h = ctypes.c_void_p()
        call("sq_angle_table_create", self.kind, *self.widths, l.ctypes.data_as(ctypes.c_void_p),
             r.ctypes.data_as(ctypes.c_void_p), l.size, byref(h))
        self._h = h

    @staticmethod
    def word(kind: int, lhs_width: int, rhs_width: int, out_width: int, lhs: int, rhs: int) -> int:
        w = ctypes.c_uint64()
        call("sq_angle_word", int(kind), int(lhs_width), int(rhs_width), int(out_width), int(lhs), int(rhs), byref(w))
        return w.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                from ._native import lib
                lib().sq_qram_destroy(h)
            except Exception:
                pass
            self._h = None


class _AngleXor(_Regs, SelfAdjointOperator):
    """out ^= angle(lhs, rhs) (XOR-out, self-adjoint). The angle comes from
    `table` (an AngleTable made for these register widths); without one, the
    distinct (lhs, rhs) pairs of the state are read back, their angles
    computed on the host and applied (one round trip)."""

    opcode = "ANGLE_XOR"
    kind = SQ_ANGLE_DIV_SQRT_ARCCOS

    def __init__(self, lhs, rhs, out, table: AngleTable | None = None):
        super().__init__(lhs, rhs, out)
        self.table = table

    def _fill(self, ins, dag):
        _set_regs(ins, *self.regs)
        ins.imm[0] = self.kind
        if self.table is not None:
            ins.qram = self.table._h.value

    def _table_for(self, state: SparseState) -> AngleTable:
        import numpy as np
        regs, _ = state.download()
        pairs = np.unique(regs[:, self.regs[:2]], axis=0) if len(regs) else np.zeros((0, 2), dtype=np.uint64)
        return AngleTable(self.kind, *(System.size_of(r) for r in self.regs), pairs[:, 0], pairs[:, 1])

    def __call__(self, state: SparseState) -> None:
        if self.table is None:
            op = type(self)(*self.regs, table=self._table_for(state))
            self.copy_control_conditions_to(op)
            _run(state, op.spec(False))
            return
        super().__call__(state)

    def dag(self, state: SparseState) -> None:
        self(state)


class Div_Sqrt_Arccos_UInt_UInt(_AngleXor):
    """out ^= get_rational(acos(sqrt(lhs / rhs)) / (2 pi)) (quantum_arithmetic.cpp:413-432)."""

    kind = SQ_ANGLE_DIV_SQRT_ARCCOS


class GetRotateAngle_Int_Int(_AngleXor):
    """out ^= get_rational(atan2(rhs, lhs) / (2 pi) in [0, 1)), 0.25 / 0.75 for
    lhs = 0, of the two's-complement values (quantum_arithmetic.cpp:458-487)."""

    kind = SQ_ANGLE_ROTATE


class BitGather(ElementwiseOperator):
    """A bit permutation of one register: the bits of `mask` move, in
    ascending order, to the lowest bits and the others, in order, above
    them; dag moves them back. It is the index map of Hadamard_Partial
    (map_position / from_map_position, hadamard.cpp:443-466)."""

    opcode = "BIT_GATHER"

    def __init__(self, reg, mask: int):
        super().__init__()
        self.id = _R(reg)
        self.mask = int(mask)

    def _fill(self, ins, dag):
        ins.reg[0] = self.id
        ins.imm[0] = self.mask


class Hadamard_Partial(SelfAdjointOperator):
    """H on a set of bit positions of a register (hadamard.cpp:470-712): one
    position as the reference's active path (pairs of entries equal except
    that bit), several as H on each of them (the reference's
    Hadamard_Partial::operate over groups equal outside the set)."""

    def __init__(self, reg, positions):
        super().__init__()
        self.id = _R(reg)
        self.positions = sorted({int(p) for p in positions})

    def spec(self, dag=False):
        return ("hadamard_partial", self.id, self.positions, self._cond())


class ClearZero(SelfAdjointOperator):
    """Drop entries with |a|^2 < eps (system_operations.cpp:371-382)."""

    def __init__(self, eps: float | None = None):
        super().__init__()
        self.eps = eps

    def spec(self, dag=False):
        from .core import get_clearzero_default_eps
        return ("clear_zero", get_clearzero_default_eps() if self.eps is None else float(self.eps))


class Normalize(SelfAdjointOperator):
    """a *= 1/sqrt(sum |a|^2) (dark_magic.cpp:11-32)."""

    def spec(self, dag=False):
        return ("normalize",)


class PartialTraceSelect:
    """Keep the entries whose registers hold the selected values, scale them by
    1/sqrt(p) and return that factor (+inf if none is left)
    (partial_trace.cpp:148-185). Built from {reg: value} or (regs, values)."""

    def __init__(self, regs, values=None):
        if values is None:
            items = list(dict(regs).items())
        else:
            items = list(zip(regs, values))
        self.regs = [_R(r) for r, _ in items]
        self.values = [int(v) & U64 for _, v in items]

    def __call__(self, state: SparseState) -> float:
        import numpy as np
        r = np.array(self.regs, dtype=np.uint32)
        v = np.array(self.values, dtype=np.uint64)
        out = c_double()
        call("sq_partial_trace_select", state._h, r.ctypes.data_as(ctypes.c_void_p),
             v.ctypes.data_as(ctypes.c_void_p), len(self.regs), byref(out))
        return out.value

    def spec(self, dag=False):
        return ("partial_trace_select", self.regs, self.values)


class PartialTraceSelectRange:
    """The same for lo <= value(reg) <= hi (partial_trace.cpp:187-225)."""

    def __init__(self, reg, select_range):
        self.reg = _R(reg)
        self.lo, self.hi = int(select_range[0]), int(select_range[1])

    def __call__(self, state: SparseState) -> float:
        out = c_double()
        call("sq_partial_trace_select_range", state._h, self.reg, self.lo, self.hi, byref(out))
        return out.value

    def spec(self, dag=False):
        return ("partial_trace_select_range", self.reg, self.lo, self.hi)


# ---------------------------------------------------------------------- register surgery
class AddRegister:
    """New zero-valued register (system_operations.cpp:252-272); returns its id."""

    def __init__(self, name: str, type_: StateStorageType, size: int):
        if size > 64:
            raise ValueError("register size > 64")
        self.name, self.type, self.size = name, type_, int(size)

    def __call__(self, state: SparseState) -> int:
        return System.add_register_synchronous(self.name, self.type, self.size, state)


class AddRegisterWithHadamard:
    """New register of `size` bits, every entry copied once per value of it
    with the amplitude unchanged: no 2^(-size/2) factor, no prune
    (system_operations.cpp:281-305); returns its id."""

    def __init__(self, name: str, type_: StateStorageType, size: int):
        if size > 64:
            raise ValueError("register size > 64")
        self.name, self.type, self.size = name, type_, int(size)

    def __call__(self, state: SparseState) -> int:
        rid = c_uint32()
        call("sq_add_register_with_hadamard", state._h, int(self.type), self.size, byref(rid))
        System._set_name(rid.value, self.name)
        return rid.value


class CheckNormalization:
    """Raise (the reference's throw_bad_result) unless |sum |a|^2 - 1| <
    threshold (debugger.cpp:12-27); the state is left as it is."""

    def __init__(self, threshold: float = 1e-5):
        self.threshold = float(threshold)

    def __call__(self, state: SparseState) -> None:
        f = state.norm_sq()
        if math.isnan(f) or not abs(f - 1.0) < self.threshold:
            raise SparQError(SQ_ERR_BAD_RESULT, f"State is not normalized (sum |a|^2 = {f!r}).")

    dag = __call__


class CheckNan:
    """Raise (throw_bad_result) if an amplitude is NaN (debugger.cpp:52-66):
    the sum of |a|^2 is NaN exactly then."""

    def __call__(self, state: SparseState) -> None:
        if math.isnan(state.norm_sq()):
            raise SparQError(SQ_ERR_BAD_RESULT, "NaN amplitude in the state.")

    dag = __call__


class RemoveRegister:
    """Zero the register in every entry and deactivate it (system_operations.cpp:310-330)."""

    def __init__(self, reg):
        self.register_id = _R(reg)

    def __call__(self, state: SparseState) -> None:
        call("sq_remove_register_sync", state._h, self.register_id)


class SplitRegister:
    """Low `second_size` bits of `first` become register `second_name`
    (system_operations.cpp:124-158); returns the new id."""

    def __init__(self, first, second_name: str, second_size: int):
        self.first, self.second_name, self.second_size = first, second_name, int(second_size)

    def __call__(self, state: SparseState) -> int:
        rid = c_uint32()
        call("sq_split_register", state._h, _R(self.first), self.second_size, byref(rid))
        System._set_name(rid.value, self.second_name)
        return rid.value


class CombineRegister:
    """first = first << |second| | second; second removed (system_operations.cpp:170-203)."""

    def __init__(self, first, second):
        self.first, self.second = first, second

    def __call__(self, state: SparseState) -> int:
        f = _R(self.first)
        call("sq_combine_register", state._h, f, _R(self.second))
        return f


def get_output(state: SparseState, zero_regs, idx_regs):
    """Dense read-out of a post-selected block (GetOutput,
    qda_fundamental.cpp:123-166): the entries whose `zero_regs` all hold 0
    land at index concat(idx_regs) (first register lowest); returns (complex
    vector of 2^(sum of index widths), their total probability p), the vector
    scaled by 1/sqrt(p) unless |p - 1| < 1e-14. The state is unchanged."""
    import numpy as np
    z = np.array([_R(r) for r in zero_regs], dtype=np.uint32)
    ix = np.array([_R(r) for r in idx_regs], dtype=np.uint32)
    n = 1 << sum(System.size_of(int(r)) for r in ix)
    out = np.zeros(2 * n, dtype=np.float64)
    prob = c_double()
    call("sq_get_output", state._h, z.ctypes.data_as(ctypes.c_void_p), len(z), ix.ctypes.data_as(ctypes.c_void_p),
         len(ix), out.ctypes.data_as(ctypes.c_void_p), n, byref(prob))
    return out.view(np.complex128), prob.value


def add_systems(current: SparseState, new_state: SparseState, coef: float = 1.0) -> None:
    """current += coef * new_state, equal keys merged, |a|^2 < epsilon dropped
    (system_operations.h:157-175)."""
    call("sq_add_systems", current._h, new_state._h, float(coef))


def synchronize() -> None:
    call("sq_synchronize")
