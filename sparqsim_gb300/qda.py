"""Discrete-adiabatic (QDA) linear-system walks on the GB300 engine.

The walk of Costa et al., "Optimal scaling quantum linear-systems solver via
discrete adiabatic theorem", PRX Quantum 3, 040303 (2022), in the circuit
form SparQ uses, so that a walk is the same operator sequence as the
reference's:

- the schedule f(s) (Eq. 69) and the 2x2 rotation R_s
  (SparQ_Algorithm/include/DiscreteAdiabatic/qda_fundamental.h:53-90);
- the block encoding of H(s) (qda_fundamental.h:92-130), one walk step
  W_s = R . U_H(s) . i (qda_fundamental.h:344-470);
- the tridiagonal block encoding of A = alpha I + beta (S + S^T)
  (SparQ_Algorithm/include/BlockEncoding/block_encoding_tridiagonal.h:33-108,
  src/BlockEncoding/block_encoding_tridiagonal.cpp:84-130): an LCU over
  {I, +1 shift, -1 shift, annihilation} prepared on two ancilla qubits;
- the read-out of GetOutput (qda_fundamental.h:556-660,
  qda_fundamental.cpp:123-166): post-selection on anc_UA = anc_2 = anc_3 = 0,
  a dense vector indexed main + anc_1 * n + anc_4 * 2n whose block
  anc_1 = 1, anc_4 = 0 holds the solution.

Conditions on a composite operator apply to every operator inside it (the
reference partitions the state by the conditions, applies the inside, and
merges back; per-entry conditions give the same result because no inside
operator writes a condition register).

Every operator goes through a runner (`run.op(op)`, `run.split(...)`,
`run.combine(...)`), so the same walk drives a GPU state alone or a GPU state
and the CPU oracle side by side.
"""
from __future__ import annotations

import copy
import math

import numpy as np

from .core import SparseState, System
from .operators import (CombineRegister, CondRot_General_Bool, ElementwiseOperator, GlobalPhase, Hadamard_Bool,
                        Hadamard_Int_Full, PlusOneAndOverflow, Reflection_Bool, Rot_Bool, Rot_GeneralStatePrep,
                        SplitRegister, X_Bool, _run)
from . import core


# ------------------------------------------------------------------ schedule
def schedule_f(s: float, kappa: float, p: float) -> float:
    """f(s) = kappa/(kappa-1) (1 - (1 + s (kappa^(p-1) - 1))^(1/(1-p))), in [0, 1]."""
    if kappa == 1:
        return s
    inner = 1 + s * (kappa ** (p - 1) - 1)
    if inner <= 0:
        return 1.0
    return max(0.0, min(1.0, kappa / (kappa - 1) * (1 - inner ** (1 / (1 - p)))))


def rotation_R(fs: float) -> list:
    """R_s = c [[1 - f, f], [f, f - 1]], c = 1 / sqrt((1 - f)^2 + f^2)."""
    c = 1.0 / math.sqrt((1 - fs) ** 2 + fs ** 2)
    return [complex(c * (1 - fs), 0), complex(c * fs, 0), complex(c * fs, 0), complex(c * (fs - 1), 0)]


# ------------------------------------------------------------------ runners
class Runner:
    """Applies operators to one GPU state.

    Consecutive elementwise operators are queued and applied as one fused
    program (one pass over the entries instead of one per operator: each
    entry maps on its own under every one of them, so the order within the
    run is kept entry by entry). Anything else (a split of amplitudes, a
    register change, ClearZero, Normalize) applies the queue first, and
    `flush()` applies it on demand; the walk drivers flush at the end of each
    step, before the state is read. `fuse=False` applies every operator as it
    comes."""

    def __init__(self, state: SparseState, fuse: bool = True):
        self.state = state
        self.fuse = fuse
        self._queue = []

    def op(self, o, dag: bool = False):
        if self.fuse and isinstance(o, ElementwiseOperator):
            if dag and not o.has_dag:
                raise NotImplementedError("Dagger is not implemented.")
            self._queue.append(o.instr(dag and not o.self_adjoint))
            return
        self.flush()
        (o.dag if dag else o)(self.state)

    def flush(self):
        if self._queue:
            q, self._queue = self._queue, []
            _run(self.state, ("prog", q))

    def split(self, first, name: str, size: int):
        self.flush()
        return SplitRegister(first, name, size)(self.state)

    def combine(self, first, second):
        self.flush()
        CombineRegister(first, second)(self.state)

    def add_register(self, name: str, type_, size: int):
        from .operators import AddRegister
        self.flush()
        return AddRegister(name, type_, size)(self.state)

    def remove_register(self, reg):
        from .operators import RemoveRegister
        self.flush()
        RemoveRegister(reg)(self.state)


def flush(run):
    """Apply whatever a runner has queued (runners without a queue: nothing)."""
    f = getattr(run, "flush", None)
    if f is not None:
        f()


def _with(op, outer):
    """A copy of `op` that also carries the conditions of `outer`."""
    if outer is None or not outer.has_condition():
        return op
    o = copy.copy(op)
    o.condition_variable_nonzeros = list(op.condition_variable_nonzeros) + list(outer.condition_variable_nonzeros)
    o.condition_variable_all_ones = list(op.condition_variable_all_ones) + list(outer.condition_variable_all_ones)
    o.condition_variable_by_bit = list(op.condition_variable_by_bit) + list(outer.condition_variable_by_bit)
    o.condition_variable_by_value = list(op.condition_variable_by_value) + list(outer.condition_variable_by_value)
    return o


class Composite(core.Controllable):
    """An operator made of other operators; its conditions apply to each."""

    def __init__(self):
        self._init_controls()

    def _do(self, run, op, dag=False, outer=None):
        run.op(_with(op, outer if outer is not None else self), dag)

    def conditioned(self, outer):
        """A copy carrying `outer`'s conditions besides its own."""
        o = copy.copy(self)
        o._init_controls()
        self.copy_control_conditions_to(o)
        o.condition_variable_all_ones = list(o.condition_variable_all_ones) + list(outer.condition_variable_all_ones)
        o.condition_variable_nonzeros = list(o.condition_variable_nonzeros) + list(outer.condition_variable_nonzeros)
        o.condition_variable_by_bit = list(o.condition_variable_by_bit) + list(outer.condition_variable_by_bit)
        o.condition_variable_by_value = list(o.condition_variable_by_value) + list(outer.condition_variable_by_value)
        return o


# ------------------------------------------------------------------ block encodings
class BlockEncodingTridiagonal(Composite):
    """Block encoding of A = alpha I + beta (S + S^T) on `main_reg`, with a
    4-bit ancilla register `anc_UA` (two LCU qubits, the overflow bit and one
    more). The LCU amplitudes are (sqrt|alpha|, sqrt|beta|, sqrt|beta|,
    sqrt(s - |alpha| - 2|beta|)) / sqrt(s), s = sqrt(N alpha^2 + 2 (N-1) beta^2)
    (block_encoding_tridiagonal.cpp:84-130)."""

    def __init__(self, main_reg, anc_UA, alpha: float, beta: float):
        super().__init__()
        self.main_reg, self.anc_UA, self.alpha, self.beta = main_reg, anc_UA, float(alpha), float(beta)
        n = 1 << System.size_of(main_reg)
        norm_f = math.sqrt(n * abs(alpha) ** 2 + 2 * (n - 1) * abs(beta) ** 2)
        p0 = math.sqrt(abs(alpha)) / math.sqrt(norm_f)
        p1 = math.sqrt(abs(beta)) / math.sqrt(norm_f)
        p3 = math.sqrt(max(0.0, 1.0 - (abs(alpha) + 2 * abs(beta)) / norm_f))
        self.prep = [complex(p0, 0), complex(p1, 0), complex(p1, 0), complex(p3, 0)]
        self.norm = norm_f

    def _body(self, run, dag: bool):
        ov = run.split(self.anc_UA, "overflow", 1)
        other = run.split(self.anc_UA, "other", 1)
        prep = Rot_GeneralStatePrep(self.anc_UA, self.prep)
        self._do(run, prep)
        first, second = (1, 2) if not dag else (2, 1)
        self._do(run, PlusOneAndOverflow(self.main_reg, ov).conditioned_by_value(self.anc_UA, first))
        if self.beta < 0:
            self._do(run, Reflection_Bool([self.main_reg, ov], False).conditioned_by_value(self.anc_UA, first))
            self._do(run, Reflection_Bool([self.main_reg, ov], False).conditioned_by_value(self.anc_UA, second))
        self._do(run, PlusOneAndOverflow(self.main_reg, ov).conditioned_by_value(self.anc_UA, second), dag=True)
        self._do(run, X_Bool(other, 0).conditioned_by_all_ones(self.anc_UA))
        self._do(run, prep, dag=True)
        run.combine(self.anc_UA, other)
        run.combine(self.anc_UA, ov)

    def apply(self, run):
        self._body(run, False)

    def apply_dag(self, run):
        self._body(run, True)


class StatePrepHadamard(Composite):
    """|b> = uniform superposition: Hadamard on the whole main register."""

    def __init__(self, main_reg):
        super().__init__()
        self.main_reg = main_reg

    def apply(self, run):
        self._do(run, Hadamard_Int_Full(self.main_reg))

    def apply_dag(self, run):
        self._do(run, Hadamard_Int_Full(self.main_reg))


class BlockEncodingHs(Composite):
    """Block encoding of H(s) = (1 - f) H_0 + f H_1 (qda_fundamental.h:92-130).

    Batched: with `inst_reg`, the state holds several walks of the same
    system side by side, told apart by the value of `inst_reg`, and `fs` is a
    list with one f(s) per value; the only operator that depends on s, the
    rotation R_s of anc_2, then rotates each walk by its own matrix
    (CondRot_General_Bool on inst_reg). Every other operator is the same for
    all walks and maps each walk's entries among themselves."""

    def __init__(self, enc_A, enc_b, main_reg, anc_UA, anc_1, anc_2, anc_3, anc_4, fs, inst_reg=None):
        super().__init__()
        self.enc_A, self.enc_b = enc_A, enc_b
        self.main_reg, self.anc_UA = main_reg, anc_UA
        self.a1, self.a2, self.a3, self.a4 = anc_1, anc_2, anc_3, anc_4
        self.inst = inst_reg
        fs = list(fs) if isinstance(fs, (list, tuple)) else [fs]
        if inst_reg is None and len(fs) != 1:
            raise ValueError("BlockEncodingHs: several f(s) need an instance register")
        self.R = [rotation_R(f) for f in fs]

    def _rot(self):
        """R_s on anc_2: Rot_Bool when every walk is at the same f(s) (the
        plain walk; at s = 0 R is diagonal and Rot_Bool's in-place form makes
        no new entries), else one matrix per value of the instance register."""
        if self.inst is None or all(r == self.R[0] for r in self.R):
            return Rot_Bool(self.a2, self.R[0])
        return CondRot_General_Bool.from_table(self.inst, self.a2, self.R)

    def apply(self, run):
        a1, a2, a3, a4 = self.a1, self.a2, self.a3, self.a4
        d = self._do
        d(run, Hadamard_Bool(a3))
        self.enc_b.conditioned(self).apply_dag(run)
        d(run, X_Bool(a1, 0))
        d(run, Reflection_Bool(self.main_reg, True).conditioned_by_all_ones([a1, a3, a4]))
        d(run, X_Bool(a1, 0))
        self.enc_b.conditioned(self).apply(run)
        d(run, X_Bool(a4, 0))
        d(run, self._rot().conditioned_by_all_ones(a4))
        d(run, X_Bool(a4, 0))
        d(run, Hadamard_Bool(a2).conditioned_by_all_ones(a4))
        enc = self.enc_A.conditioned(self)
        enc.condition_variable_all_ones = list(enc.condition_variable_all_ones) + [System.resolve(a1),
                                                                                  System.resolve(a2)]
        enc.apply(run)
        d(run, X_Bool(a1, 0).conditioned_by_all_ones(a2))
        d(run, Reflection_Bool(a2, True).conditioned_by_all_ones(a1))
        enc.apply_dag(run)
        d(run, X_Bool(a4, 0))
        d(run, Hadamard_Bool(a2).conditioned_by_all_ones(a4))
        d(run, X_Bool(a4, 0))
        d(run, self._rot().conditioned_by_all_ones(a4))
        d(run, X_Bool(a4, 0))
        self.enc_b.conditioned(self).apply_dag(run)
        d(run, X_Bool(a1, 0))
        d(run, Reflection_Bool(self.main_reg, True).conditioned_by_all_ones([a1, a3, a4]))
        d(run, X_Bool(a1, 0))
        self.enc_b.conditioned(self).apply(run)
        d(run, Hadamard_Bool(a3))


class WalkS(Composite):
    """One walk step at s: U_H(s), then the reflection about anc_UA = anc_2 =
    anc_3 = 0, then the global phase i (qda_fundamental.h:344-470)."""

    def __init__(self, enc_A, enc_b, main_reg, anc_UA, anc_1, anc_2, anc_3, anc_4, s, kappa: float,
                 p: float, inst_reg=None):
        super().__init__()
        if isinstance(s, (list, tuple)):  # batched: one s per value of inst_reg
            self.fs = [schedule_f(x, kappa, p) for x in s]
        else:
            self.fs = schedule_f(s, kappa, p)
        self.enc_Hs = BlockEncodingHs(enc_A, enc_b, main_reg, anc_UA, anc_1, anc_2, anc_3, anc_4, self.fs,
                                      inst_reg=inst_reg)
        self.refl = [anc_UA, anc_2, anc_3]

    def apply(self, run):
        self.enc_Hs.conditioned(self).apply(run)
        self._do(run, Reflection_Bool(self.refl, False))
        run.op(GlobalPhase(complex(0, 1)))  # outside the conditions, as in the reference
        flush(run)


# ------------------------------------------------------------------ driver
REGS = ("main_reg", "anc_UA", "anc_1", "anc_2", "anc_3", "anc_4")


def tridiagonal_matrix(n: int, alpha: float, beta: float) -> np.ndarray:
    """alpha on the diagonal, beta on the first off-diagonals."""
    return alpha * np.eye(n) + beta * (np.eye(n, k=1) + np.eye(n, k=-1))


def declare_registers(run, n_bits: int):
    """main register (n bits), anc_UA (4 bits), anc_1..anc_4 (1 bit each)."""
    from .operators import AddRegister
    flush(run)
    state = run.state
    AddRegister("main_reg", core.UnsignedInteger, n_bits)(state)
    AddRegister("anc_UA", core.UnsignedInteger, 4)(state)
    for a in ("anc_1", "anc_2", "anc_3", "anc_4"):
        AddRegister(a, core.Boolean, 1)(state)


def read_solution(state: SparseState, n_bits: int):
    """Amplitudes of the main register where anc_UA = anc_2 = anc_3 = anc_4 = 0
    and anc_1 = 1, and the probability of that sector. The post-selection
    runs on the GPU (PartialTraceSelect, which also renormalises the state);
    only the selected entries are read back."""
    from .operators import PartialTraceSelect
    f = PartialTraceSelect({"anc_UA": 0, "anc_1": 1, "anc_2": 0, "anc_3": 0, "anc_4": 0})(state)
    x = np.zeros(1 << n_bits, dtype=np.complex128)
    if not np.isfinite(f) or f == 0:
        return x, 0.0
    regs, amps = state.download()
    main = System.resolve("main_reg")
    np.add.at(x, regs[:, main].astype(np.int64), amps / f)
    return x, float(1.0 / (f * f))


class GetOutput:
    """The QDA read-out (qda_fundamental.h:556-660; qda_fundamental.cpp:123-166):
    post-selects anc_UA = anc_3 = anc_2 = 0 and returns (the 4n amplitudes
    indexed main + anc_1 * n + anc_4 * 2n, scaled to unit norm unless already
    within 1e-14 of it; the post-selected probability). The state is left as
    it is; the scatter and the probability sum run on the GPU. `is_PD` is
    accepted and unused, as in the reference."""

    def __init__(self, main_reg, anc_UA, anc_4, anc_3, anc_2, anc_1, is_PD: bool = False):
        self.zero = [System.resolve(r) for r in (anc_UA, anc_3, anc_2)]
        self.idx = [System.resolve(r) for r in (main_reg, anc_1, anc_4)]

    def __call__(self, state: SparseState):
        from .operators import get_output
        return get_output(state, self.zero, self.idx)


def walk_sequence(run, n_bits: int, alpha: float, beta: float, kappa: float, p: float, steps: int,
                  first: int = 0, clear_zero=None):
    """Walk steps first..steps-1 of the schedule s = n / steps."""
    enc_A = BlockEncodingTridiagonal("main_reg", "anc_UA", alpha, beta)
    enc_b = StatePrepHadamard("main_reg")
    for n in range(first, steps):
        WalkS(enc_A, enc_b, *REGS, n / steps, kappa, p).apply(run)
        if clear_zero is not None:
            run.op(clear_zero)


def solve_tridiagonal(n_bits: int, alpha: float, beta: float, p: float = 0.5, steps: int | None = None,
                      step_rate: float = 0.2, kappa: float | None = None):
    """Run the QDA walk for A = alpha I + beta (S + S^T), b uniform; returns
    (normalised solution amplitudes, success probability, fidelity with the
    classical solution, kappa, steps)."""
    from .operators import ClearZero
    n = 1 << n_bits
    A = tridiagonal_matrix(n, alpha, beta)
    enc_norm = math.sqrt(n * alpha ** 2 + 2 * (n - 1) * beta ** 2)
    if kappa is None:
        kappa = float(min(np.linalg.cond(A / enc_norm) if n <= 4096 else 1e9, 10.0))
    if steps is None:
        steps = int(step_rate * 2305 * kappa)
        steps += steps % 2
    System.clear()
    state = SparseState()
    run = Runner(state)
    declare_registers(run, n_bits)
    run.op(Hadamard_Int_Full("main_reg"))
    run.op(ClearZero())
    walk_sequence(run, n_bits, alpha, beta, kappa, p, steps, clear_zero=ClearZero())
    x, prob = read_solution(state, n_bits)
    b = np.ones(n) / math.sqrt(n)
    x_ref = np.linalg.solve(A, b)
    x_ref /= np.linalg.norm(x_ref)
    xn = x / max(np.linalg.norm(x), 1e-300)
    fid = float(abs(np.vdot(xn, x_ref)) ** 2)
    return xn, prob, fid, kappa, steps
