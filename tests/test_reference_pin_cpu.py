"""The oracle pinned against the reference's own CPU operators.

oracle/build_reference.py compiles SparQ/src/*.cpp of the reference checkout,
unmodified, with a stand-in for the header of its absent submodule
(oracle/refshim/) and a C driver (oracle/reference_driver.cpp), into
oracle/_ref/libsparq_ref.so. Each test runs the same operation on the same
seeded state in the oracle (oracle/sparq_oracle.cpp) and in the reference,
and requires the two states to be equal bit for bit: the same entries, and
amplitudes equal to the last bit (no tolerance). Where the reference checkout
is absent (the GPU machine), the file is skipped: the pin is a property of the
oracle, checked where the reference can be built.

What the pin covers: every elementwise opcode the reference has one operator
for (with and without conditions, and the adjoints), the noise-free QRAM
load, Hadamard_Int / Hadamard_Int_Full / Hadamard_Bool / Hadamard_Partial,
Rot_Bool (general, diagonal, off-diagonal), CondRot_Rational_Bool,
CondRot_General_Bool_Fast, Phase_Bool, GlobalPhase, ClearZero, Normalize,
SplitRegister and CombineRegister. What it rests on: the stand-in's helpers
(the submodule's two's complement, masks, epsilon, 1/sqrt 2 and the
sort-merge of add_systems), which the oracle restates the same way.
"""
from __future__ import annotations

import ctypes
import math
from ctypes import POINTER, byref, c_double, c_int, c_uint32, c_uint64, c_void_p

import numpy as np
import pytest

from oracle import build_reference

pytestmark = pytest.mark.skipif(not build_reference.available(), reason="reference checkout absent")

GEN, U, S, B, R = 0, 1, 2, 3, 4  # register types (SQ_GENERAL ...)


def load_reference_library():
    path = build_reference.build()
    lib = ctypes.CDLL(str(path))
    lib.ref_last_error.restype = ctypes.c_char_p
    lib.ref_state_new.restype = c_void_p
    lib.ref_state_free.argtypes = [c_void_p]
    lib.ref_state_size.restype = c_uint64
    lib.ref_state_size.argtypes = [c_void_p]
    lib.ref_set_clearzero_eps.argtypes = [c_double]
    lib.ref_clear_zero.argtypes = [c_void_p, c_double]
    for name in ("ref_state_set", "ref_state_get", "ref_apply", "ref_qram_load", "ref_hadamard_int",
                 "ref_hadamard_int_full", "ref_hadamard_bool", "ref_hadamard_partial", "ref_rot_bool",
                 "ref_condrot", "ref_condrot_general", "ref_normalize", "ref_split_register",
                 "ref_combine_register"):
        getattr(lib, name).restype = c_int
    lib.ref_state_set.argtypes = [c_void_p, c_uint64, c_void_p, c_uint32, c_void_p]
    lib.ref_state_get.argtypes = [c_void_p, c_void_p, c_uint32, c_void_p]
    return lib


@pytest.fixture(scope="module")
def ref():
    return load_reference_library()


class Both:
    """One state in the oracle and the same state in the reference."""

    def __init__(self, ref):
        from oracle import oracle as O
        from sparqsim_gb300._native import SqCond, SqInstr
        self.O, self.R, self.SqInstr, self.SqCond = O, ref, SqInstr, SqCond
        O.clear()
        self._chk(ref.ref_clear())
        O.set_clearzero_eps(1e-14)
        self._chk(ref.ref_set_clearzero_eps(1e-14))
        self.ost = O.OracleState()
        self.rst = ref.ref_state_new()

    def __del__(self):
        if getattr(self, "rst", None):
            self.R.ref_state_free(self.rst)
            self.rst = None

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError(self.R.ref_last_error().decode())

    def reg(self, type_, width):
        a = self.O.add_register(type_, width)
        r = c_uint32()
        self._chk(self.R.ref_add_register(type_, width, byref(r)))
        assert a == r.value
        return a

    def nregs(self):
        return self.O.register_count()

    def start(self, regs, amps):
        regs = np.ascontiguousarray(regs, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.complex128)
        self.ost.set(regs, amps)
        self._chk(self.R.ref_state_set(self.rst, len(amps), regs.ctypes.data, regs.shape[1], amps.ctypes.data))

    def states(self):
        n = self.nregs()
        o_regs, o_amps = self.ost.get(n)
        m = self.R.ref_state_size(self.rst)
        r_regs = np.zeros((m, max(n, 1)), dtype=np.uint64)
        r_amps = np.zeros(m, dtype=np.complex128)
        if m:
            self._chk(self.R.ref_state_get(self.rst, r_regs.ctypes.data, n, r_amps.ctypes.data))
        return (o_regs, o_amps), (r_regs[:, :n], r_amps)

    def compare(self):
        """Same entries, amplitudes equal bit for bit (canonical order)."""
        (orr, oa), (rr, ra) = self.states()
        ids = self.O.active_ids()
        assert len(oa) == len(ra), (len(oa), len(ra))
        ok, oa_ = self.O.canonical(orr, oa, ids)
        rk, ra_ = self.O.canonical(rr, ra, ids)
        assert np.array_equal(ok, rk)
        assert np.array_equal(oa_.view(np.uint64), ra_.view(np.uint64)), np.max(np.abs(oa_ - ra_))
        return len(oa)

    # ---------------------------------------------------------------- operations
    def cond(self, conds=()):
        c = self.SqCond()
        for i, (kind, reg, param) in enumerate(conds):
            c.c[i].kind, c.c[i].reg, c.c[i].param = kind, reg, param
        c.count = len(conds)
        return c

    def instr(self, op, regs=(), imm=(), dag=False, conds=()):
        from sparqsim_gb300._native import OP
        ins = self.SqInstr()
        ins.op = OP[op]
        ins.dag = 1 if dag else 0
        for i, r in enumerate(regs):
            ins.reg[i] = r
        for i, v in enumerate(imm):
            ins.imm[i] = v
        ins.cond = self.cond(conds)
        arr = (self.SqInstr * 1)(ins)
        self.O._chk(self.O.lib().sqo_apply(self.ost.h, arr, 1))
        self._chk(self.R.ref_apply(c_void_p(self.rst), arr, 1))

    def call(self, oracle_fn, ref_fn, *args):
        self.O._chk(getattr(self.O.lib(), oracle_fn)(self.ost.h, *args))
        self._chk(getattr(self.R, ref_fn)(c_void_p(self.rst), *args))


def random_state(rng, widths, n, complex_amps=True):
    cols = [rng.integers(0, 1 << w, n, dtype=np.uint64) if w < 64 else rng.integers(0, 2 ** 63, n, dtype=np.uint64)
            for w in widths]
    regs = np.unique(np.stack(cols, axis=1), axis=0)
    amps = rng.normal(size=len(regs)) + (1j * rng.normal(size=len(regs)) if complex_amps else 0)
    return regs, amps / np.linalg.norm(amps)


COND_NONZERO, COND_ALL_ONES, COND_BIT, COND_VALUE = 0, 1, 2, 3

UNSIGNED3 = ["ADD_UINT_UINT", "SUB_UINT_UINT", "MUL_UINT_UINT", "DIV_UINT_UINT", "AND_UINT_UINT", "OR_UINT_UINT",
             "XOR_UINT_UINT"]


@pytest.mark.parametrize("seed", [0, 1])
def test_elementwise_opcodes(ref, seed):
    """Every arithmetic opcode on registers of the types the reference's
    constructors require, unconditioned and under three condition sets, the
    in-place ones forward and adjoint."""
    b = Both(ref)
    rng = np.random.default_rng(100 + seed)
    widths = [7, 7, 12, 5, 9, 7, 7, 1, 1]
    types = [U, U, U, U, S, S, U, B, B]
    a, a2, c, d, s1, s2, m, f1, f2 = [b.reg(t, w) for t, w in zip(types, widths)]
    b.start(*random_state(rng, widths, 800))
    conds = [(), ((COND_BIT, d, 2),), ((COND_NONZERO, a, 0), (COND_VALUE, f1, 1)), ((COND_ALL_ONES, f2, 0),)]
    for k, cd in enumerate(conds):
        for op in UNSIGNED3:
            b.instr(op, (a, d, c), conds=cd)
        b.instr("LESS_UINT_UINT", (a, d, f1), conds=cd)
        b.instr("LESS_SINT_SINT", (s1, s2, f2), conds=cd)
        b.instr("GETMID_UINT_UINT", (a, a2, m), conds=cd)
        b.instr("NEG_UINT", (a, c), conds=cd)
        b.instr("ABS_SINT", (s1, c), conds=cd)
        b.instr("SQRT_UINT", (c, d), conds=cd)
        b.instr("ISZERO_UINT", (d, f1), conds=cd)
        b.instr("NEGATIVE_SINT", (s2, f2), conds=cd)
        b.instr("ASSIGN", (d, c), conds=cd)
        b.instr("CARRY_UINT_UINT", (a, d, c, f1), conds=cd)
        b.instr("OVERFLOW_SINT_SINT", (s1, s2, c, f2), conds=cd)
        b.instr("MULOVERFLOW_UINT_UINT", (a, d, c, f1), conds=cd)
        b.instr("SELECT_BOOL", (f1, a, d, c), conds=cd)
        b.instr("COMPARE_UINT_UINT", (a, d, f1, f2), conds=cd)
        b.compare()
        b.instr("FLIP_BOOLS", (d,), conds=cd)
        b.instr("SWAP_BOOL_BOOL", (a, d), (3, 1), conds=cd)
        for dag in (False, True):
            b.instr("SHIFT_LEFT", (c,), (3 + k,), dag=dag, conds=cd)
            b.instr("SHIFT_RIGHT", (a,), (2,), dag=dag, conds=cd)
            b.instr("ADD_MULT_UINT_CONST", (a, 0, c), (77 + k,), dag=dag, conds=cd)
            b.instr("ADD_UINT_UINT_INPLACE", (a, c), dag=dag, conds=cd)
            b.instr("ADD_CONST_INPLACE", (c,), (1000 + k,), dag=dag, conds=cd)
            b.instr("ADD_ANYINT_INPLACE", (c, s1), dag=dag, conds=cd)
            b.compare()
        b.instr("MULT_UINT_CONST", (a, 0, c), (13,), conds=cd)
        b.instr("ADD_UINT_CONST", (d, 0, c), (5,), conds=cd)
        b.instr("SWAP_GENERAL", (a, a2), conds=cd)
        b.instr("X_BOOL", (c,), (4,), conds=cd)
        b.instr("Y_BOOL", (a,), (1,), conds=cd)
        b.instr("REFLECTION_BOOL", (), ((1 << f1) | (1 << d), k & 1), conds=cd)
        b.instr("ZERO_COND_PHASE_FLIP", (), ((1 << d) | (1 << f2),), conds=cd)
        b.compare()


def test_angle_operators(ref):
    """Div_Sqrt_Arccos_UInt_UInt and GetRotateAngle_Int_Int (the C library's
    angle bits, truncated to the rational register)."""
    b = Both(ref)
    rng = np.random.default_rng(7)
    l_ = b.reg(U, 50)  # the reference's constructor wants unsigned operands
    r_ = b.reg(U, 50)
    o = b.reg(R, 51)
    sl = b.reg(S, 50)
    sr = b.reg(S, 50)
    n = 500
    r = rng.integers(1, 1 << 49, n).astype(np.uint64)
    l = (rng.random(n) * r).astype(np.uint64)
    l[:4] = 0
    sa = rng.integers(0, 1 << 50, n).astype(np.uint64)
    sb = rng.integers(0, 1 << 50, n).astype(np.uint64)
    sa[:3] = 0
    sb[1] = (1 << 50) - 1
    regs = np.stack([l, r, np.zeros(n, dtype=np.uint64), sa, sb], axis=1)
    b.start(regs, np.full(n, 1 / math.sqrt(n), dtype=np.complex128))
    b.instr("ANGLE_XOR", (l_, r_, o), (0,))
    b.compare()
    b.instr("ANGLE_XOR", (sl, sr, o), (1,))
    b.compare()
    b.instr("ANGLE_XOR", (l_, r_, o), (0,), conds=((COND_BIT, sl, 4),))
    b.compare()


def test_qram_load(ref):
    from oracle import oracle as O
    b = Both(ref)
    rng = np.random.default_rng(8)
    addr = b.reg(U, 8)
    data = b.reg(U, 20)
    flag = b.reg(B, 1)
    mem = rng.integers(0, 1 << 20, 1 << 6, dtype=np.uint64)
    b.start(*random_state(rng, [8, 20, 1], 700))
    q = O.Qram(6, 20, mem)
    for conds in ((), ((COND_NONZERO, flag, 0),)):
        from sparqsim_gb300._native import OP
        ins = b.SqInstr()
        ins.op = OP["QRAM_LOAD"]
        ins.reg[0], ins.reg[1] = addr, data
        ins.qram = q.h
        ins.cond = b.cond(conds)
        arr = (b.SqInstr * 1)(ins)
        O._chk(O.lib().sqo_apply(b.ost.h, arr, 1))
        c = b.cond(conds)
        b._chk(ref.ref_qram_load(c_void_p(b.rst), 6, 20, c_void_p(mem.ctypes.data), c_uint64(mem.size), addr, data,
                                  byref(c)))
        b.compare()


@pytest.mark.parametrize("case", ["int", "int_cond", "full", "bool"])
def test_hadamards(ref, case):
    b = Both(ref)
    rng = np.random.default_rng(hash(case) % 1000)
    a = b.reg(U, 6)
    r = b.reg(U, 5)
    f = b.reg(B, 1)
    regs, amps = random_state(rng, [6, 5, 1], 150)
    if case == "int":  # the bits of `a` above the 4 transformed ones: a function of the other registers
        regs[:, 0] = (regs[:, 0] & 15) | ((regs[:, 1] & 3) << 4)
        regs, idx = np.unique(regs, axis=0, return_index=True)
        amps = amps[idx] / np.linalg.norm(amps[idx])
    b.start(regs, amps)
    none = b.cond(())
    cflag = b.cond(((COND_NONZERO, f, 0),))
    for _ in range(2):
        if case == "int":
            b.call("sqo_hadamard_int", "ref_hadamard_int", a, 4, byref(none))
        elif case == "int_cond":
            b.call("sqo_hadamard_int", "ref_hadamard_int", a, 6, byref(cflag))
        elif case == "full":
            b.call("sqo_hadamard_int_full", "ref_hadamard_int_full", a, byref(none))
        else:
            b.call("sqo_hadamard_bool", "ref_hadamard_bool", f, byref(none))
        b.compare()


def _keys_unique(regs):
    return len(np.unique(regs, axis=0)) == len(regs)


def test_hadamard_partial_where_the_reference_is_defined(ref):
    """Hadamard_Partial on one position of a state in which no two entries
    differ in that bit alone. The reference's active path (hash buckets
    under SAFE_HASH, global_macros.h:464; hadamard.cpp:619-712) then takes
    every entry through operate_alone_zero / operate_alone_one, which is the
    transform itself, and the oracle matches it bit for bit."""
    b = Both(ref)
    rng = np.random.default_rng(12)
    a = b.reg(U, 6)
    r = b.reg(U, 5)
    regs, amps = random_state(rng, [6, 5], 200)
    regs[:, 0] &= ~np.uint64(8)  # bit 3 clear everywhere: no entry has a partner on it
    regs, idx = np.unique(regs, axis=0, return_index=True)
    b.start(regs, amps[idx] / np.linalg.norm(amps[idx]))
    none = b.cond(())
    pos = (c_uint32 * 1)(3)
    b.call("sqo_hadamard_partial", "ref_hadamard_partial", a, pos, 1, byref(none))
    assert b.compare() == 2 * len(idx)


def test_hadamard_partial_reference_leaves_partners_unmerged(ref):
    """Where two entries differ in the position alone, the reference's
    bucket order StateLessExceptQubits (quantum_interfere_basic.cpp:151-177)
    ends by comparing the whole register, so the two never share a bucket:
    each is transformed alone and the state is left with two entries per key
    (|0> + |8> on bit 3 gives four entries on two keys). The oracle and the
    engine interfere the partners (one entry per key, the Hadamard of the
    pair); this records the reference's behaviour the divergence answers."""
    b = Both(ref)
    a = b.reg(U, 6)
    b.reg(U, 5)
    b.start(np.array([[0, 0], [8, 0], [1, 2]], dtype=np.uint64), np.array([0.6, 0.8, 1e-3j]))
    none = b.cond(())
    pos = (c_uint32 * 1)(3)
    b.call("sqo_hadamard_partial", "ref_hadamard_partial", a, pos, 1, byref(none))
    (orr, oa), (rr, ra) = b.states()
    assert _keys_unique(orr) and len(oa) == 4
    assert not _keys_unique(rr) and len(ra) == 6
    s2 = 1 / math.sqrt(2)
    got = {int(k[0]): v for k, v in zip(orr[:, :2], oa) if k[1] == 0}
    assert abs(got[0] - (0.6 + 0.8) * s2) < 1e-15 and abs(got[8] - (0.6 - 0.8) * s2) < 1e-15


def test_rotations_and_phases(ref):
    b = Both(ref)
    rng = np.random.default_rng(21)
    a = b.reg(U, 5)
    q = b.reg(B, 1)
    th = b.reg(R, 10)
    regs, amps = random_state(rng, [5, 1, 10], 300)
    b.start(regs, amps)
    none = b.cond(())
    cbit = b.cond(((COND_BIT, a, 1),))
    th_ = 0.7
    general = [math.cos(th_), 0, -math.sin(th_), 0.1, math.sin(th_), 0.1, math.cos(th_), 0]
    diag = [0.6, 0.8, 0, 0, 0, 0, 0.8, -0.6]
    off = [0, 0, 0.6, 0.8, 0.8, -0.6, 0, 0]
    for m in (general, diag, off):
        for dag in (0, 1):
            for c in (none, cbit):
                m8 = (c_double * 8)(*m)
                b.O._chk(b.O.lib().sqo_rot_bool(b.ost.h, a, 2, m8, byref(c), dag))
                b._chk(ref.ref_rot_bool(c_void_p(b.rst), a, 2, m8, dag, byref(c)))
                b.compare()
    for dag in (0, 1):
        b.call("sqo_condrot", "ref_condrot", th, q, dag, byref(none))
        b.compare()
    mats = []
    for v in range(32):
        t = 0.1 * v
        mats += [math.cos(t), 0, -math.sin(t), 0, math.sin(t), 0, math.cos(t), 0]
    tab = (c_double * len(mats))(*mats)
    b.call("sqo_condrot_general", "ref_condrot_general", a, q, tab, c_uint64(32), byref(none))
    b.compare()
    # Phase_Bool: the oracle takes (cos, sin) as the engine computes them, the reference the angle
    for lam, dag in ((0.3, False), (1.1, True)):
        from sparqsim_gb300._native import OP
        ins = b.SqInstr()
        ins.op = OP["PHASE_BOOL"]
        ins.reg[0], ins.imm[0] = a, 3
        ins.c[0], ins.c[1] = math.cos(lam), -math.sin(lam) if dag else math.sin(lam)
        ins.cond = b.cond(((COND_NONZERO, q, 0),))
        arr = (b.SqInstr * 1)(ins)
        b.O._chk(b.O.lib().sqo_apply(b.ost.h, arr, 1))
        c = b.cond(((COND_NONZERO, q, 0),))
        b._chk(ref.ref_phase_bool(c_void_p(b.rst), a, 3, c_double(lam), 1 if dag else 0, byref(c)))
        b.compare()
    ins = b.SqInstr()
    ins.op = OP["GLOBAL_PHASE"]
    ins.c[0], ins.c[1] = 0.0, 1.0
    arr = (b.SqInstr * 1)(ins)
    b.O._chk(b.O.lib().sqo_apply(b.ost.h, arr, 1))
    b._chk(ref.ref_global_phase(c_void_p(b.rst), c_double(0.0), c_double(1.0), byref(none)))
    b.compare()


def test_clear_zero_normalize_split_combine(ref):
    b = Both(ref)
    rng = np.random.default_rng(33)
    a = b.reg(U, 8)
    c = b.reg(U, 6)
    regs, amps = random_state(rng, [8, 6], 900)
    amps[::7] *= 1e-8  # below the threshold after squaring
    b.start(regs, amps)
    b.call("sqo_clear_zero", "ref_clear_zero", c_double(1e-14))
    n = b.compare()
    assert n < len(amps)
    b.O._chk(b.O.lib().sqo_normalize(b.ost.h, None))
    b._chk(ref.ref_normalize(c_void_p(b.rst)))
    b.compare()
    r_o = b.O.split_register(b.ost, a, 3)
    rid = c_uint32()
    b._chk(ref.ref_split_register(c_void_p(b.rst), a, 3, byref(rid)))
    assert r_o == rid.value
    b.compare()
    none = b.cond(())
    b.call("sqo_hadamard_int_full", "ref_hadamard_int_full", r_o, byref(none))
    b.compare()
    b.O.combine_register(b.ost, a, r_o)
    b._chk(ref.ref_combine_register(c_void_p(b.rst), a, r_o))
    b.compare()
