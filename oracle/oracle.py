"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of the CPU oracle
(oracle/sparq_oracle.cpp, a restatement of SparQ's CPU operator path).

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the
checker. It consumes the operation descriptions produced by
``sparqsim_gb300`` operators' ``spec()`` so both sides run the same program.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_double, c_int, c_uint32, c_uint64, c_void_p

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        from sparqsim_gb300._native import SqCond, SqInstr
        sigs = {
            "sqo_last_error": (ctypes.c_char_p, []),
            "sqo_clear": (c_int, []),
            "sqo_set_clearzero_eps": (c_int, [c_double]),
            "sqo_add_register": (c_int, [c_uint32, c_uint32, POINTER(c_uint32)]),
            "sqo_remove_register": (c_int, [c_uint32]),
            "sqo_register_count": (c_int, [POINTER(c_uint32)]),
            "sqo_register_info": (c_int, [c_uint32, POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]),
            "sqo_state_new": (c_void_p, []),
            "sqo_state_free": (None, [c_void_p]),
            "sqo_state_size": (c_uint64, [c_void_p]),
            "sqo_state_copy": (c_int, [c_void_p, c_void_p]),
            "sqo_state_set": (c_int, [c_void_p, c_uint64, c_void_p, c_uint32, c_void_p]),
            "sqo_state_get": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
            "sqo_qram_new": (c_void_p, [c_uint32, c_uint32, c_void_p, c_uint64]),
            "sqo_qram_free": (None, [c_void_p]),
            "sqo_apply": (c_int, [c_void_p, POINTER(SqInstr), c_uint32]),
            "sqo_hadamard_int": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
            "sqo_hadamard_int_full": (c_int, [c_void_p, c_uint32, POINTER(SqCond)]),
            "sqo_hadamard_bool": (c_int, [c_void_p, c_uint32, POINTER(SqCond)]),
            "sqo_rot_bool": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_double), POINTER(SqCond), c_int]),
            "sqo_condrot": (c_int, [c_void_p, c_uint32, c_uint32, c_int, POINTER(SqCond)]),
            "sqo_clear_zero": (c_int, [c_void_p, c_double]),
            "sqo_condrot_general": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_double), c_uint64, POINTER(SqCond)]),
            "sqo_rot_general_unitary": (c_int, [c_void_p, c_uint32, POINTER(c_double), c_uint64, POINTER(SqCond), c_int]),
            "sqo_hadamard_partial": (c_int, [c_void_p, c_uint32, POINTER(c_uint32), c_uint32, POINTER(SqCond)]),
            "sqo_normalize": (c_int, [c_void_p, POINTER(c_double)]),
            "sqo_partial_trace_select": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_int, c_uint64, c_uint64,
                                                 POINTER(c_double)]),
            "sqo_get_output": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_uint64,
                                       POINTER(c_double)]),
            "sqo_qw_rotate_angle": (c_int, [c_void_p, c_uint32, c_uint32, c_uint32, c_int, POINTER(SqCond)]),
            "sqo_add_systems": (c_int, [c_void_p, c_void_p, c_double]),
            "sqo_add_register_sync": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_uint32)]),
            "sqo_remove_register_sync": (c_int, [c_void_p, c_uint32]),
            "sqo_split_register": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_uint32)]),
            "sqo_combine_register": (c_int, [c_void_p, c_uint32, c_uint32]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _chk(rc):
    if rc != 0:
        raise OracleError(lib().sqo_last_error().decode())


# ---------------------------------------------------------------- register table
def clear():
    _chk(lib().sqo_clear())


def set_clearzero_eps(eps: float):
    _chk(lib().sqo_set_clearzero_eps(eps))


def add_register(type_: int, width: int) -> int:
    r = c_uint32()
    _chk(lib().sqo_add_register(int(type_), int(width), byref(r)))
    return r.value


def remove_register(rid: int):
    _chk(lib().sqo_remove_register(int(rid)))


def register_count() -> int:
    n = c_uint32()
    _chk(lib().sqo_register_count(byref(n)))
    return n.value


def active_ids() -> list:
    out = []
    for i in range(register_count()):
        t, w, a = c_uint32(), c_uint32(), c_uint32()
        _chk(lib().sqo_register_info(i, byref(t), byref(w), byref(a)))
        if a.value:
            out.append(i)
    return out


class Qram:
    def __init__(self, address_size: int, data_size: int, memory):
        mem = np.ascontiguousarray(np.asarray(memory, dtype=np.uint64))
        self.memory = mem
        self.h = lib().sqo_qram_new(address_size, data_size, mem.ctypes.data_as(c_void_p), mem.size)

    def __del__(self):
        if getattr(self, "h", None):
            lib().sqo_qram_free(self.h)
            self.h = None


class OracleState:
    """A SparseState of the CPU restatement: starts as one |0...0> entry."""

    def __init__(self, other: "OracleState | None" = None):
        self.h = lib().sqo_state_new()
        if other is not None:
            _chk(lib().sqo_state_copy(self.h, other.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().sqo_state_free(self.h)
            self.h = None

    def size(self) -> int:
        return lib().sqo_state_size(self.h)

    def set(self, regs: np.ndarray, amps: np.ndarray):
        regs = np.ascontiguousarray(regs, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.complex128)
        _chk(lib().sqo_state_set(self.h, amps.shape[0], regs.ctypes.data_as(c_void_p), regs.shape[1],
                                  amps.ctypes.data_as(c_void_p)))

    def get(self, nregs: int | None = None):
        if nregs is None:
            nregs = register_count()
        n = self.size()
        regs = np.zeros((n, max(nregs, 1)), dtype=np.uint64)
        amps = np.zeros(n, dtype=np.complex128)
        if n:
            _chk(lib().sqo_state_get(self.h, regs.ctypes.data_as(c_void_p), nregs, amps.ctypes.data_as(c_void_p)))
        return regs[:, :nregs], amps


# ---------------------------------------------------------------- operations
_qram_map: dict = {}


def register_qram(qram_circuit) -> Qram:
    """Give the oracle its own copy of a product QRAM table (matched by handle)."""
    q = Qram(qram_circuit.address_size, qram_circuit.data_size, qram_circuit.memory)
    _qram_map[qram_circuit._h.value] = q
    return q


def apply(state: OracleState, spec) -> None:
    """Apply one operation description (sparqsim_gb300 operator .spec())."""
    from sparqsim_gb300._native import OP, SqInstr
    L = lib()
    kind = spec[0]
    h = state.h
    if kind == "prog":
        instrs = []
        for ins in spec[1]:
            c = SqInstr()
            ctypes.pointer(c)[0] = ins
            if ins.op in (OP["QRAM_LOAD"], OP["PAULI_NOISE"], OP["QBS_XOR"]):
                c.qram = _qram_map[ins.qram].h
            instrs.append(c)
        arr = (SqInstr * len(instrs))(*instrs)
        _chk(L.sqo_apply(h, arr, len(instrs)))
    elif kind == "hadamard_int":
        _chk(L.sqo_hadamard_int(h, spec[1], spec[2], byref(spec[3])))
    elif kind == "hadamard_int_batched":
        # reference composition: Hadamard_Int(reg, h).conditioned_by_value(width_reg, h) for each h
        from sparqsim_gb300._native import COND_VALUE, SqCond
        reg, wreg, maxd, cond = spec[1], spec[2], spec[3], spec[4]
        for hd in range(1, maxd + 1):
            c = SqCond()
            ctypes.pointer(c)[0] = cond
            if c.count >= 8:
                raise ValueError("too many conditions")
            c.c[c.count].kind = COND_VALUE
            c.c[c.count].reg = wreg
            c.c[c.count].param = hd
            c.count += 1
            _chk(L.sqo_hadamard_int(h, reg, hd, byref(c)))
    elif kind == "hadamard_int_full":
        _chk(L.sqo_hadamard_int_full(h, spec[1], byref(spec[2])))
    elif kind == "hadamard_bool":
        _chk(L.sqo_hadamard_bool(h, spec[1], byref(spec[2])))
    elif kind == "rot_bool":
        m = (c_double * 8)(*spec[3])
        _chk(L.sqo_rot_bool(h, spec[1], spec[2], m, byref(spec[4]), 0))
    elif kind == "condrot":
        _chk(L.sqo_condrot(h, spec[1], spec[2], 1 if spec[3] else 0, byref(spec[4])))
    elif kind == "condrot_general":
        tab = spec[3]
        _chk(L.sqo_condrot_general(h, spec[1], spec[2], tab.ctypes.data_as(POINTER(c_double)), tab.size // 8,
                                   byref(spec[4])))
    elif kind == "rot_general_unitary":
        mat = spec[2]
        _chk(L.sqo_rot_general_unitary(h, spec[1], mat.ctypes.data_as(POINTER(c_double)), spec[3], byref(spec[4]),
                                       1 if spec[5] else 0))
    elif kind == "hadamard_partial":
        pos = (c_uint32 * len(spec[2]))(*spec[2])
        _chk(L.sqo_hadamard_partial(h, spec[1], pos, len(spec[2]), byref(spec[3])))
    elif kind == "qw_rotate_angle":
        _chk(L.sqo_qw_rotate_angle(h, spec[1], spec[2], spec[3], 1 if spec[4] else 0, byref(spec[5])))
    elif kind == "clear_zero":
        _chk(L.sqo_clear_zero(h, spec[1]))
    elif kind == "normalize":
        _chk(L.sqo_normalize(h, None))
    elif kind in ("partial_trace_select", "partial_trace_select_range"):
        out = c_double()
        if kind == "partial_trace_select":
            regs = np.array(spec[1], dtype=np.uint32)
            vals = np.array(spec[2], dtype=np.uint64)
            _chk(L.sqo_partial_trace_select(h, regs.ctypes.data_as(c_void_p), vals.ctypes.data_as(c_void_p),
                                            len(regs), 0, 0, 0, byref(out)))
        else:
            regs = np.array([spec[1]], dtype=np.uint32)
            _chk(L.sqo_partial_trace_select(h, regs.ctypes.data_as(c_void_p), None, 1, 1, spec[2], spec[3],
                                            byref(out)))
        return out.value
    else:
        raise ValueError(kind)


def get_output(state: "OracleState", zero_regs, idx_regs, width_of):
    """GetOutput (qda_fundamental.cpp:123-166): (dense amplitude vector,
    post-selected probability); width_of(reg) gives a register's width."""
    z = np.array(zero_regs, dtype=np.uint32)
    ix = np.array(idx_regs, dtype=np.uint32)
    n = 1 << sum(width_of(r) for r in idx_regs)
    out = np.zeros(2 * n, dtype=np.float64)
    prob = c_double()
    _chk(lib().sqo_get_output(state.h, z.ctypes.data_as(c_void_p), len(z), ix.ctypes.data_as(c_void_p), len(ix),
                              out.ctypes.data_as(c_void_p), n, byref(prob)))
    return out.view(np.complex128), prob.value


def add_systems(dst: OracleState, src: OracleState, coef: float):
    _chk(lib().sqo_add_systems(dst.h, src.h, coef))


def add_register_sync(state: OracleState, type_: int, width: int) -> int:
    r = c_uint32()
    _chk(lib().sqo_add_register_sync(state.h, int(type_), int(width), byref(r)))
    return r.value


def remove_register_sync(state: OracleState, rid: int):
    _chk(lib().sqo_remove_register_sync(state.h, int(rid)))


def split_register(state: OracleState, first: int, second_size: int) -> int:
    r = c_uint32()
    _chk(lib().sqo_split_register(state.h, int(first), int(second_size), byref(r)))
    return r.value


def combine_register(state: OracleState, first: int, second: int):
    _chk(lib().sqo_combine_register(state.h, int(first), int(second)))


def canonical(regs: np.ndarray, amps: np.ndarray, ids: list):
    """Sort entries by the active register values (lexicographic in id order)."""
    keys = regs[:, ids] if len(ids) else np.zeros((regs.shape[0], 0), dtype=np.uint64)
    if keys.shape[1] == 0:
        return keys, amps
    order = np.lexsort(keys.T[::-1])
    return keys[order], amps[order]
