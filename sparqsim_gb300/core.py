"""Register table, GPU-resident sparse state and QRAM table — the pysparq
names (System, SparseState, QRAMCircuit_qutrit, StateStorageType) over the
GB300 engine's C ABI.

Mirrors PySparQ/core.cpp:67-160 (System, SparseState bindings) and
SparQ/include/basic_components.h:239-283 (the process-global register table).
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_uint32, c_uint64, c_void_p
from enum import IntEnum
from typing import Iterable, Union

import numpy as np

from ._native import SqCond, call, lib

RegRef = Union[str, int]


class StateStorageType(IntEnum):
    """Register types (reference StateStorageType)."""

    General = 0
    UnsignedInteger = 1
    SignedInteger = 2
    Boolean = 3
    Rational = 4


General = StateStorageType.General
UnsignedInteger = StateStorageType.UnsignedInteger
SignedInteger = StateStorageType.SignedInteger
Boolean = StateStorageType.Boolean
Rational = StateStorageType.Rational


class System:
    """Process-global register table (System::name_register_map).

    Register ids, reuse of freed ids and the name lookup follow
    basic_components.cpp:226-364: names map to the most recent active
    register of that name.
    """

    _names: list = []  # name per id (None when the slot was never named)

    @staticmethod
    def clear() -> None:
        call("sq_system_clear")
        System._names = []

    @staticmethod
    def add_register(name: str, type_: StateStorageType, size: int) -> int:
        rid = c_uint32(0)
        call("sq_system_add_register", int(type_), int(size), byref(rid))
        System._set_name(rid.value, name)
        return rid.value

    @staticmethod
    def _set_name(rid: int, name: str) -> None:
        while len(System._names) <= rid:
            System._names.append(None)
        System._names[rid] = name

    @staticmethod
    def add_register_synchronous(name: str, type_: StateStorageType, size: int, state: "SparseState") -> int:
        rid = c_uint32(0)
        call("sq_add_register_sync", state._h, int(type_), int(size), byref(rid))
        System._set_name(rid.value, name)
        return rid.value

    @staticmethod
    def remove_register(reg: RegRef) -> None:
        call("sq_system_remove_register", System.resolve(reg))

    @staticmethod
    def remove_register_synchronous(reg: RegRef, state: "SparseState") -> None:
        call("sq_remove_register_sync", state._h, System.resolve(reg))

    @staticmethod
    def _info(rid: int):
        t, w, a, wd, sh = (c_uint32(), c_uint32(), c_uint32(), c_uint32(), c_uint32())
        call("sq_system_register_info", int(rid), byref(t), byref(w), byref(a), byref(wd), byref(sh))
        return t.value, w.value, bool(a.value), wd.value, sh.value

    @staticmethod
    def register_count() -> int:
        n = c_uint32()
        call("sq_system_register_count", byref(n))
        return n.value

    @staticmethod
    def get_id(name: str) -> int:
        for rid in range(min(len(System._names), System.register_count()) - 1, -1, -1):
            if System._names[rid] == name and System._info(rid)[2]:
                return rid
        raise ValueError(f"Register not found: {name!r}")

    get = get_id

    @staticmethod
    def resolve(reg: RegRef) -> int:
        if isinstance(reg, (int, np.integer)):
            return int(reg)
        return System.get_id(reg)

    @staticmethod
    def name_of(reg: RegRef) -> str:
        return System._names[System.resolve(reg)]

    @staticmethod
    def size_of(reg: RegRef) -> int:
        return System._info(System.resolve(reg))[1]

    @staticmethod
    def type_of(reg: RegRef) -> StateStorageType:
        return StateStorageType(System._info(System.resolve(reg))[0])

    @staticmethod
    def status_of(reg: RegRef) -> bool:
        return System._info(System.resolve(reg))[2]

    @staticmethod
    def set_register_type(reg: RegRef, type_: StateStorageType) -> None:
        call("sq_system_set_register_type", System.resolve(reg), int(type_))

    @staticmethod
    def active_ids() -> list:
        return [i for i in range(System.register_count()) if System._info(i)[2]]

    @staticmethod
    def get_qubit_count() -> int:
        return sum(System._info(i)[1] for i in System.active_ids())

    @staticmethod
    def get_activated_register_size() -> int:
        return len(System.active_ids())

    @staticmethod
    def key_words() -> int:
        k = c_uint32()
        call("sq_system_key_words", byref(k))
        return k.value


def set_group_strategy(strategy: str) -> None:
    """'auto', 'sort' (onesweep radix sort) or 'hash' (hash-table buckets):
    how split/merge operators group entries ('autotune', the default, times
    sort and hash per shape class and keeps the faster). Results are identical."""
    call("sq_set_group_strategy", {"auto": 0, "sort": 1, "hash": 2, "autotune": 3}[strategy])


def get_group_strategy() -> str:
    from ctypes import c_int
    v = c_int()
    call("sq_get_group_strategy", byref(v))
    return ["auto", "sort", "hash", "autotune"][v.value]


def autotune_reset() -> None:
    call("sq_autotune_reset")


def autotune_classes() -> tuple:
    """(shape classes seen, classes whose choice is made)."""
    c, d = ctypes.c_uint64(), ctypes.c_uint64()
    call("sq_autotune_classes", byref(c), byref(d))
    return c.value, d.value


def set_output_sizing(mode: str) -> None:
    """'auto' (single pass with per-group atomic reservation when the output
    bound fits) or 'exact' (count pass, scan, write pass)."""
    call("sq_set_output_sizing", {"auto": 0, "exact": 1}[mode])


def set_fwht_arithmetic(mode: str) -> None:
    """Arithmetic of the Hadamard butterflies: 'reference' (FP64 in the
    reference's stage order, bit-identical results) or 'exact-sum' (default:
    exact integer sums on a per-group grid, one rounding per output)."""
    call("sq_set_fwht_arithmetic", {"reference": 0, "exact-sum": 1}[mode])


def get_fwht_arithmetic() -> str:
    from ctypes import c_int
    v = c_int()
    call("sq_get_fwht_arithmetic", byref(v))
    return ["reference", "exact-sum"][v.value]


def set_download_engine(engine: str) -> None:
    """How `SparseState.download_packed_async` moves data into pinned host
    memory: "sm" (default: a few low-priority blocks store over the host link,
    about 150 GB/s on every system measured, leaving the copy engine to the
    small count reads of eager operators) or "copy" (the copy engine: no SM
    resources taken from the work it overlaps, but its rate into pinned memory
    varied from 84 to over 170 GB/s between systems) or "split" (half of each
    destination each way, at once)."""
    modes = {"sm": 0, "copy": 1, "split": 2}
    if engine not in modes:
        raise ValueError(f"download engine must be one of {sorted(modes)}")
    call("sq_set_download_engine", modes[engine])


def set_clearzero_default_eps(eps: float) -> None:
    """clearzero_default_eps (system_operations.h:577)."""
    call("sq_set_clearzero_eps", float(eps))


def get_clearzero_default_eps() -> float:
    v = c_double()
    call("sq_get_clearzero_eps", byref(v))
    return v.value


class SparseState:
    """A sparse state resident in GPU memory (replaces CuSparseState).

    A new state holds the single entry |0...0> with amplitude 1, like
    SparseState() (basic_components.h:604-606).
    """

    def __init__(self, other: "SparseState | None" = None, capacity: int = 1024):
        h = c_void_p()
        call("sq_state_create", int(max(capacity, 1)), byref(h))
        self._h = h
        if other is not None:
            call("sq_state_copy", self._h, other._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().sq_state_destroy(h)
            except Exception:
                pass
            self._h = None

    def size(self) -> int:
        n = c_uint64()
        call("sq_state_size", self._h, byref(n))
        return n.value

    __len__ = size

    def empty(self) -> bool:
        return self.size() == 0

    def capacity(self) -> int:
        n = c_uint64()
        call("sq_state_capacity", self._h, byref(n))
        return n.value

    def reserve(self, capacity: int) -> None:
        call("sq_state_reserve", self._h, int(capacity))

    def reset(self) -> None:
        call("sq_state_reset", self._h)

    def copy(self) -> "SparseState":
        return SparseState(self)

    def upload(self, regs: np.ndarray, amps: np.ndarray) -> None:
        """Set the state from host arrays: regs[i, id] (uint64) and amps[i] (complex128)."""
        regs = np.ascontiguousarray(regs, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.complex128)
        n = amps.shape[0]
        if regs.ndim != 2 or regs.shape[0] != n:
            raise ValueError("regs must be [n, nregs]")
        call("sq_state_upload", self._h, n, regs.ctypes.data_as(c_void_p), regs.shape[1],
             amps.ctypes.data_as(c_void_p))

    def download(self, nregs: int | None = None):
        """Return (regs[n, nregs] uint64, amps[n] complex128); inactive ids read 0."""
        if nregs is None:
            nregs = System.register_count()
        n = self.size()
        regs = np.zeros((n, max(nregs, 1)), dtype=np.uint64)
        amps = np.zeros(n, dtype=np.complex128)
        if n:
            call("sq_state_download", self._h, regs.ctypes.data_as(c_void_p), nregs,
                 amps.ctypes.data_as(c_void_p))
        return regs[:, :nregs], amps

    def download_packed_async(self, keys_ptr: int, amps_ptr: int) -> None:
        """Start copying the packed key words (K x n uint64, word-major) and
        the amplitudes (n complex128) into host memory at the given addresses
        (pinned memory for full speed) and return at once; `wait()` blocks
        until the copy is done. Later operations on this state wait for it on
        the device."""
        call("sq_state_download_packed_async", self._h, c_void_p(keys_ptr), c_void_p(amps_ptr))

    def wait(self) -> None:
        """Block until this state's last asynchronous download has finished."""
        call("sq_state_wait", self._h)

    def to_dict(self) -> dict:
        """{tuple(values of the active registers in id order): amplitude}."""
        regs, amps = self.download()
        ids = System.active_ids()
        return {tuple(int(v) for v in r[ids]): complex(a) for r, a in zip(regs, amps)}

    def norm_sq(self) -> float:
        v = c_double()
        call("sq_norm_sq", self._h, byref(v))
        return v.value

    def device_arrays(self):
        """(list of K key-word device pointers, amplitude device pointer) as ints."""
        k = c_uint32()
        ptrs = (c_void_p * 8)()
        amp = c_void_p()
        call("sq_state_device_arrays", self._h, ptrs, byref(k), byref(amp))
        return [ptrs[i] for i in range(k.value)], amp.value

    def __repr__(self) -> str:
        return f"SparseState(size={self.size()}, device=GB300)"


class QRAMCircuit_qutrit:
    """Noise-free QRAM table (qram_qutrit::QRAMCircuit(addr_size, data_size, memory)).

    The table is copied to HBM once; QRAMLoad gathers from it
    (qram.cpp:15-35). Only the noise-free path is provided.
    """

    def __init__(self, addr_size: int, data_size: int, memory: Iterable[int] | None = None):
        self.address_size = int(addr_size)
        self.data_size = int(data_size)
        if memory is None:
            memory = np.zeros(1 << self.address_size, dtype=np.uint64)
        mem = np.ascontiguousarray(np.asarray(memory, dtype=np.uint64))
        self.memory = mem
        h = c_void_p()
        call("sq_qram_create", self.address_size, self.data_size, mem.ctypes.data_as(c_void_p), mem.size, byref(h))
        self._h = h

    def write(self, memory) -> None:
        """New table words, written in place (launches queued or captured earlier
        keep reading the same device table); they must fit the table's stored
        width. `memory` may be a NumPy array or the address of 2^address_size
        uint64 words (pinned memory for full speed)."""
        if isinstance(memory, int):
            call("sq_qram_write", self._h, c_void_p(memory), 1 << self.address_size)
            return
        mem = np.ascontiguousarray(np.asarray(memory, dtype=np.uint64))
        call("sq_qram_write", self._h, mem.ctypes.data_as(c_void_p), mem.size)
        self.memory = mem

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().sq_qram_destroy(h)
            except Exception:
                pass
            self._h = None


# ---------------------------------------------------------------------- conditions
class Controllable:
    """conditioned_by_* / clear_control_* (global_macros.h:104-284, BindUtils.h:117-165)."""

    def _init_controls(self) -> None:
        self.condition_variable_nonzeros = []
        self.condition_variable_all_ones = []
        self.condition_variable_by_bit = []
        self.condition_variable_by_value = []

    @staticmethod
    def _ids(conds) -> list:
        if isinstance(conds, (str, int, np.integer)):
            conds = [conds]
        return [System.resolve(c) for c in conds]

    @staticmethod
    def _pairs(a, b=None) -> list:
        if b is not None:
            return [(System.resolve(a), int(b))]
        return [(System.resolve(x), int(y)) for x, y in a]

    def conditioned_by_nonzeros(self, conds):
        self.condition_variable_nonzeros = self._ids(conds)
        return self

    def conditioned_by_all_ones(self, conds):
        self.condition_variable_all_ones = self._ids(conds)
        return self

    def conditioned_by_bit(self, cond, pos=None):
        self.condition_variable_by_bit = self._pairs(cond, pos)
        return self

    def conditioned_by_value(self, cond, value=None):
        self.condition_variable_by_value = self._pairs(cond, value)
        return self

    def clear_control_nonzeros(self):
        self.condition_variable_nonzeros = []

    def clear_control_all_ones(self):
        self.condition_variable_all_ones = []

    def clear_control_by_bit(self):
        self.condition_variable_by_bit = []

    def clear_control_by_value(self):
        self.condition_variable_by_value = []

    def copy_control_conditions_to(self, other: "Controllable") -> None:
        other.condition_variable_nonzeros = list(self.condition_variable_nonzeros)
        other.condition_variable_all_ones = list(self.condition_variable_all_ones)
        other.condition_variable_by_bit = list(self.condition_variable_by_bit)
        other.condition_variable_by_value = list(self.condition_variable_by_value)

    def has_condition(self) -> bool:
        return bool(self.condition_variable_nonzeros or self.condition_variable_all_ones
                    or self.condition_variable_by_bit or self.condition_variable_by_value)

    def _cond(self) -> SqCond:
        from ._native import COND_ALL_ONES, COND_BIT, COND_NONZERO, COND_VALUE, SQ_MAX_CONDITIONS
        c = SqCond()
        items = ([(COND_NONZERO, r, 0) for r in self.condition_variable_nonzeros]
                 + [(COND_ALL_ONES, r, 0) for r in self.condition_variable_all_ones]
                 + [(COND_BIT, r, p) for r, p in self.condition_variable_by_bit]
                 + [(COND_VALUE, r, v) for r, v in self.condition_variable_by_value])
        if len(items) > SQ_MAX_CONDITIONS:
            raise ValueError(f"at most {SQ_MAX_CONDITIONS} conditions per operator")
        c.count = len(items)
        for i, (k, r, p) in enumerate(items):
            c.c[i].kind = k
            c.c[i].reg = r
            c.c[i].param = p & 0xFFFFFFFFFFFFFFFF
        return c


class Graph:
    """A sequence of operators on one state, replayed as one CUDA graph
    launch (sq_graph_*). `prepare()` brings the state to its input (for
    example uploads it) and `apply()` applies the operators. Construction
    runs them once eagerly (recording every count the host reads back), then
    once under capture; `replay()` prepares the state and launches the graph,
    which runs every kernel again with no host round trip in between. The
    counts a replay produces are checked on the device against the recorded
    ones: a replay on an input whose split sizes differ is reported at the
    next synchronising call (SparQInvalid) and leaves the state invalid. The
    operators must leave the state's double buffers in their roles (an even
    number of splits), so that each replay starts as the last one ended."""

    def __init__(self, state: "SparseState", apply, prepare):
        self.state, self._apply, self._prepare = state, apply, prepare
        self._h = c_void_p()
        prepare()
        call("sq_graph_record_begin", state._h)
        try:
            apply()
        finally:
            call("sq_graph_record_end")
        prepare()
        call("sq_graph_capture_begin", state._h)
        try:
            apply()
        except BaseException:
            try:
                call("sq_graph_capture_end", byref(self._h))  # closes the capture
            except Exception:
                pass
            raise
        call("sq_graph_capture_end", byref(self._h))

    def launch(self) -> None:
        """Launch on the state as it is (asynchronous)."""
        call("sq_graph_launch", self._h)

    def replay(self) -> None:
        self._prepare()
        self.launch()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                call("sq_graph_destroy", h)
            except Exception:
                pass
            self._h = None

