"""ctypes binding of libsparq_gb300.so (the C ABI in include/sparq_gb300.h).

The engine has no CPU fallback: if the shared library is missing or no CUDA
device is visible, calls raise instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name("libsparq_gb300.so")

SQ_MAX_CONDITIONS = 8
SQ_MAX_PROGRAM = 32
SQ_MAX_REGISTERS = 64
SQ_MAX_KEY_WORDS = 8

# status codes
SQ_OK, SQ_ERR_INVALID, SQ_ERR_CUDA, SQ_ERR_OOM, SQ_ERR_CAPACITY, SQ_ERR_DEVICE_TIMEOUT, \
    SQ_ERR_BAD_RESULT, SQ_ERR_UNSUPPORTED, SQ_ERR_NO_DEVICE = range(9)

# condition kinds
COND_NONZERO, COND_ALL_ONES, COND_BIT, COND_VALUE = range(4)

# opcodes (sq_opcode)
OP = dict(
    NOP=0, FLIP_BOOLS=1, SWAP_BOOL_BOOL=2, SHIFT_LEFT=3, SHIFT_RIGHT=4, MULT_UINT_CONST=5,
    ADD_MULT_UINT_CONST=6, MOD_MULT_CONST=7, ADD_UINT_UINT=8, ADD_UINT_UINT_INPLACE=9,
    ADD_UINT_CONST=10, ADD_CONST_INPLACE=11, SUB_UINT_UINT=12, NEG_UINT=13, ABS_SINT=14,
    MUL_UINT_UINT=15, DIV_UINT_UINT=16, SQRT_UINT=17, SELECT_BOOL=18, AND_UINT_UINT=19,
    OR_UINT_UINT=20, XOR_UINT_UINT=21, LESS_SINT_SINT=22, CARRY_UINT_UINT=23,
    OVERFLOW_SINT_SINT=24, MULOVERFLOW_UINT_UINT=25, ISZERO_UINT=26, NEGATIVE_SINT=27,
    ADD_ANYINT_INPLACE=28, ASSIGN=29, COMPARE_UINT_UINT=30, LESS_UINT_UINT=31, SWAP_GENERAL=32,
    GETMID_UINT_UINT=33, X_BOOL=34, INIT_UNSAFE=35, QRAM_LOAD=36, PLUS_ONE_OVERFLOW=37, BIT_GATHER=38,
    PHASE_BOOL=64, GLOBAL_PHASE=65,
    Y_BOOL=66, REFLECTION_BOOL=67, ZERO_COND_PHASE_FLIP=68, ROT_DIAGONAL=69, ROT_OFF_DIAGONAL=70,
    PAULI_NOISE=71, TRIDIAG_ELEMENT=72, TRIDIAG_SLOT_COLUMN=73, LOOKUP_XOR=74, PARITY_PHASE=75,
    ANGLE_XOR=76, ADDR_XOR=77, QBS_XOR=78,
)


class SqCondition(ctypes.Structure):
    _fields_ = [("kind", c_uint32), ("reg", c_uint32), ("param", c_uint64)]


class SqCond(ctypes.Structure):
    _fields_ = [("count", c_uint32), ("reserved", c_uint32), ("c", SqCondition * SQ_MAX_CONDITIONS)]


class SqInstr(ctypes.Structure):
    _fields_ = [
        ("op", c_uint32),
        ("dag", c_uint32),
        ("reg", c_uint32 * 4),
        ("imm", c_uint64 * 3),
        ("c", c_double * 8),
        ("qram", c_void_p),
        ("cond", SqCond),
    ]


assert ctypes.sizeof(SqInstr) == 256, ctypes.sizeof(SqInstr)


class SparQError(RuntimeError):
    """Error raised for a non-zero sq_status (status in .code)."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class SparQInvalid(SparQError, ValueError):
    pass


# (name, restype, argtypes) for every exported entry point
_SIGS = [
    ("sq_abi_version", c_int, []),
    ("sq_last_error", ctypes.c_char_p, []),
    ("sq_init", c_int, [c_int]),
    ("sq_synchronize", c_int, []),
    ("sq_launch_count", c_int, [POINTER(c_uint64)]),
    ("sq_get_stream", c_int, [POINTER(c_void_p)]),
    ("sq_profile_enable", c_int, [c_int]),
    ("sq_profile_reset", c_int, []),
    ("sq_profile_read", c_int, [c_void_p, ctypes.c_size_t, POINTER(c_uint64), POINTER(c_double),
                                POINTER(c_double), c_uint32, POINTER(c_uint32)]),
    ("sq_system_clear", c_int, []),
    ("sq_system_add_register", c_int, [c_uint32, c_uint32, POINTER(c_uint32)]),
    ("sq_system_remove_register", c_int, [c_uint32]),
    ("sq_system_register_info", c_int, [c_uint32] + [POINTER(c_uint32)] * 5),
    ("sq_system_register_count", c_int, [POINTER(c_uint32)]),
    ("sq_system_key_words", c_int, [POINTER(c_uint32)]),
    ("sq_system_set_register_type", c_int, [c_uint32, c_uint32]),
    ("sq_state_create", c_int, [c_uint64, POINTER(c_void_p)]),
    ("sq_state_destroy", c_int, [c_void_p]),
    ("sq_state_size", c_int, [c_void_p, POINTER(c_uint64)]),
    ("sq_state_capacity", c_int, [c_void_p, POINTER(c_uint64)]),
    ("sq_state_reserve", c_int, [c_void_p, c_uint64]),
    ("sq_state_reset", c_int, [c_void_p]),
    ("sq_state_copy", c_int, [c_void_p, c_void_p]),
    ("sq_state_upload", c_int, [c_void_p, c_uint64, c_void_p, c_uint32, c_void_p]),
    ("sq_state_download", c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    ("sq_state_upload_packed", c_int, [c_void_p, c_uint64, c_void_p, c_void_p]),
    ("sq_state_download_packed", c_int, [c_void_p, c_void_p, c_void_p]),
    ("sq_state_download_packed_async", c_int, [c_void_p, c_void_p, c_void_p]),
    ("sq_state_wait", c_int, [c_void_p]),
    ("sq_set_download_engine", c_int, [c_int]),
    ("sq_graph_record_begin", c_int, [c_void_p]),
    ("sq_graph_record_end", c_int, []),
    ("sq_graph_capture_begin", c_int, [c_void_p]),
    ("sq_graph_capture_end", c_int, [POINTER(c_void_p)]),
    ("sq_graph_launch", c_int, [c_void_p]),
    ("sq_graph_destroy", c_int, [c_void_p]),
    ("sq_graph_debug_dot", c_int, [c_void_p, c_char_p]),
    ("sq_state_debug_layout", c_int, [c_void_p, c_char_p, c_uint64]),
    ("sq_state_device_arrays", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_uint32), POINTER(c_void_p)]),
    ("sq_qram_create", c_int, [c_uint32, c_uint32, c_void_p, c_uint64, POINTER(c_void_p)]),
    ("sq_qram_write", c_int, [c_void_p, c_void_p, c_uint64]),
    ("sq_qram_destroy", c_int, [c_void_p]),
    ("sq_lookup_create", c_int, [c_void_p, c_uint64, c_void_p, c_void_p, c_uint64, POINTER(c_void_p)]),
    ("sq_angle_table_create", c_int, [c_int, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_uint64,
                                      POINTER(c_void_p)]),
    ("sq_angle_word", c_int, [c_int, c_uint32, c_uint32, c_uint32, c_uint64, c_uint64, POINTER(c_uint64)]),
    ("sq_qw_rotate_angle_words", c_int, [c_void_p, c_uint64, c_uint32, c_int, c_uint32, c_void_p]),
    ("sq_apply_program", c_int, [c_void_p, POINTER(SqInstr), c_uint32]),
    ("sq_add_uint_uint", c_int, [c_void_p, c_uint32, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_add_uint_uint_inplace", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond), c_int]),
    ("sq_add_uint_const", c_int, [c_void_p, c_uint32, c_uint64, c_uint32, POINTER(SqCond)]),
    ("sq_add_const_inplace", c_int, [c_void_p, c_uint32, c_uint64, POINTER(SqCond), c_int]),
    ("sq_mult_uint_const", c_int, [c_void_p, c_uint32, c_uint64, c_uint32, POINTER(SqCond)]),
    ("sq_add_mult_uint_const", c_int, [c_void_p, c_uint32, c_uint64, c_uint32, POINTER(SqCond), c_int]),
    ("sq_mul_uint_uint", c_int, [c_void_p, c_uint32, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_add_anyint_inplace", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond), c_int]),
    ("sq_assign", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_shift", c_int, [c_void_p, c_uint32, c_uint32, c_int, POINTER(SqCond)]),
    ("sq_swap", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_x_bool", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_flip_bools", c_int, [c_void_p, c_uint32, POINTER(SqCond)]),
    ("sq_init_unsafe", c_int, [c_void_p, c_uint32, c_uint64]),
    ("sq_qram_load", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_phase_bool", c_int, [c_void_p, c_uint32, c_uint32, c_double, POINTER(SqCond), c_int]),
    ("sq_global_phase", c_int, [c_void_p, c_double, c_double, POINTER(SqCond), c_int]),
    ("sq_reflection_bool", c_int, [c_void_p, POINTER(c_uint32), c_uint32, c_int, POINTER(SqCond)]),
    ("sq_zero_cond_phase_flip", c_int, [c_void_p, POINTER(c_uint32), c_uint32, POINTER(SqCond)]),
    ("sq_hadamard_int", c_int, [c_void_p, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_hadamard_int_batched", c_int, [c_void_p, c_uint32, c_uint32, c_uint32, POINTER(SqCond)]),
    ("sq_hadamard_int_full", c_int, [c_void_p, c_uint32, POINTER(SqCond)]),
    ("sq_hadamard_bool", c_int, [c_void_p, c_uint32, POINTER(SqCond)]),
    ("sq_rot_bool", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_double), POINTER(SqCond), c_int]),
    ("sq_condrot_rational_bool", c_int, [c_void_p, c_uint32, c_uint32, c_int]),
    ("sq_condrot_rational_bool_cond", c_int, [c_void_p, c_uint32, c_uint32, c_int, POINTER(SqCond)]),
    ("sq_condrot_general_bool", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_double), c_uint64]),
    ("sq_condrot_general_bool_cond", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_double), c_uint64,
                                             POINTER(SqCond)]),
    ("sq_rot_general_unitary", c_int, [c_void_p, c_uint32, POINTER(c_double), c_uint64, POINTER(SqCond), c_int]),
    ("sq_hadamard_partial", c_int, [c_void_p, c_uint32, POINTER(c_uint32), c_uint32, POINTER(SqCond)]),
    ("sq_set_group_strategy", c_int, [c_int]),
    ("sq_get_group_strategy", c_int, [POINTER(c_int)]),
    ("sq_set_output_sizing", c_int, [c_int]),
    ("sq_partial_trace_select", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, POINTER(c_double)]),
    ("sq_partial_trace_select_range", c_int, [c_void_p, c_uint32, c_uint64, c_uint64, POINTER(c_double)]),
    ("sq_get_output", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_uint64,
                              POINTER(c_double)]),
    ("sq_autotune_reset", c_int, []),
    ("sq_autotune_classes", c_int, [POINTER(c_uint64), POINTER(c_uint64)]),
    ("sq_get_output_sizing", c_int, [POINTER(c_int)]),
    ("sq_set_fwht_arithmetic", c_int, [c_int]),
    ("sq_set_single_pass_limit", c_int, [c_uint64]),
    ("sq_set_hash_groups_hint", c_int, [c_uint64]),
    ("sq_predictor_reset", c_int, [c_uint64]),
    ("sq_predictor_get_params", c_int, [c_void_p, c_uint64]),
    ("sq_predictor_set_params", c_int, [c_void_p, c_uint64]),
    ("sq_predictor_gradient", c_int, [c_void_p, c_void_p, c_uint64, c_void_p, POINTER(c_float)]),
    ("sq_predictor_predict", c_int, [c_void_p, c_uint64, c_void_p]),
    ("sq_predictor_train", c_int, [c_void_p, c_void_p, c_uint64, c_uint32, c_uint32, c_float, c_uint64,
                                   POINTER(c_float)]),
    ("sq_predictor_enable", c_int, [c_int]),
    ("sq_predictor_log_enable", c_int, [c_int]),
    ("sq_predictor_log_size", c_int, [POINTER(c_uint64)]),
    ("sq_predictor_log_read", c_int, [c_void_p, c_void_p, c_uint64, POINTER(c_uint64)]),
    ("sq_predictor_log_clear", c_int, []),
    ("sq_predictor_stats", c_int, [POINTER(c_uint64), POINTER(c_uint64)]),
    ("sq_get_fwht_arithmetic", c_int, [POINTER(c_int)]),
    ("sq_set_clearzero_eps", c_int, [c_double]),
    ("sq_set_wait_limit", c_int, [c_uint32]),
    ("sq_get_wait_limit", c_int, [POINTER(c_uint32)]),
    ("sq_selftest_wait_timeout", c_int, [c_uint32]),
    ("sq_device_allocation_count", c_int, [POINTER(c_uint64)]),
    ("sq_get_clearzero_eps", c_int, [POINTER(c_double)]),
    ("sq_clear_zero", c_int, [c_void_p, c_double]),
    ("sq_clear_zero_noalloc", c_int, [POINTER(c_void_p), c_void_p, c_uint32, c_uint64, c_double, POINTER(c_void_p),
                                      c_void_p, POINTER(c_uint64), c_void_p]),
    ("sq_normalize", c_int, [c_void_p, POINTER(c_double)]),
    ("sq_norm_sq", c_int, [c_void_p, POINTER(c_double)]),
    ("sq_add_systems", c_int, [c_void_p, c_void_p, c_double]),
    ("sq_add_register_sync", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_uint32)]),
    ("sq_add_register_with_hadamard", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_uint32)]),
    ("sq_remove_register_sync", c_int, [c_void_p, c_uint32]),
    ("sq_split_register", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_uint32)]),
    ("sq_combine_register", c_int, [c_void_p, c_uint32, c_uint32]),
]

EXPORTED = [s[0] for s in _SIGS]

_lib = None


def lib() -> ctypes.CDLL:
    """Load the engine (once). Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"native engine {LIB_PATH.name} is not built; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, res, args in _SIGS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SQ_OK:
        msg = lib().sq_last_error().decode(errors="replace")
        if rc == SQ_ERR_INVALID:
            raise SparQInvalid(rc, msg)
        raise SparQError(rc, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def profile_enable(on: bool) -> None:
    call("sq_profile_enable", 1 if on else 0)


def profile_reset() -> None:
    call("sq_profile_reset")


def profile_read(max_kernels: int = 64) -> dict:
    """{kernel name: (launches, total device ms, total algorithmic bytes)} from
    the engine's event timers."""
    buf = ctypes.create_string_buffer(64 * max_kernels)
    counts = (c_uint64 * max_kernels)()
    ms = (c_double * max_kernels)()
    nbytes = (c_double * max_kernels)()
    n = c_uint32()
    call("sq_profile_read", buf, len(buf), counts, ms, nbytes, max_kernels, ctypes.byref(n))
    names = buf.raw.split(b"\0")[: n.value]
    return {nm.decode(): (counts[i], ms[i], nbytes[i]) for i, nm in enumerate(names)}


def launch_count() -> int:
    v = c_uint64(0)
    call("sq_launch_count", ctypes.byref(v))
    return v.value
