"""CPU-only checks of the C ABI: the shared library loads, exports every entry
point include/sparq_gb300.h declares, the struct layouts match, and the
process-global register table (System) behaves like the reference's
(basic_components.cpp:226-459) — all without a GPU."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300 import _native

HEADER = Path(__file__).resolve().parent.parent / "include" / "sparq_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(sq_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_native.LIB_PATH))
    names = declared_functions()
    assert len(names) > 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers exactly the declared surface
    assert sorted(_native.EXPORTED) == names


def test_abi_version_and_struct_sizes():
    lib = _native.lib()
    assert lib.sq_abi_version() == 1
    assert ctypes.sizeof(_native.SqCondition) == 16
    assert ctypes.sizeof(_native.SqCond) == 8 + 16 * _native.SQ_MAX_CONDITIONS
    assert ctypes.sizeof(_native.SqInstr) == 256


def test_register_ids_reuse_lifo_like_reference():
    a = ps.System.add_register("a", ps.UnsignedInteger, 12)
    b = ps.System.add_register("b", ps.UnsignedInteger, 16)
    c = ps.System.add_register("c", ps.UnsignedInteger, 16)
    assert (a, b, c) == (0, 1, 2)
    ps.System.remove_register("b")
    ps.System.remove_register("a")
    # reusable_registers is a stack: the last freed id comes back first
    assert ps.System.add_register("x", ps.Boolean, 1) == a
    assert ps.System.add_register("y", ps.Boolean, 1) == b
    assert ps.System.add_register("z", ps.Boolean, 1) == 3
    assert ps.System.get_id("c") == c
    assert ps.System.size_of("x") == 1 and ps.System.type_of("c") == ps.UnsignedInteger
    with pytest.raises(ValueError):
        ps.System.get_id("b")


def test_register_packing_first_fit_without_straddling():
    widths = [12, 16, 16, 30, 20, 64, 1]
    ids = [ps.System.add_register(f"r{i}", ps.UnsignedInteger, w) for i, w in enumerate(widths)]
    fields = [ps.System._info(i)[3:] for i in ids]
    used = {}
    for (word, shift), w in zip(fields, widths):
        assert shift + w <= 64, "register straddles two key words"
        for bit in range(shift, shift + w):
            assert (word, bit) not in used, "overlapping registers"
            used[(word, bit)] = True
    assert ps.System.key_words() == 3  # 12+16+16+1 | 30+20 | 64
    assert ps.System.get_qubit_count() == sum(widths)


def test_removed_bits_are_reused():
    ps.System.add_register("a", ps.UnsignedInteger, 60)
    ps.System.add_register("b", ps.UnsignedInteger, 4)
    assert ps.System.key_words() == 1
    ps.System.remove_register("a")
    ps.System.add_register("c", ps.UnsignedInteger, 50)
    assert ps.System.key_words() == 1


def test_width_limits_and_errors_are_statuses():
    with pytest.raises(ValueError):
        ps.System.add_register("big", ps.UnsignedInteger, 65)
    lib = _native.lib()
    assert lib.sq_system_remove_register(999) == _native.SQ_ERR_INVALID
    assert b"not found" in lib.sq_last_error()
    # key space: 8 words of 64 bits
    for i in range(8):
        ps.System.add_register(f"w{i}", ps.UnsignedInteger, 64)
    rid = ctypes.c_uint32()
    assert lib.sq_system_add_register(1, 1, ctypes.byref(rid)) == _native.SQ_ERR_CAPACITY


def test_operator_construction_validates_like_reference():
    ps.System.add_register("a", ps.UnsignedInteger, 4)
    ps.System.add_register("q", ps.Boolean, 1)
    ps.System.add_register("wide", ps.UnsignedInteger, 3)
    with pytest.raises(ValueError):
        ps.Hadamard_Bool("wide")          # Hadamard_Bool needs a 1-bit register
    with pytest.raises(ValueError):
        ps.X_Bool("a", 4)                 # digit >= register size (GateBase)
    with pytest.raises(ValueError):
        ps.CondRot_Rational_Bool("a", "q")  # input must be Rational
    with pytest.raises(ValueError):
        ps.Mod_Mult_UInt_ConstUInt_InPlace("a", 6, 1, 15)  # a and N not coprime
    op = ps.Add_UInt_UInt("a", "a", "wide").conditioned_by_nonzeros(["q"]).conditioned_by_bit("a", 1)
    c = op._cond()
    assert c.count == 2 and c.c[0].kind == _native.COND_NONZERO and c.c[1].kind == _native.COND_BIT
    # conditioned_by_* replaces conditions of the same kind (global_macros.h:112-127)
    op.conditioned_by_nonzeros("a")
    assert op.condition_variable_nonzeros == [0]


def test_fused_dag_reverses_and_inverts():
    ps.System.add_register("a", ps.UnsignedInteger, 8)
    ps.System.add_register("b", ps.UnsignedInteger, 8)
    chain = ps.Fused([ps.Add_UInt_UInt_InPlace("a", "b"), ps.Add_ConstUInt_InPlace("b", 3), ps.X_Bool("a", 0)])
    fwd = chain.spec(False)[1]
    inv = chain.spec(True)[1]
    assert [i.op for i in inv] == [i.op for i in reversed(fwd)]
    assert [i.dag for i in inv] == [0, 1, 1]
    with pytest.raises(TypeError):
        ps.Fused([ps.Hadamard_Int("a", 2)])


def test_clearzero_default_eps_survives_system_clear():
    """clearzero_default_eps is a global of its own
    (system_operations.h:577): System::clear leaves it as it was."""
    saved = ps.get_clearzero_default_eps()
    try:
        ps.set_clearzero_default_eps(3e-15)
        ps.System.clear()
        assert ps.get_clearzero_default_eps() == 3e-15
    finally:
        ps.set_clearzero_default_eps(saved)
        ps.System.clear()
