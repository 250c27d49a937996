"""Writes tests/golden/reference_kats.json: known-answer cases taken from the
reference's own unit tests (SparQ/test/*.cpp, test/GPUTest/..., PySparQ/test/...).

Each case records the test it comes from (file:line in the SparQSim project),
the registers it declares, the initial register values of a single-entry
state (or a list of entries), the operators applied in order, and the
expected result exactly as that reference test asserts it (its expected-value
formula evaluated here). Run: python tests/golden/make_reference_kats.py
"""
from __future__ import annotations

import json
import math
from pathlib import Path

OUT = Path(__file__).with_name("reference_kats.json")
U, S, B, R = "UnsignedInteger", "SignedInteger", "Boolean", "Rational"


def sext(v, w):
    return v - (1 << w) if (v >> (w - 1)) & 1 else v


def isqrt(v):
    return math.isqrt(v)


def mask(w):
    return (1 << w) - 1 if w < 64 else (1 << 64) - 1


tables = {}


def single(src, regs, init, ops, expect):
    """One single-entry case; cases with the same (src, regs, ops) share a table
    whose rows are [initial values..., expected values...]."""
    key = json.dumps([src, regs, ops])
    t = tables.get(key)
    if t is None:
        t = tables[key] = {"src": src, "regs": regs, "ops": ops, "init_names": sorted(init),
                           "expect_names": sorted(expect), "rows": []}
    assert t["init_names"] == sorted(init) and t["expect_names"] == sorted(expect)
    t["rows"].append([init[k] for k in t["init_names"]] + [expect[k] for k in t["expect_names"]])


# ---- SparQ/test/quantum_arithmetic.cpp
single("SparQ/test/quantum_arithmetic.cpp:155-172", [["lhs", U, 4], ["rhs", U, 4], ["res", U, 4]],
       {"lhs": 3, "rhs": 5}, [["Add_UInt_UInt", "lhs", "rhs", "res"]], {"res": 8})
for lhs, rhs in [(7, 3), (0, 9), (15, 1), (11, 14)]:
    single("SparQ/test/quantum_arithmetic.cpp:175-194", [["lhs", U, 4], ["rhs", U, 4]], {"lhs": lhs, "rhs": rhs},
           [["Add_UInt_UInt_InPlace", "lhs", "rhs"]], {"lhs": lhs, "rhs": (lhs + rhs) & 0xF})
for lhs, start in [(6, 0), (15, 3), (9, 12)]:
    single("SparQ/test/quantum_arithmetic.cpp:196-215", [["lhs", U, 4], ["res", U, 4]], {"lhs": lhs, "res": start},
           [["Add_UInt_ConstUInt", "lhs", 4, "res"]], {"lhs": lhs, "res": start ^ ((lhs + 4) & 0xF)})
single("SparQ/test/quantum_arithmetic.cpp:217-234", [["reg", U, 4]], {"reg": 12},
       [["Add_ConstUInt_InPlace", "reg", 3]], {"reg": 15})
for lhs, start in [(3, 0), (7, 5), (15, 10)]:
    single("SparQ/test/quantum_arithmetic.cpp:236-257", [["lhs", U, 4], ["res", U, 4]], {"lhs": lhs, "res": start},
           [["Mult_UInt_ConstUInt", "lhs", 4, "res"]], {"lhs": lhs, "res": start ^ ((lhs * 4) & 0xF)})
for lhs, res in [(1, 2), (0, 7), (7, 5), (15, 15)]:
    single("SparQ/test/quantum_arithmetic.cpp:259-280", [["lhs", U, 4], ["res", U, 4]], {"lhs": lhs, "res": res},
           [["Add_Mult_UInt_ConstUInt_InPlace", "lhs", 2, "res"]], {"lhs": lhs, "res": (res + lhs * 2) & 0xF})
for v in range(16):
    single("SparQ/test/quantum_arithmetic.cpp:282-296", [["reg", U, 4]], {"reg": v}, [["FlipBools", "reg"]],
           {"reg": v ^ 0xF})
single("SparQ/test/quantum_arithmetic.cpp:298-316", [["src", U, 4], ["dst", U, 4]], {"src": 7, "dst": 0},
       [["Assign", "src", "dst"]], {"dst": 7})
single("SparQ/test/quantum_arithmetic.cpp:318-340", [["l", U, 4], ["r", U, 4], ["lt", B, 1], ["eq", B, 1]],
       {"l": 3, "r": 3}, [["Compare_UInt_UInt", "l", "r", "lt", "eq"]], {"eq": 1, "lt": 0})
for a, b in [(8, 6), (0, 9), (15, 1), (12, 11)]:
    single("SparQ/test/quantum_arithmetic.cpp:342-363", [["lhs", U, 4], ["rhs", U, 4]], {"lhs": a, "rhs": b},
           [["Add_AnyInt_AnyInt_InPlace", "lhs", "rhs"]], {"lhs": (a + b) & 0xF, "rhs": b})
single("SparQ/test/quantum_arithmetic.cpp:389-409", [["left", U, 4], ["right", U, 4], ["mid", U, 4]],
       {"left": 0, "right": 10}, [["GetMid_UInt_UInt", "left", "right", "mid"]], {"mid": 5})
for v in [0, 1, 3, 7]:
    for sh in (1, 2, 3):
        single("SparQ/test/quantum_arithmetic.cpp:503-522", [["reg", U, 3]], {"reg": v},
               [["ShiftLeft_InPlace", "reg", sh], ["ShiftLeft_InPlace.dag", "reg", sh]], {"reg": v})
        single("SparQ/test/quantum_arithmetic.cpp:524-542", [["reg", U, 3]], {"reg": v},
               [["ShiftRight_InPlace", "reg", sh], ["ShiftRight_InPlace.dag", "reg", sh]], {"reg": v})
single("SparQ/test/quantum_arithmetic.cpp:584-602", [["reg", U, 4]], {"reg": 3},
       [["Mod_Mult_UInt_ConstUInt_InPlace", "reg", 7, 0, 15]], {"reg": 6})
single("SparQ/test/quantum_arithmetic.cpp:604-624", [["reg", U, 4]], {"reg": 1},
       [["Mod_Mult_UInt_ConstUInt_InPlace", "reg", 7, 2, 15]], {"reg": 1})
for ctrl in (0, 1):
    single("SparQ/test/quantum_arithmetic.cpp:626-643", [["reg", U, 4], ["ctrl", B, 1]], {"reg": 3, "ctrl": ctrl},
           [["Mod_Mult_UInt_ConstUInt_InPlace@all_ones:ctrl", "reg", 7, 0, 15]], {"reg": 6 if ctrl else 3, "ctrl": ctrl})
for a in range(8):
    for b in range(32):
        single("SparQ/test/quantum_arithmetic.cpp:766-790", [["l", U, 3], ["r", U, 5], ["res", U, 4]],
               {"l": a, "r": b, "res": 0}, [["Sub_UInt_UInt", "l", "r", "res"]], {"res": (a - b) & 0xF})
single("SparQ/test/quantum_arithmetic.cpp:791-799", [["l", U, 3], ["r", U, 5], ["res", U, 4]],
       {"l": 1, "r": 2, "res": 0xF}, [["Sub_UInt_UInt", "l", "r", "res"]], {"res": 0xF ^ ((1 - 2) & 0xF)})
for v in range(8):
    single("SparQ/test/quantum_arithmetic.cpp:802-826", [["reg", U, 3], ["res", U, 5]], {"reg": v},
           [["Neg_UInt", "reg", "res"]], {"res": (0 - v) & 0x1F})
for v in range(32):
    single("SparQ/test/quantum_arithmetic.cpp:802-826", [["reg", U, 5], ["res", U, 3]], {"reg": v},
           [["Neg_UInt", "reg", "res"]], {"res": (0 - v) & 0x7})
for bits in range(16):
    v = sext(bits, 4)
    single("SparQ/test/quantum_arithmetic.cpp:828-855", [["reg", S, 4], ["res", U, 5]], {"reg": bits},
           [["Abs_SInt", "reg", "res"]], {"res": abs(v) & 0x1F})
for bits in range(32):
    v = sext(bits, 5)
    single("SparQ/test/quantum_arithmetic.cpp:828-855", [["reg", S, 5], ["res", U, 3]], {"reg": bits},
           [["Abs_SInt", "reg", "res"]], {"res": abs(v) & 0x7})
for a in range(8):
    for b in range(8):
        single("SparQ/test/quantum_arithmetic.cpp:857-889", [["l", U, 3], ["r", U, 3], ["res", U, 4]],
               {"l": a, "r": b}, [["Mul_UInt_UInt", "l", "r", "res"]], {"res": (a * b) & 0xF})
for a in range(32):
    for b in range(8):
        single("SparQ/test/quantum_arithmetic.cpp:891-914", [["l", U, 5], ["r", U, 3], ["res", U, 5]],
               {"l": a, "r": b}, [["Div_UInt_UInt", "l", "r", "res"]], {"res": 0 if b == 0 else a // b})
for v in range(16):
    single("SparQ/test/quantum_arithmetic.cpp:916-930", [["reg", U, 4], ["res", U, 3]], {"reg": v},
           [["Sqrt_UInt", "reg", "res"]], {"res": isqrt(v) & 0x7})
for c in range(2):
    for a in range(8):
        for b in range(0, 32, 3):
            single("SparQ/test/quantum_arithmetic.cpp:932-958", [["c", B, 1], ["l", U, 3], ["r", U, 5], ["res", U, 4]],
                   {"c": c, "l": a, "r": b}, [["Select_Bool_UInt_UInt", "c", "l", "r", "res"]],
                   {"res": (a & 0xF) if c else (b & 0xF)})
for a in range(8):
    for b in range(32):
        single("SparQ/test/quantum_arithmetic.cpp:960-990",
               [["l", U, 3], ["r", U, 5], ["ra", U, 4], ["ro", U, 4], ["rx", U, 4]], {"l": a, "r": b},
               [["And_UInt_UInt", "l", "r", "ra"], ["Or_UInt_UInt", "l", "r", "ro"], ["Xor_UInt_UInt", "l", "r", "rx"]],
               {"ra": (a & b) & 0xF, "ro": (a | b) & 0xF, "rx": (a ^ b) & 0xF})
for lb in range(16):
    for rb in range(8):
        single("SparQ/test/quantum_arithmetic.cpp:993-1016", [["l", S, 4], ["r", S, 3], ["f", B, 1]],
               {"l": lb, "r": rb}, [["Less_SInt_SInt", "l", "r", "f"]], {"f": 1 if sext(lb, 4) < sext(rb, 3) else 0})
for a in range(8):
    for b in range(16):
        single("SparQ/test/quantum_arithmetic.cpp:1019-1043", [["l", U, 3], ["r", U, 4], ["res", U, 3], ["f", B, 1]],
               {"l": a, "r": b}, [["Carry_UInt_UInt", "l", "r", "res", "f"]],
               {"f": 1 if (a >= 8 or b >= 8 - a) else 0})
M = (1 << 64) - 1
for (a, b), e in [((M, 1), 1), ((1, 1), 0), ((M, M), 1), ((M - 1, 1), 0)]:
    single("SparQ/test/quantum_arithmetic.cpp:1045-1087",
           [["l", U, 64], ["r", U, 64], ["res", U, 64], ["f", B, 1]],
           {"l": a, "r": b, "res": 0x123456789ABCDEF0}, [["Carry_UInt_UInt", "l", "r", "res", "f"]],
           {"f": e, "res": 0x123456789ABCDEF0})


def ovf(l, r, w):
    m = mask(w)
    A, Bv = l & m, r & m
    Sm = (A + Bv) & m
    sa, sb, ss = (A >> (w - 1)) & 1, (Bv >> (w - 1)) & 1, (Sm >> (w - 1)) & 1
    return 1 if (sa == sb and ss != sa) else 0


for lb in range(16):
    for rb in range(8):
        l, r = sext(lb, 4), sext(rb, 3)
        single("SparQ/test/quantum_arithmetic.cpp:1090-1130",
               [["l", S, 4], ["r", S, 3], ["r4", U, 4], ["r3", U, 3], ["f4", B, 1], ["f3", B, 1]],
               {"l": lb, "r": rb},
               [["Overflow_SInt_SInt", "l", "r", "r4", "f4"], ["Overflow_SInt_SInt", "l", "r", "r3", "f3"]],
               {"f4": ovf(l, r, 4), "f3": ovf(l, r, 3)})
for a in range(8):
    for b in range(8):
        single("SparQ/test/quantum_arithmetic.cpp:1132-1158",
               [["l", U, 3], ["r", U, 3], ["r4", U, 4], ["r6", U, 6], ["f4", B, 1], ["f6", B, 1]],
               {"l": a, "r": b},
               [["MulOverflow_UInt_UInt", "l", "r", "r4", "f4"], ["MulOverflow_UInt_UInt", "l", "r", "r6", "f6"]],
               {"f4": 1 if a * b >= 16 else 0, "f6": 1 if a * b >= 64 else 0})
for v in range(8):
    single("SparQ/test/quantum_arithmetic.cpp:1160-1194", [["reg", U, 3], ["f", B, 1]], {"reg": v},
           [["IsZero_UInt", "reg", "f"]], {"f": 1 if v == 0 else 0})
for bits in range(16):
    single("SparQ/test/quantum_arithmetic.cpp:1160-1194", [["reg", S, 4], ["f", B, 1]], {"reg": bits},
           [["Negative_SInt", "reg", "f"]], {"f": 1 if sext(bits, 4) < 0 else 0})


def sample_values(w):
    # small sweep when the operand space is small, otherwise 0, 1, all-ones and a few mids
    m = mask(w)
    return sorted({0, 1, m, m // 2, (m // 2) + 1, m // 3})


for lw in (1, 2, 3, 5, 8):
    for rw in (1, 2, 3, 5, 8):
        for ow in (1, 2, 4, 8):
            full = lw + rw <= 6
            lv = range(1 << lw) if full else sample_values(lw)
            rv = range(1 << rw) if full else sample_values(rw)
            for a in lv:
                for b in rv:
                    single("SparQ/test/quantum_arithmetic.cpp:1197-1250",
                           [["l", U, lw], ["r", U, rw], ["ra", U, ow], ["rm", U, ow], ["rd", U, ow]], {"l": a, "r": b},
                           [["Add_UInt_UInt", "l", "r", "ra"], ["Mul_UInt_UInt", "l", "r", "rm"],
                            ["Div_UInt_UInt", "l", "r", "rd"]],
                           {"ra": (a + b) & mask(ow), "rm": (a * b) & mask(ow),
                            "rd": (0 if b == 0 else a // b) & mask(ow)})
for a in range(16):
    for b in range(16):
        single("SparQ/test/quantum_arithmetic.cpp:1253-1272", [["l", U, 4], ["r", U, 4]], {"l": a, "r": b},
               [["Add_AnyInt_AnyInt_InPlace", "l", "r"]], {"l": (a + b) & 0xF, "r": b})
for a in range(64):
    for rb in range(8):
        single("SparQ/test/quantum_arithmetic.cpp:1274-1295", [["l", U, 6], ["r", S, 3]], {"l": a, "r": rb},
               [["Add_AnyInt_AnyInt_InPlace", "l", "r"]], {"l": (a + sext(rb, 3)) & 0x3F, "r": rb})
        single("SparQ/test/quantum_arithmetic.cpp:1297-1324", [["l", U, 6], ["r", S, 3]], {"l": a, "r": rb},
               [["Add_AnyInt_AnyInt_InPlace", "l", "r"], ["Add_AnyInt_AnyInt_InPlace.dag", "l", "r"]], {"l": a, "r": rb})

# ---- SparQ/test/basic_gates.cpp
s2 = 1 / math.sqrt(2)
single("SparQ/test/basic_gates.cpp:31-42", [["q", B, 1]], {"q": 0}, [["X_Bool", "q"]], {"q": 1, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:44-56", [["q", B, 1]], {"q": 1}, [["X_Bool", "q"]], {"q": 0, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:58-70", [["q", B, 1]], {"q": 0}, [["X_Bool", "q"], ["X_Bool", "q"]],
       {"q": 0, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:74-86", [["q", B, 1]], {"q": 0}, [["Y_Bool", "q"]], {"q": 1, "@amp": [0, 1]})
single("SparQ/test/basic_gates.cpp:88-101", [["q", B, 1]], {"q": 1}, [["Y_Bool", "q"]], {"q": 0, "@amp": [0, -1]})
single("SparQ/test/basic_gates.cpp:105-117", [["q", B, 1]], {"q": 0}, [["Z_Bool", "q"]], {"q": 0, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:119-132", [["q", B, 1]], {"q": 1}, [["Z_Bool", "q"]], {"q": 1, "@amp": [-1, 0]})
single("SparQ/test/basic_gates.cpp:136-147", [["q", B, 1]], {"q": 0}, [["S_Bool", "q"]], {"q": 0, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:149-161", [["q", B, 1]], {"q": 1}, [["S_Bool", "q"]], {"q": 1, "@amp": [0, 1]})
single("SparQ/test/basic_gates.cpp:163-177", [["q", B, 1]], {"q": 1}, [["S_Bool", "q"], ["S_Bool", "q"]],
       {"q": 1, "@amp": [-1, 0]})
single("SparQ/test/basic_gates.cpp:181-192", [["q", B, 1]], {"q": 0}, [["T_Bool", "q"]], {"q": 0, "@amp": [1, 0]})
single("SparQ/test/basic_gates.cpp:194-208", [["q", B, 1]], {"q": 1}, [["T_Bool", "q"]],
       {"q": 1, "@amp": [math.cos(math.pi / 4), math.sin(math.pi / 4)]})
single("SparQ/test/basic_gates.cpp:210-226", [["q", B, 1]], {"q": 1}, [["T_Bool", "q"]] * 4, {"q": 1, "@amp": [-1, 0]})
single("SparQ/test/basic_gates.cpp:229-246", [["q", U, 2]], {"q": 0},
       [["X_Bool", "q", 0], ["X_Bool", "q", 1], ["X_Bool", "q", 0]], {"q": 2})
# ---- SparQ/test/condrot.cpp (Phase_Bool KATs and CondRot on |0>)
single("SparQ/test/condrot.cpp:55-67", [["q", B, 1]], {"q": 1}, [["Phase_Bool", "q", 0, math.pi / 2]],
       {"q": 1, "@amp": [math.cos(math.pi / 2), math.sin(math.pi / 2)]})
single("SparQ/test/condrot.cpp:69-80", [["q", B, 1]], {"q": 1}, [["Phase_Bool", "q", 0, math.pi]], {"@amp": [-1, 0]})
single("SparQ/test/condrot.cpp:22-34", [["in", R, 1], ["out", B, 1]], {}, [["CondRot_Rational_Bool", "in", "out"]],
       {"out": 0, "@size": 1})
single("SparQ/test/condrot.cpp:82-95", [["in", R, 2], ["out", B, 1]], {}, [["CondRot_Rational_Bool", "in", "out"]],
       {"out": 0, "@size": 1})

# ---- multi-entry known answers
multi = []
# SparQ/test/hadamard.cpp:14-111
multi.append({"src": "SparQ/test/hadamard.cpp:14-42", "regs": [["q", B, 1]], "init": [{"q": 0}],
              "ops": [["Hadamard_Int_Full", "q"]], "expect": [[[0], [s2, 0]], [[1], [s2, 0]]]})
multi.append({"src": "SparQ/test/hadamard.cpp:44-73", "regs": [["q", B, 1]], "init": [{"q": 1}],
              "ops": [["Hadamard_Int_Full", "q"]], "expect": [[[0], [s2, 0]], [[1], [-s2, 0]]]})
multi.append({"src": "SparQ/test/hadamard.cpp:75-90", "regs": [["q", B, 1]], "init": [{"q": 0}],
              "ops": [["Hadamard_Int_Full", "q"], ["Hadamard_Int_Full", "q"]], "expect": [[[0], [1, 0]]]})
multi.append({"src": "SparQ/test/hadamard.cpp:92-111", "regs": [["q", U, 2]], "init": [{"q": 0}],
              "ops": [["Hadamard_Int_Full", "q"]], "expect": [[[v], [0.5, 0]] for v in range(4)]})
# test/GPUTest/Benchmark/CudaBenchmark.cu:13-18, 188-218 (analytic spot checks, n = 8)
n = 8
ph = complex(math.cos(math.pi / 5), math.sin(math.pi / 5))
inv = 1 / math.sqrt(2 ** n)
th = math.pi / 3
exp = []
for k in range(1 << n):
    a1 = 0.5 * ph * inv
    a0 = -math.sqrt(3) / 2 * ph * inv
    exp.append([[k, 2 * k, isqrt(k), 1], [a1.real, a1.imag]])
    exp.append([[k, 2 * k, isqrt(k), 0], [a0.real, a0.imag]])
multi.append({"src": "test/GPUTest/Benchmark/CudaBenchmark.cu:13-18,96-118,188-218",
              "regs": [["addr", U, n], ["sum", U, n + 1], ["sq", U, n // 2 + 1], ["b", U, 1]],
              "init": [{}],
              "ops": [["Hadamard_Int", "addr", n], ["Add_UInt_UInt", "addr", "addr", "sum"], ["Sqrt_UInt", "addr", "sq"],
                      ["X_Bool", "b"], ["Rot_Bool", "b", 0, [[math.cos(th), 0], [-math.sin(th), 0], [math.sin(th), 0],
                                                             [math.cos(th), 0]]],
                      ["GlobalPhase", [ph.real, ph.imag]], ["Normalize"]],
              "expect": exp})
# PySparQ/test/test_semantic_conformance.py:430-489 — QRAMLoad data ^= memory[addr] over every address
mem = [(i * 3 + 1) % 16 for i in range(8)]
for addr in range(8):
    for d0 in (0, 5, 15):
        single("PySparQ/test/test_semantic_conformance.py:430-489",
               [["addr", U, 3], ["data", U, 4]], {"addr": addr, "data": d0},
               [["QRAMLoad", [3, 4, mem], "addr", "data"]], {"addr": addr, "data": d0 ^ mem[addr]})

doc = {"generator": "tests/golden/make_reference_kats.py", "tables": list(tables.values()), "multi": multi}
OUT.write_text(json.dumps(doc, separators=(",", ":")))
nrows = sum(len(t["rows"]) for t in tables.values())
print(f"wrote {OUT} ({len(tables)} tables, {nrows} single-entry cases, {len(multi)} multi-entry cases)")
