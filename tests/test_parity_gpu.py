"""GPU engine vs the CPU oracle, operator by operator, on seeded random
states: keys bit-exact, amplitudes bit-exact where the arithmetic order is
fixed (elementwise ops, FWHT, pair formulas) and within 1e-12 relative
otherwise. Modelled on the reference's CPU-vs-GPU harness
(test/GPUTest/Benchmark/CudaBenchmark.cu:40-74, key-sorted comparison)."""
from __future__ import annotations

import math
import zlib

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


@pytest.fixture(params=["sort", "hash", "hash-exact", "sort-fix", "hash-fix", "auto"])
def strategy(request, dual):
    """Grouping strategy x output sizing x FWHT arithmetic. The '-fix' cases
    run the Hadamard butterflies in exact-sum arithmetic: keys stay bit-exact,
    amplitudes are held to 1e-12 relative (of the largest) instead of bit-exact.
    'auto' (as the default 'autotune') runs 1-bit splits by partner lookup."""
    ps.set_group_strategy(request.param.split("-")[0])
    ps.set_output_sizing("exact" if request.param.endswith("exact") else "auto")
    if request.param.endswith("fix"):
        ps.set_fwht_arithmetic("exact-sum")
        dual.relaxed = True
    yield request.param
    ps.set_group_strategy("autotune")
    ps.set_output_sizing("auto")


def random_state(rng, widths, n, types=None):
    """n distinct random keys over registers of the given widths."""
    keys = set()
    limit = 1
    for w in widths:
        limit *= 1 << w
    n = min(n, limit)
    out = []
    while len(out) < n:
        k = tuple(int(rng.integers(0, 1 << w)) if w < 63 else int(rng.integers(0, 1 << 62)) for w in widths)
        if k not in keys:
            keys.add(k)
            out.append(k)
    regs = np.array(out, dtype=np.uint64).reshape(n, len(widths))
    amps = rng.normal(size=n) + 1j * rng.normal(size=n)
    amps /= np.linalg.norm(amps)
    return regs, amps


def grouped_state(rng, widths, target, n_digits, groups, fill):
    """States whose groups (equal except the low n_digits of register `target`)
    hold a chosen number of members: fill(i) -> members of group i."""
    rows = []
    seen = set()
    for g in range(groups):
        base = [int(rng.integers(0, 1 << w)) for w in widths]
        base[target] &= ~((1 << n_digits) - 1)
        # groups must differ outside the whole target register: the reference
        # groups by every other register, so two groups that differ only in
        # the target's high bits would be one (undefined) reference group
        key0 = tuple(v for i, v in enumerate(base) if i != target)
        if key0 in seen:
            continue
        seen.add(key0)
        m = fill(g)
        for t in rng.choice(1 << n_digits, size=m, replace=False):
            r = list(base)
            r[target] |= int(t)
            rows.append(r)
    regs = np.array(rows, dtype=np.uint64)
    amps = rng.normal(size=len(rows)) + 1j * rng.normal(size=len(rows))
    amps /= np.linalg.norm(amps)
    return regs, amps


# ----------------------------------------------------------------- elementwise
ELEMENTWISE_CASES = [
    ("Add_UInt_UInt", lambda: ps.Add_UInt_UInt("a", "b", "c")),
    ("Sub_UInt_UInt", lambda: ps.Sub_UInt_UInt("a", "b", "c")),
    ("Mul_UInt_UInt", lambda: ps.Mul_UInt_UInt("a", "b", "c")),
    ("Div_UInt_UInt", lambda: ps.Div_UInt_UInt("a", "b", "c")),
    ("And", lambda: ps.And_UInt_UInt("a", "b", "c")),
    ("Or", lambda: ps.Or_UInt_UInt("a", "b", "c")),
    ("Xor", lambda: ps.Xor_UInt_UInt("a", "b", "c")),
    ("Less_UInt", lambda: ps.Less_UInt_UInt("a", "b", "f")),
    ("Less_SInt", lambda: ps.Less_SInt_SInt("s", "a", "f")),
    ("GetMid", lambda: ps.GetMid_UInt_UInt("a", "m", "c")),
    ("Neg", lambda: ps.Neg_UInt("a", "c")),
    ("Abs", lambda: ps.Abs_SInt("s", "c")),
    ("Sqrt", lambda: ps.Sqrt_UInt("b", "c")),
    ("IsZero", lambda: ps.IsZero_UInt("a", "f")),
    ("Negative", lambda: ps.Negative_SInt("s", "f")),
    ("Carry", lambda: ps.Carry_UInt_UInt("a", "b", "c", "f")),
    ("Overflow", lambda: ps.Overflow_SInt_SInt("s", "a", "c", "f")),
    ("MulOverflow", lambda: ps.MulOverflow_UInt_UInt("a", "b", "c", "f")),
    ("Select", lambda: ps.Select_Bool_UInt_UInt("f", "a", "b", "c")),
    ("Compare", lambda: ps.Compare_UInt_UInt("a", "b", "f", "g")),
    ("Assign", lambda: ps.Assign("a", "c")),
    ("Swap", lambda: ps.Swap_General_General("a", "a2")),
    ("FlipBools", lambda: ps.FlipBools("b")),
    ("Swap_Bool_Bool", lambda: ps.Swap_Bool_Bool("a", 2, "b", 5)),
    ("ShiftLeft", lambda: ps.ShiftLeft_InPlace("b", 3)),
    ("ShiftRight", lambda: ps.ShiftRight_InPlace("b", 5)),
    ("Add_UInt_ConstUInt", lambda: ps.Add_UInt_ConstUInt("a", 77, "c")),
    ("Mult_UInt_ConstUInt", lambda: ps.Mult_UInt_ConstUInt("a", 12345, "c")),
    ("Add_Mult_InPlace", lambda: ps.Add_Mult_UInt_ConstUInt_InPlace("a", 99, "c")),
    ("Add_ConstUInt_InPlace", lambda: ps.Add_ConstUInt_InPlace("b", 1000)),
    ("Add_InPlace", lambda: ps.Add_UInt_UInt_InPlace("a", "b")),
    ("AnyInt_InPlace", lambda: ps.Add_AnyInt_AnyInt_InPlace("b", "s")),
    ("Mod_Mult", lambda: ps.Mod_Mult_UInt_ConstUInt_InPlace("m", 7, 2, 15)),
    ("X_Bool", lambda: ps.X_Bool("b", 4)),
    ("Y_Bool", lambda: ps.Y_Bool("b", 1)),
    ("Phase_Bool", lambda: ps.Phase_Bool("c", 0, 0.37)),
    ("Z_Bool", lambda: ps.Z_Bool("f")),
    ("S_Bool", lambda: ps.S_Bool("f")),
    ("T_Bool", lambda: ps.T_Bool("f")),
    ("GlobalPhase", lambda: ps.GlobalPhase(complex(math.cos(0.3), math.sin(0.3)))),
    ("Reflection", lambda: ps.Reflection_Bool(["f", "g"], False)),
    ("Reflection_inv", lambda: ps.Reflection_Bool("f", True)),
    ("ZeroCondFlip", lambda: ps.ZeroConditionalPhaseFlip(["f", "g"])),
    ("Init_Unsafe", lambda: ps.Init_Unsafe("c", 5)),
]


def _arith_registers(dual):
    dual.reg("a", U, 12)
    dual.reg("b", U, 20)
    dual.reg("c", U, 16)
    dual.reg("f", ps.Boolean, 1)
    dual.reg("g", ps.Boolean, 1)
    dual.reg("s", ps.SignedInteger, 9)
    dual.reg("m", U, 4)
    dual.reg("a2", U, 12)
    return [12, 20, 16, 1, 1, 9, 4, 12]


@pytest.mark.parametrize("name,make", ELEMENTWISE_CASES, ids=[c[0] for c in ELEMENTWISE_CASES])
@pytest.mark.parametrize("cond", ["none", "nonzero", "bit", "value"])
def test_elementwise_vs_oracle(dual, name, make, cond):
    widths = _arith_registers(dual)
    rng = np.random.default_rng(zlib.crc32(f"{name}/{cond}".encode()))
    regs, amps = random_state(rng, widths, 3000)
    regs[:, 6] %= 15  # Mod_Mult acts on values < N
    dual.start(regs, amps)
    op = make()
    if cond == "nonzero":
        op.conditioned_by_nonzeros("g")
    elif cond == "bit":
        op.conditioned_by_bit("m", 1)
    elif cond == "value":
        op.conditioned_by_value("m", 3)
    dual.apply(op)
    dual.compare(exact_amp=True)
    if not op.self_adjoint:
        dual.apply(op, dag=True)
        dual.compare(exact_amp=True)
        # forward then adjoint is the identity on keys
        g = dual.gpu.to_dict()
        assert set(g.keys()) == {tuple(int(v) for v in r) for r in regs}


def test_fused_program_equals_sequence(dual):
    widths = _arith_registers(dual)
    rng = np.random.default_rng(7)
    regs, amps = random_state(rng, widths, 5000)
    regs[:, 6] %= 15
    dual.start(regs, amps)
    chain = [ps.Add_UInt_UInt("a", "b", "c"), ps.Mul_UInt_UInt("a", "b", "c").conditioned_by_nonzeros("f"),
             ps.Phase_Bool("c", 0, 0.37), ps.Add_UInt_UInt_InPlace("a", "b"), ps.X_Bool("g", 0),
             ps.GlobalPhase(1j).conditioned_by_bit("b", 3), ps.ShiftLeft_InPlace("c", 5)]
    fused = ps.Fused(chain)
    fused(dual.gpu)
    for op in chain:
        dual.O.apply(dual.ora, op.spec(False))
    dual.compare(exact_amp=True)
    before = ps.launch_count()
    fused.dag(dual.gpu)
    assert ps.launch_count() - before == 1  # one pass for the whole chain
    for op in reversed(chain):
        dual.O.apply(dual.ora, op.spec(not op.self_adjoint))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("addr_bits,data_bits", [(12, 16), (10, 32), (6, 48)])
def test_qram_load(dual, addr_bits, data_bits):
    dual.reg("addr", U, addr_bits + 2)
    dual.reg("data", U, data_bits)
    dual.reg("x", U, 5)
    rng = np.random.default_rng(addr_bits)
    table = rng.integers(0, 1 << min(data_bits, 62), 1 << addr_bits, dtype=np.uint64)
    q = dual.qram(addr_bits, data_bits, table)
    regs, amps = random_state(rng, [addr_bits + 2, data_bits, 5], 4000)
    dual.start(regs, amps)
    dual.apply(ps.QRAMLoad(q, "addr", "data"))
    dual.compare(exact_amp=True)
    dual.apply(ps.QRAMLoad(q, "addr", "data").conditioned_by_bit("x", 2))
    dual.compare(exact_amp=True)


def test_sparse_matrix_address_and_search(dual):
    """GetRowAddr / GetDataAddr (XOR of offset + row_sz * row (+ col)) and
    QuantumBinarySearch_Fast (a bisection of sorted runs of QRAM words per
    entry, hamiltonian_simulation.cpp:182-253): keys bit-exact; hits, misses
    and a conditioned form."""
    dual.reg("off", U, 10)
    dual.reg("row", U, 6)
    dual.reg("col", U, 3)
    dual.reg("out", U, 12)
    dual.reg("tgt", U, 12)
    dual.reg("res", U, 12)
    dual.reg("x", U, 2)
    rng = np.random.default_rng(77)
    # 64 rows of 8 sorted distinct words at 512 + 8 row: searched by row
    table = np.zeros(1 << 10, dtype=np.uint64)
    for r in range(64):
        table[512 + 8 * r: 512 + 8 * r + 8] = np.sort(rng.choice(4000, 8, replace=False))
    q = dual.qram(10, 12, table)
    n = 3000
    rows = rng.integers(0, 64, n)
    tg = np.where(rng.random(n) < 0.7, table[512 + 8 * rows + rng.integers(0, 8, n)], rng.integers(0, 4096, n))
    regs = np.stack([np.full(n, 512), rows, rng.integers(0, 8, n), rng.integers(0, 4096, n), tg,
                     np.zeros(n), rng.integers(0, 4, n)], axis=1).astype(np.uint64)
    regs = np.unique(regs, axis=0)
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    dual.start(regs, amps / np.linalg.norm(amps))
    dual.apply(ps.GetRowAddr("off", "row", 8, "out"))
    dual.compare(exact_amp=True)
    dual.apply(ps.GetDataAddr("off", "row", "col", 8, "out"))
    dual.compare(exact_amp=True)
    dual.apply(ps.GetRowAddr("off", "row", 8, "out"))  # out = its start value ^ data_addr
    dual.compare(exact_amp=True)
    dual.apply(ps.Init_Unsafe("out", 0))
    dual.apply(ps.GetRowAddr("off", "row", 8, "out"))  # out = 512 + 8 row
    dual.apply(ps.QuantumBinarySearch_Fast(q, "out", 8, "tgt", "res"))
    dual.compare(exact_amp=True)
    dual.apply(ps.QuantumBinarySearch_Fast(q, "out", 8, "tgt", "res").conditioned_by_nonzeros("x"))
    dual.compare(exact_amp=True)
    r, _ = dual.gpu.download()
    ids = {name: ps.System.resolve(name) for name in ("tgt", "res", "x")}
    sel = r[:, ids["x"]] == 0  # searched once: res holds the hit's address, 0 on a miss
    res, tgt = r[sel, ids["res"]].astype(np.int64), r[sel, ids["tgt"]]
    assert np.all(table[res[res > 0]] == tgt[res > 0])
    assert (res > 0).any() and (res == 0).any()


def test_multiword_keys(dual):
    # 3 words of packed keys; ops touching registers in different words
    for i, w in enumerate([40, 40, 40, 30, 20]):
        dual.reg(f"r{i}", U, w)
    assert ps.System.key_words() == 4  # first fit: 40 | 40 | 40 | 30, the 20-bit register joins word 0
    rng = np.random.default_rng(3)
    regs, amps = random_state(rng, [40, 40, 40, 30, 20], 3000)
    dual.start(regs, amps)
    for op in [ps.Add_UInt_UInt("r0", "r1", "r2"), ps.Mul_UInt_UInt("r3", "r4", "r1"),
               ps.Swap_General_General("r0", "r2"), ps.Phase_Bool("r2", 7, 1.1).conditioned_by_nonzeros("r4")]:
        dual.apply(op)
        dual.compare(exact_amp=True)


# ----------------------------------------------------------------- split / merge
@pytest.mark.parametrize("n_digits", [1, 2, 3, 5, 8, 10, 12])
@pytest.mark.parametrize("fill", ["singleton", "full", "mixed", "collide"])
def test_hadamard_int(dual, strategy, n_digits, fill):
    """'collide': mostly singleton groups with every tenth holding two or
    three members (the fan-out kernel lists those for the warp-per-group
    kernel, targets up to 8 bits)."""
    dual.reg("x", U, 14)
    dual.reg("y", U, 9)
    dual.reg("z", U, 6)
    rng = np.random.default_rng(n_digits * 7 + len(fill))
    S = 1 << n_digits
    groups = max(1, min(200, 6000 // S))
    if fill == "singleton":
        f = lambda g: 1  # noqa: E731
    elif fill == "full":
        f = lambda g: S  # noqa: E731
    elif fill == "collide":
        f = lambda g: min(S, 2 + g % 20 // 10) if g % 10 == 0 else 1  # noqa: E731
    else:
        f = lambda g: int(rng.integers(1, S + 1))  # noqa: E731
    regs, amps = grouped_state(rng, [9, 14, 6], 1, n_digits, groups, f)
    regs = regs[:, [1, 0, 2]]  # columns in register-id order x, y, z
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Int("x", n_digits))
    dual.compare(exact_amp=True)
    dual.apply(ps.Hadamard_Int("x", n_digits))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
@pytest.mark.parametrize("n", [4097, 7000, 8192])
@pytest.mark.parametrize("case", ["singletons", "one-pair", "one-failing"])
def test_hadamard_int_one_cta_grouping(dual, n, case, arith):
    """States of 4097 to 8192 entries (the most one CTA groups) with two key
    words, so that every thread of the one-CTA grouping has entries in both
    of its load batches: every group a singleton (written in entry order
    without the scan and bucket pass), one group of two members, and one
    entry failing the condition (both through the scan and bucket pass).
    Split on 2 bits and merged back, against the oracle."""
    ps.set_group_strategy("hash")
    ps.set_fwht_arithmetic(arith)
    dual.relaxed = arith == "exact-sum"
    try:
        dual.reg("x", U, 10)
        dual.reg("y", U, 50)
        dual.reg("z", U, 8)
        dual.reg("c", ps.Boolean, 1)
        assert ps.System.key_words() == 2
        rng = np.random.default_rng(n * 3 + len(case))
        y = rng.permutation(np.arange(n, dtype=np.uint64) * np.uint64(7919) + np.uint64(12345))  # distinct groups
        x = rng.integers(0, 1 << 10, n).astype(np.uint64)
        z = rng.integers(0, 1 << 8, n).astype(np.uint64)
        c = np.ones(n, dtype=np.uint64)
        if case == "one-pair":  # entry 1 joins entry 0's group with another target
            y[1], z[1], x[1] = y[0], z[0], x[0] ^ np.uint64(1)
        if case == "one-failing":
            c[n // 2] = 0
        regs = np.stack([x, y, z, c], axis=1)
        amps = rng.normal(size=n) + 1j * rng.normal(size=n)
        dual.start(regs, amps / np.linalg.norm(amps))
        op = ps.Hadamard_Int("x", 2).conditioned_by_nonzeros("c")
        dual.apply(op)
        dual.compare(exact_amp=True)
        dual.apply(op)
        dual.compare(exact_amp=True)
    finally:
        ps.set_group_strategy("autotune")


def test_hadamard_int_conditioned(dual, strategy):
    dual.reg("x", U, 6)
    dual.reg("y", U, 8)
    dual.reg("c", ps.Boolean, 1)
    rng = np.random.default_rng(11)
    regs, amps = random_state(rng, [6, 8, 1], 500)
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Int("x", 6).conditioned_by_nonzeros("c"))
    dual.compare(exact_amp=True)
    dual.apply(ps.Hadamard_Int("x", 6).conditioned_by_value("y", int(regs[0, 1])))
    dual.compare(exact_amp=True)
    # partial-width Hadamard on a state whose groups share the high bits of x
    regs2, amps2 = random_state(rng, [4, 8, 1], 400)
    dual.start(regs2, amps2)
    dual.apply(ps.Hadamard_Int("x", 4).conditioned_by_bit("y", 2))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("width", [1, 2, 4, 7, 10])
def test_hadamard_int_full(dual, strategy, width):
    dual.reg("q", U, width)
    dual.reg("r", U, 10)
    rng = np.random.default_rng(width)
    S = 1 << width
    regs, amps = grouped_state(rng, [width, 10], 0, width, 60, lambda g: int(rng.integers(1, S + 1)))
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Int_Full("q"))
    dual.compare(exact_amp=True)


def test_hadamard_bool(dual, strategy):
    dual.reg("q", ps.Boolean, 1)
    dual.reg("r", U, 12)
    dual.reg("c", U, 3)
    rng = np.random.default_rng(5)
    regs, amps = random_state(rng, [1, 12, 3], 3000)
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Bool("q"))
    dual.compare(exact_amp=True)
    dual.apply(ps.Hadamard_Bool("q").conditioned_by_bit("c", 1))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("kind", ["general", "diagonal", "offdiagonal", "rx", "ry"])
def test_rot_bool(dual, strategy, kind):
    dual.reg("q", U, 4)
    dual.reg("r", U, 10)
    rng = np.random.default_rng(len(kind))
    regs, amps = random_state(rng, [4, 10], 3000)
    dual.start(regs, amps)
    th = 0.7
    if kind == "general":
        op = ps.Rot_Bool("q", 2, [math.cos(th), -math.sin(th), math.sin(th), math.cos(th)])
    elif kind == "diagonal":
        op = ps.Rot_Bool("q", 1, [complex(math.cos(th), math.sin(th)), 0, 0, complex(math.cos(th), -math.sin(th))])
    elif kind == "offdiagonal":
        op = ps.Rot_Bool("q", 3, [0, 1j, 1j, 0])
    elif kind == "rx":
        op = ps.RX_Bool("q", 0, 1.3)
    else:
        op = ps.RY_Bool("q", 2, 2.1)
    dual.apply(op)
    dual.compare(exact_amp=True)
    dual.apply(op, dag=True)
    dual.compare(exact_amp=True)
    dual.apply(op.conditioned_by_value("r", int(regs[3, 1])))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("w_in", [1, 3, 8, 16])
def test_condrot(dual, strategy, w_in):
    dual.reg("in", ps.Rational, w_in)
    dual.reg("out", ps.Boolean, 1)
    dual.reg("r", U, 6)
    rng = np.random.default_rng(w_in)
    regs, amps = random_state(rng, [w_in, 1, 6], 2000)
    dual.start(regs, amps)
    op = ps.CondRot_Rational_Bool("in", "out")
    dual.apply(op)
    dual.compare(rel=1e-12)  # device sin/cos may differ from libm in the last ulp
    dual.apply(op, dag=True)
    dual.compare(rel=1e-12)


def test_clear_zero_and_normalize(dual):
    dual.reg("a", U, 20)
    rng = np.random.default_rng(9)
    regs, amps = random_state(rng, [20], 100000)
    amps[rng.random(amps.size) < 0.4] *= 1e-9  # |a|^2 ~ 1e-18 < eps
    dual.start(regs, amps)
    dual.apply(ps.ClearZero())
    dual.compare(exact_amp=True)
    dual.apply(ps.ClearZero(1e-6))
    dual.compare(exact_amp=True)
    dual.apply(ps.Normalize())
    dual.compare(rel=1e-13)
    assert abs(dual.gpu.norm_sq() - 1.0) < 1e-12


def test_add_systems(dual):
    dual.reg("a", U, 10)
    dual.reg("b", U, 10)
    rng = np.random.default_rng(13)
    r1, a1 = random_state(rng, [10, 10], 3000)
    r2, a2 = random_state(rng, [10, 10], 3000)
    r2[:1000] = r1[:1000]  # overlapping keys merge
    a2[:10] = -a1[:10] / 0.5  # exact cancellation with coef 0.5 -> pruned
    dual.start(r1, a1)
    g2 = ps.SparseState()
    g2.upload(r2, a2)
    o2 = dual.O.OracleState()
    o2.set(r2, a2)
    ps.add_systems(dual.gpu, g2, 0.5)
    dual.O.add_systems(dual.ora, o2, 0.5)
    dual.compare(exact_amp=True)


def test_register_surgery(dual):
    dual.reg("a", U, 12)
    dual.reg("b", U, 8)
    rng = np.random.default_rng(21)
    regs, amps = random_state(rng, [12, 8], 1000)
    dual.start(regs, amps)
    lo = dual.split("a", "lo", 5)
    dual.compare(exact_amp=True)
    dual.apply(ps.Add_UInt_UInt_InPlace("b", "lo"))
    dual.compare(exact_amp=True)
    dual.combine("a", "lo")
    dual.compare(exact_amp=True)
    t = dual.add_register("t", U, 16)
    dual.apply(ps.Mul_UInt_UInt("a", "b", "t"))
    dual.compare(exact_amp=True)
    dual.apply(ps.Mul_UInt_UInt("a", "b", "t"))  # uncompute
    dual.remove_register("t")
    dual.compare(exact_amp=True)
    # non-adjacent combine moves bits into a fresh field
    x = dual.add_register("x", U, 6)
    dual.apply(ps.Add_UInt_UInt("a", "b", "x"))
    dual.combine("b", "x")
    dual.compare(exact_amp=True)
    assert lo >= 0 and t >= 0


def test_many_varying_bits_multichunk_sort(dual, strategy):
    # > 64 varying group-key bits: the sort runs over several 64-bit chunks
    for i, w in enumerate([3, 60, 60, 20]):
        dual.reg(f"r{i}", U, w)
    rng = np.random.default_rng(17)
    regs, amps = grouped_state(rng, [3, 60, 60, 20], 0, 3, 400, lambda g: int(rng.integers(1, 9)))
    dual.start(regs, amps)
    dual.apply(ps.Hadamard_Int("r0", 3).conditioned_by_nonzeros("r3"))
    dual.compare(exact_amp=True)


def test_empty_state(dual):
    dual.reg("a", U, 8)
    dual.start(np.zeros((0, 1), dtype=np.uint64), np.zeros(0, dtype=np.complex128))
    for op in [ps.Hadamard_Int("a", 8), ps.Add_ConstUInt_InPlace("a", 3), ps.ClearZero(), ps.Hadamard_Bool]:
        if op is ps.Hadamard_Bool:
            continue
        dual.apply(op)
    assert dual.gpu.size() == 0 and dual.ora.size() == 0


def test_config1_small_circuit(dual, strategy):
    """The config-1 circuit shape at reduced widths: H(a), b ^= T[a], c ^= a*b,
    phase on c bit 0, H(a) — keys bit-exact, amplitudes bit-exact."""
    dual.reg("a", U, 8)
    dual.reg("b", U, 12)
    dual.reg("c", U, 12)
    rng = np.random.default_rng(20261203)
    table = rng.integers(0, 1 << 12, 1 << 8, dtype=np.uint64)
    q = dual.qram(8, 12, table)
    dual.start()
    for op in [ps.Hadamard_Int("a", 8), ps.QRAMLoad(q, "a", "b"), ps.Mul_UInt_UInt("a", "b", "c"),
               ps.Phase_Bool("c", 0, 0.37), ps.Hadamard_Int("a", 8)]:
        dual.apply(op)
        dual.compare(exact_amp=True)
    assert dual.gpu.size() > 1 << 14
    assert abs(dual.gpu.norm_sq() - 1.0) < 1e-12


def test_config1_full_size(dual, strategy):
    """Config 1 at its literal size: a 12-bit, b/c 16-bit, 4096-word uint16
    table; the final Hadamard fans out to ~2^24 entries. Keys bit-exact and
    amplitudes bit-exact against the oracle on the full state."""
    dual.reg("a", U, 12)
    dual.reg("b", U, 16)
    dual.reg("c", U, 16)
    rng = np.random.default_rng(20261203)
    table = rng.integers(0, 1 << 16, 4096, dtype=np.uint64)
    q = dual.qram(12, 16, table)
    dual.start()
    for op in [ps.Hadamard_Int("a", 12), ps.QRAMLoad(q, "a", "b"), ps.Mul_UInt_UInt("a", "b", "c"),
               ps.Phase_Bool("c", 0, 0.37), ps.Hadamard_Int("a", 12)]:
        dual.apply(op)
    assert dual.gpu.size() > 16_000_000
    dual.compare(exact_amp=True)
    assert abs(dual.gpu.norm_sq() - 1.0) < 1e-12
    # and back: 4096 full 4096-member groups merge (the 12-stage FWHT at scale)
    dual.apply(ps.Hadamard_Int("a", 12))
    assert dual.gpu.size() == 4096
    dual.compare(exact_amp=True)


def _random_unitary(rng, dim):
    z = rng.normal(size=(dim, dim)) + 1j * rng.normal(size=(dim, dim))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("width", [1, 2, 3, 5])
def test_rot_general_unitary(dual, strategy, width):
    dual.reg("q", U, width)
    dual.reg("r", U, 9)
    rng = np.random.default_rng(100 + width)
    S = 1 << width
    regs, amps = grouped_state(rng, [width, 9], 0, width, 80, lambda g: int(rng.integers(1, S + 1)))
    dual.start(regs, amps)
    op = ps.Rot_GeneralUnitary("q", _random_unitary(rng, S))
    dual.apply(op)
    dual.compare(exact_amp=True)
    dual.apply(op, dag=True)
    dual.compare(exact_amp=True)
    dual.apply(op.conditioned_by_bit("r", 3))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("w_in", [1, 4, 10])
def test_condrot_general_bool(dual, strategy, w_in):
    dual.reg("in", U, w_in)
    dual.reg("out", ps.Boolean, 1)
    dual.reg("r", U, 7)
    rng = np.random.default_rng(200 + w_in)
    regs, amps = random_state(rng, [w_in, 1, 7], 3000)
    dual.start(regs, amps)
    mats = [_random_unitary(rng, 2) for _ in range(1 << w_in)]
    op = ps.CondRot_General_Bool("in", "out", lambda v: mats[v].reshape(-1))
    dual.apply(op)
    dual.compare(exact_amp=True)
    # conditioned: entries failing the condition stay as they are (a pair with
    # one member on each side is two unpaired members of the rotated part)
    dual.apply(op.conditioned_by_bit("r", 2))
    dual.compare(exact_amp=True)
    dual.apply(ps.CondRot_General_Bool.from_table("in", "out", [m.reshape(-1) for m in mats[:3]])
               .conditioned_by_value("r", 5).conditioned_by_nonzeros("in"))
    dual.compare(exact_amp=True)


def test_hadamard_partial(dual, strategy):
    dual.reg("q", U, 6)
    dual.reg("r", U, 10)
    rng = np.random.default_rng(300)
    regs, amps = random_state(rng, [6, 10], 3000)
    dual.start(regs, amps)
    for pos in (0, 3, 5):
        dual.apply(ps.Hadamard_Partial("q", [pos]))
        dual.compare(exact_amp=True)
    # conditioned: entries failing the condition stay as they are
    dual.apply(ps.Hadamard_Partial("q", [2]).conditioned_by_bit("r", 4))
    dual.compare(exact_amp=True)
    dual.apply(ps.Hadamard_Partial("q", [1]).conditioned_by_nonzeros("r"))
    dual.compare(exact_amp=True)


@pytest.mark.parametrize("positions", [[0, 3], [1, 2, 5], [0, 1, 2], [4, 5], [0, 2, 3, 5], list(range(6)),
                                       [2, 2, 4]])
def test_hadamard_partial_several_positions(dual, strategy, positions):
    """H on a set of bits: singletons fan out, full groups run the FWHT in
    place, partial groups are completed (Hadamard_Partial::operate's three
    cases); applied twice it merges back to the input. Conditions on another
    register and on a bit of the target outside the set."""
    dual.reg("q", U, 6)
    dual.reg("r", U, 10)
    rng = np.random.default_rng(310 + len(positions))
    regs, amps = random_state(rng, [6, 10], 3000)
    dual.start(regs, amps)
    op = ps.Hadamard_Partial("q", positions)
    dual.apply(op)
    dual.compare(exact_amp=True)
    dual.apply(op)
    dual.compare(exact_amp=True)
    assert dual.gpu.size() == 3000  # H.H = I
    dual.apply(ps.Hadamard_Partial("q", positions).conditioned_by_bit("r", 3))
    dual.compare(exact_amp=True)
    rest = [b for b in range(6) if b not in positions]
    if rest:
        dual.apply(ps.Hadamard_Partial("q", positions).conditioned_by_bit("q", rest[-1]))
        dual.compare(exact_amp=True)


def test_bit_gather_round_trip(dual):
    """The bit permutation behind several-position Hadamard_Partial, against
    the oracle, and its inverse."""
    dual.reg("q", U, 13)
    dual.reg("r", U, 7)
    rng = np.random.default_rng(320)
    regs, amps = random_state(rng, [13, 7], 2000)
    dual.start(regs, amps)
    for mask in (0b1000100100001, 0b0000000000111, 0b1111111111111, 0b1010101010101):
        g = ps.BitGather("q", mask)
        dual.apply(g)
        dual.compare(exact_amp=True)
        dual.apply(g, dag=True)
        dual.compare(exact_amp=True)
        assert np.array_equal(np.sort(dual.gpu.download()[0][:, 0]), np.sort(regs[:, 0]))
