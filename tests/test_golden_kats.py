"""Known-answer tests from the reference's own unit tests
(tests/golden/reference_kats.json, written by make_reference_kats.py).

The CPU oracle must reproduce every case (this pins the restatement); the GPU
engine must reproduce them too (marked gpu). Elementwise tables are run as one
multi-entry state (entries do not interact), others case by case."""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np
import pytest

import sparqsim_gb300 as ps
from oracle import oracle as O

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
ELEMENTWISE = {"Add_UInt_UInt", "Add_UInt_UInt_InPlace", "Add_UInt_ConstUInt", "Add_ConstUInt_InPlace",
               "Mult_UInt_ConstUInt", "Add_Mult_UInt_ConstUInt_InPlace", "FlipBools", "Assign", "Compare_UInt_UInt",
               "Add_AnyInt_AnyInt_InPlace", "GetMid_UInt_UInt", "ShiftLeft_InPlace", "ShiftRight_InPlace",
               "Mod_Mult_UInt_ConstUInt_InPlace", "Sub_UInt_UInt", "Neg_UInt", "Abs_SInt", "Mul_UInt_UInt",
               "Div_UInt_UInt", "Sqrt_UInt", "Select_Bool_UInt_UInt", "And_UInt_UInt", "Or_UInt_UInt",
               "Xor_UInt_UInt", "Less_SInt_SInt", "Carry_UInt_UInt", "Overflow_SInt_SInt", "MulOverflow_UInt_UInt",
               "IsZero_UInt", "Negative_SInt", "X_Bool", "Y_Bool", "Z_Bool", "S_Bool", "T_Bool", "Phase_Bool",
               "QRAMLoad", "GlobalPhase"}


class _HostTable:
    """Stand-in for a QRAM table when only the oracle runs (no GPU)."""

    _next = 1

    def __init__(self, addr_size, data_size, memory):
        self.address_size, self.data_size = addr_size, data_size
        self.memory = np.asarray(memory, dtype=np.uint64)

        class _H:
            pass

        self._h = _H()
        self._h.value = 0x7F000000 + _HostTable._next
        _HostTable._next += 1


def _declare(regs):
    ids = {}
    for name, t, w in regs:
        ty = getattr(ps.StateStorageType, t)
        rid = ps.System.add_register(name, ty, w)
        assert O.add_register(int(ty), w) == rid
        ids[name] = rid
    return ids


def _make_ops(ops, backend):
    out = []
    for spec in ops:
        name, *args = spec
        dag = name.endswith(".dag")
        name = name.replace(".dag", "")
        cond = None
        if "@" in name:
            name, c = name.split("@")
            kind, reg = c.split(":")
            cond = (kind, reg)
        if name == "QRAMLoad":
            a, d, mem = args[0]
            q = ps.QRAMCircuit_qutrit(a, d, mem) if backend == "gpu" else _HostTable(a, d, mem)
            O.register_qram(q)
            op = ps.QRAMLoad(q, *args[1:])
            op._keep = q
        elif name == "Rot_Bool":
            op = ps.Rot_Bool(args[0], args[1], [complex(*m) for m in args[2]])
        elif name == "GlobalPhase":
            op = ps.GlobalPhase(complex(*args[0]))
        else:
            op = getattr(ps, name)(*args)
        if cond:
            getattr(op, "conditioned_by_" + cond[0])(cond[1])
        out.append((op, dag))
    return out


def _run(backend, ops, regs_init, amps):
    if backend == "gpu":
        st = ps.SparseState()
        st.upload(regs_init, amps)
        for op, dag in ops:
            op.dag(st) if dag else op(st)
        return st.download()
    st = O.OracleState()
    st.set(regs_init, amps)
    for op, dag in ops:
        O.apply(st, op.spec(dag and not op.self_adjoint))
    return st.get()


def _check_table(t, backend):
    ids = _declare(t["regs"])
    ops = _make_ops(t["ops"], backend)
    nreg = len(ids)
    ni = len(t["init_names"])
    rows = t["rows"]
    batch = all(o[0].split(".")[0].split("@")[0] in ELEMENTWISE for o in t["ops"])
    groups = [rows] if batch else [[r] for r in rows]
    for grp in groups:
        init = np.zeros((len(grp), nreg), dtype=np.uint64)
        for i, r in enumerate(grp):
            for k, name in enumerate(t["init_names"]):
                init[i, ids[name]] = r[k]
        amps = np.ones(len(grp), dtype=np.complex128)
        regs, out = _run(backend, ops, init, amps)
        for i, r in enumerate(grp):
            exp = dict(zip(t["expect_names"], r[ni:]))
            if "@size" in exp:
                assert regs.shape[0] == exp["@size"], t["src"]
            for name, v in exp.items():
                if name == "@amp":
                    assert abs(out[i] - complex(*v)) < 1e-9, (t["src"], r, out[i])
                elif name != "@size":
                    assert int(regs[i, ids[name]]) == v, (t["src"], name, r, int(regs[i, ids[name]]))


def _check_multi(m, backend):
    ids = _declare(m["regs"])
    ops = _make_ops(m["ops"], backend)
    nreg = len(ids)
    init = np.zeros((len(m["init"]), nreg), dtype=np.uint64)
    for i, d in enumerate(m["init"]):
        for name, v in d.items():
            init[i, ids[name]] = v
    regs, out = _run(backend, ops, init, np.ones(len(m["init"]), dtype=np.complex128))
    got = {tuple(int(x) for x in r): a for r, a in zip(regs, out)}
    assert len(got) == len(m["expect"]), (m["src"], len(got), len(m["expect"]))
    for vals, (re, im) in m["expect"]:
        a = got[tuple(vals)]
        assert abs(a - complex(re, im)) < 1e-12, (m["src"], vals, a, (re, im))


TABLE_IDS = [f"{i}:{t['src'].split('/')[-1]}" for i, t in enumerate(KATS["tables"])]


@pytest.mark.parametrize("t", KATS["tables"], ids=TABLE_IDS)
def test_oracle_reference_kats(t):
    _check_table(t, "oracle")


@pytest.mark.parametrize("m", KATS["multi"], ids=[m["src"].split("/")[-1] for m in KATS["multi"]])
def test_oracle_reference_multi(m):
    _check_multi(m, "oracle")


@pytest.mark.gpu
@pytest.mark.parametrize("t", KATS["tables"], ids=TABLE_IDS)
def test_gpu_reference_kats(t):
    _check_table(t, "gpu")


@pytest.mark.gpu
@pytest.mark.parametrize("m", KATS["multi"], ids=[m["src"].split("/")[-1] for m in KATS["multi"]])
def test_gpu_reference_multi(m):
    _check_multi(m, "gpu")


def test_kat_fixture_is_current():
    """The committed fixture matches what its generator writes."""
    import subprocess
    import sys
    gen = Path(__file__).parent / "golden" / "make_reference_kats.py"
    before = (Path(__file__).parent / "golden" / "reference_kats.json").read_bytes()
    subprocess.run([sys.executable, str(gen)], check=True, capture_output=True)
    after = (Path(__file__).parent / "golden" / "reference_kats.json").read_bytes()
    assert before == after
    assert not math.isnan(0.0)
