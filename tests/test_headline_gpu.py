"""The register circuit at scale, exactly as bench.py times it (a 20-bit, b/c/t
32-bit: K = 2 packed key words; a 2^20-word uint32 table; Hadamard on 12 bits;
2^24 entries at the peak), against the oracle for its first two layers. Layer
1 runs the singleton fan-out (1 -> 4096 -> 2^24 entries), layer 2 the merge of
4096 full cached ranges (2^24 -> 4096) and the fan-out again, so both narrowed
12-bit kernels (H_SINGLE, H_FULL) and the fused elementwise program are
covered at full size. Keys bit-exact; amplitudes within 1e-12 of the largest
in the exact-sum arithmetic (the default), bit-exact in the reference one."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300.workloads import RegisterCircuit

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rows(regs, amps):
    k0 = (regs[:, 0] << np.uint64(32)) | regs[:, 1]
    k1 = (regs[:, 2] << np.uint64(32)) | regs[:, 3]
    order = np.lexsort((k1, k0))
    return k0[order], k1[order], amps[order]


@pytest.fixture(scope="module")
def oracle_two_layers():
    from oracle import oracle as O
    circ = RegisterCircuit(12, 10).build()
    O.clear()
    for rid in ps.System.active_ids():
        O.add_register(int(ps.System.type_of(rid)), ps.System.size_of(rid))
    O.register_qram(circ.qram)
    ost = O.OracleState()
    for op in circ.ops(2):
        O.apply(ost, op.spec())
    out = _rows(*ost.get())
    O.clear()
    return out


@pytest.mark.parametrize("arith", ["exact-sum", "reference"])
def test_register_circuit_two_layers_full_size(oracle_two_layers, arith):
    ok0, ok1, oa = oracle_two_layers
    assert len(oa) > 16_000_000
    ps.set_fwht_arithmetic(arith)
    circ = RegisterCircuit(12, 10).build()
    assert ps.System.key_words() == 2
    st = ps.SparseState(capacity=1 << 24)
    circ.run(st, layers=2)
    gk0, gk1, ga = _rows(*st.download())
    assert len(ga) == len(oa)
    assert np.array_equal(gk0, ok0) and np.array_equal(gk1, ok1)
    err = float(np.max(np.abs(ga - oa))) / float(np.max(np.abs(oa)))
    if arith == "reference":
        assert np.array_equal(ga.view(np.float64), oa.view(np.float64)), err
    assert err <= TOL, err
    print(f"register circuit, 2 layers, {arith}: {len(ga)} entries, max rel amp err {err:.3e}")
