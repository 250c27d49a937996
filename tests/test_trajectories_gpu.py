"""Batched noisy trajectories: the batched form (all instances in one state,
one batched Hadamard and one fused launch per step) against the plain form
(one state per instance) and against the CPU oracle. Keys and amplitudes are
bit-identical between the two GPU forms; against the oracle, keys bit-exact
and amplitudes bit-exact in the reference arithmetic, 1e-12 in exact-sum."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300.workloads import NoisyTrajectories

pytestmark = pytest.mark.gpu


def _by_traj(regs, amps):
    out = {}
    for r, a in zip(regs, amps):
        out.setdefault(int(r[0]), []).append((tuple(int(v) for v in r[-3:]), a))
    return {t: sorted(v, key=lambda e: e[0]) for t, v in out.items()}


@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
def test_batched_equals_plain(arith):
    ps.set_fwht_arithmetic(arith)
    wl = NoisyTrajectories(n_traj=48, layers=3, p=0.05, h_min=1, h_max=6, seed=11)
    wl.build_batched()
    st = ps.SparseState()
    upd_b = wl.run_batched(st, count=True)
    batched = _by_traj(*st.download())
    wl.build_plain()
    upd_p = 0
    for t in range(wl.n_traj):
        sp = ps.SparseState()
        upd_p += wl.run_plain(sp, t, count=True)
        plain = _by_traj(*sp.download()).get(t, [])
        got = batched.get(t, [])
        assert [k for k, _ in got] == [k for k, _ in plain], f"instance {t}: keys differ"
        ga = np.array([a for _, a in got])
        pa = np.array([a for _, a in plain])
        assert np.array_equal(ga.view(np.float64), pa.view(np.float64)), f"instance {t}: amplitudes differ"
    assert upd_b == upd_p


def test_batched_against_oracle(dual):
    wl = NoisyTrajectories(n_traj=24, layers=2, p=0.05, h_min=1, h_max=5, seed=12)
    wl.build_batched()
    from oracle import oracle as O
    O.clear()
    for rid in ps.System.active_ids():
        O.add_register(int(ps.System.type_of(rid)), ps.System.size_of(rid))
    kind, qram, noise, mids, H = wl._built
    O.register_qram(qram)
    for nt in noise:
        O.register_qram(nt.table)
    dual.start(*wl.initial_batched())
    for mid in mids:
        dual.apply(H)
        dual.compare(exact_amp=True)
        dual.apply(mid)
        dual.compare(exact_amp=True)
        dual.apply(H)
        dual.compare(exact_amp=True)
    assert dual.gpu.size() > wl.n_traj
