"""Operator sequences replayed as CUDA graphs (sq_graph_*): a replay gives
the eager run's state bit for bit (batched noisy trajectories and the
register circuit), replays repeat, and a replay on another input, on a
changed table or on a state of another size is refused before it runs."""
from __future__ import annotations

import numpy as np
import pytest

import sparqsim_gb300 as ps
from sparqsim_gb300.workloads import NoisyTrajectories

pytestmark = pytest.mark.gpu


def _canon(st):
    regs, amps = st.download()
    ids = ps.System.active_ids()
    keys = regs[:, ids]
    order = np.lexsort(keys.T[::-1])
    return keys[order], amps[order]


@pytest.mark.parametrize("arith", ["reference", "exact-sum"])
def test_batched_trajectories_graph_replay_is_bit_identical(arith):
    ps.set_fwht_arithmetic(arith)
    w = NoisyTrajectories(n_traj=64, layers=3, seed=7).build_batched()
    st = ps.SparseState()
    w.run_batched(st)
    want_k, want_a = _canon(st)
    g = ps.Graph(st, apply=lambda: w.run_batched(st, upload=False), prepare=lambda: st.upload(*w.initial_batched()))
    for _ in range(3):
        g.replay()
        ps.synchronize()
        got_k, got_a = _canon(st)
        assert np.array_equal(got_k, want_k)
        assert np.array_equal(got_a.view(np.float64), want_a.view(np.float64))
    # an eager operator after a replay sees the replayed state
    ps.Hadamard_Int_Batched("a", "w", w.h_max)(st)
    assert st.size() > 0


def test_register_circuit_graph_replay_and_launch_count():
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 12)
    b = ps.System.add_register("b", ps.UnsignedInteger, 16)
    c = ps.System.add_register("c", ps.UnsignedInteger, 16)
    rng = np.random.default_rng(20261203)
    q = ps.QRAMCircuit_qutrit(12, 16, rng.integers(0, 1 << 16, 4096, dtype=np.uint64))
    ops = [ps.Hadamard_Int(a, 12), ps.QRAMLoad(q, a, b), ps.Mul_UInt_UInt(a, b, c), ps.Phase_Bool(c, 0, 0.37),
           ps.Hadamard_Int(a, 12)]

    def apply():
        for o in ops:
            o(st)

    def prepare():
        st.upload(np.zeros((1, 3), dtype=np.uint64), np.ones(1, dtype=np.complex128))

    st = ps.SparseState()
    prepare()
    apply()
    want_k, want_a = _canon(st)
    g = ps.Graph(st, apply, prepare)
    n0 = ps.launch_count()
    g.replay()
    ps.synchronize()
    assert ps.launch_count() > n0  # the graph's kernels are counted per replay
    got_k, got_a = _canon(st)
    assert np.array_equal(got_k, want_k) and np.array_equal(got_a, want_a)


def test_replay_on_other_input_is_refused():
    """Recorded on four entries that form one Hadamard group; a replay on four
    entries that form four groups (same size, other data) is refused before
    anything runs, as is a launch on a state of another size. (Two Hadamards:
    a graph needs an even number of splits; one is refused.)"""
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 2)
    b = ps.System.add_register("b", ps.UnsignedInteger, 4)
    st = ps.SparseState()
    one_group = np.array([[0, 5], [1, 5], [2, 5], [3, 5]], dtype=np.uint64)
    four_groups = np.array([[0, 1], [0, 2], [0, 3], [0, 4]], dtype=np.uint64)
    amps = np.full(4, 0.5, dtype=np.complex128)
    inp = {"regs": one_group}
    with pytest.raises(ps.SparQInvalid):
        ps.Graph(st, apply=lambda: ps.Hadamard_Int(a, 2)(st), prepare=lambda: st.upload(inp["regs"], amps))

    def two():
        ps.Hadamard_Int(a, 2)(st)
        ps.Hadamard_Int(a, 2)(st)

    g = ps.Graph(st, apply=two, prepare=lambda: st.upload(inp["regs"], amps))
    inp["regs"] = four_groups
    with pytest.raises(ps.SparQInvalid):
        g.replay()
    inp["regs"] = one_group
    g.replay()  # the recorded input again: allowed
    ps.synchronize()
    assert st.size() == 4
    st.upload(np.zeros((3, 2), dtype=np.uint64) + np.arange(3, dtype=np.uint64)[:, None], np.ones(3) / np.sqrt(3))
    with pytest.raises(ps.SparQInvalid):
        g.launch()


def test_qram_write_in_place_and_replay_guard():
    """A captured graph reads the QRAM table where it is and only runs on the
    table content it was recorded with: after new words are written the
    replay is refused; writing the recorded words back (in place) makes it
    valid again, equal to an eager run; a word wider than the stored width is
    refused."""
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 6)
    b = ps.System.add_register("b", ps.UnsignedInteger, 16)
    rng = np.random.default_rng(3)
    t1 = rng.integers(0, 1 << 16, 64, dtype=np.uint64)
    t2 = rng.integers(0, 1 << 16, 64, dtype=np.uint64)
    q = ps.QRAMCircuit_qutrit(6, 16, t1)
    ops = [ps.Hadamard_Int(a, 6), ps.QRAMLoad(q, a, b), ps.Phase_Bool(b, 3, 0.5), ps.Hadamard_Int(a, 6)]
    st = ps.SparseState()

    def apply():
        for o in ops:
            o(st)

    g = ps.Graph(st, apply, st.reset)
    st.reset()
    apply()
    want_k, want_a = _canon(st)
    q.write(t2)
    with pytest.raises(ps.SparQInvalid):
        g.replay()
    q.write(t1)
    g.replay()
    ps.synchronize()
    got_k, got_a = _canon(st)
    assert np.array_equal(got_k, want_k) and np.array_equal(got_a, want_a)
    with pytest.raises(ps.SparQInvalid):
        q.write(np.full(64, 1 << 20, dtype=np.uint64))
    # the refused write left the table as it was: the replay gate still accepts it
    g.replay()
    ps.synchronize()
    got_k, got_a = _canon(st)
    assert np.array_equal(got_k, want_k) and np.array_equal(got_a, want_a)


def _small_graph():
    ps.System.clear()
    a = ps.System.add_register("a", ps.UnsignedInteger, 4)
    b = ps.System.add_register("b", ps.UnsignedInteger, 8)
    q = ps.QRAMCircuit_qutrit(4, 8, np.arange(16, dtype=np.uint64) * 7 % 251)
    st = ps.SparseState()

    def apply():
        ps.Hadamard_Int(a, 4)(st)
        ps.QRAMLoad(q, a, b)(st)
        ps.Hadamard_Int(a, 4)(st)

    return st, q, ps.Graph(st, apply, st.reset)


def test_launch_after_table_destroyed_is_refused_on_the_host():
    """Destroying a table a graph reads makes every later launch refuse
    before any device work (no checksum kernel reads the freed table)."""
    from sparqsim_gb300 import _native
    st, q, g = _small_graph()
    g.replay()
    ps.synchronize()
    _native.call("sq_qram_destroy", q._h)
    q._h = None
    st.reset()
    n0 = ps.launch_count()
    with pytest.raises(ps.SparQInvalid, match="destroyed"):
        g.launch()
    assert ps.launch_count() == n0  # nothing was launched


def test_launch_after_state_destroyed_is_refused_on_the_host():
    from sparqsim_gb300 import _native
    st, q, g = _small_graph()
    g.replay()
    ps.synchronize()
    _native.call("sq_state_destroy", st._h)
    st._h = None
    n0 = ps.launch_count()
    with pytest.raises(ps.SparQInvalid, match="destroyed"):
        g.launch()
    assert ps.launch_count() == n0
