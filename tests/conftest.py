"""Shared fixtures: builds the engine and the oracle, resets both register
tables before each test (the reference's fresh_system fixture,
PySparQ/test/conftest.py:26-36), and a Dual runner that applies the same
operators to a GPU state and to the oracle."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


@pytest.fixture(autouse=True)
def fresh_system():
    """Fresh register tables; Hadamard butterflies in the reference's FP64
    order (bit-identical results) unless a test selects exact-sum."""
    import sparqsim_gb300 as ps
    from oracle import oracle as O
    ps.System.clear()
    O.clear()
    ps.set_fwht_arithmetic("reference")
    ps.set_group_strategy("autotune")
    ps.autotune_reset()
    yield
    ps.System.clear()
    O.clear()
    ps.set_fwht_arithmetic("reference")


# amplitude errors against the FP64 oracle, per FWHT arithmetic, reported at the end
AMP_ERRORS: dict = {}


def pytest_terminal_summary(terminalreporter):
    if AMP_ERRORS:
        terminalreporter.write_line("amplitude error vs the FP64 oracle (max |a_gpu - a_oracle| / max|a|):")
        for mode, errs in sorted(AMP_ERRORS.items()):
            terminalreporter.write_line(f"  {mode}: {len(errs)} comparisons, max {max(errs):.3e}")


class Dual:
    """Declares registers in both tables and applies operators to a GPU state
    and an oracle state side by side."""

    def __init__(self):
        import sparqsim_gb300 as ps
        from oracle import oracle as O
        self.ps, self.O = ps, O
        self.gpu = None
        self.ora = None
        self.relaxed = False  # exact-sum FWHT: amplitudes within tolerance instead of bit-exact

    def reg(self, name, type_, width):
        rid = self.ps.System.add_register(name, type_, width)
        oid = self.O.add_register(int(type_), width)
        assert rid == oid
        return rid

    def start(self, regs=None, amps=None):
        self.gpu = self.ps.SparseState()
        self.ora = self.O.OracleState()
        if regs is not None:
            self.gpu.upload(regs, amps)
            self.ora.set(regs, amps)
        return self

    def qram(self, addr_size, data_size, memory):
        q = self.ps.QRAMCircuit_qutrit(addr_size, data_size, memory)
        self.O.register_qram(q)
        return q

    def apply(self, op, dag=False):
        if dag:
            op.dag(self.gpu)
        else:
            op(self.gpu)
        self.O.apply(self.ora, op.spec(dag and not op.self_adjoint))

    def add_register(self, name, type_, width):
        rid = self.ps.AddRegister(name, type_, width)(self.gpu)
        oid = self.O.add_register_sync(self.ora, int(type_), width)
        assert rid == oid
        return rid

    def remove_register(self, name):
        rid = self.ps.System.resolve(name)
        self.ps.RemoveRegister(rid)(self.gpu)
        self.O.remove_register_sync(self.ora, rid)

    def split(self, first, second_name, second_size):
        f = self.ps.System.resolve(first)
        rid = self.ps.SplitRegister(f, second_name, second_size)(self.gpu)
        oid = self.O.split_register(self.ora, f, second_size)
        assert rid == oid
        return rid

    def combine(self, first, second):
        f, s = self.ps.System.resolve(first), self.ps.System.resolve(second)
        self.ps.CombineRegister(f, s)(self.gpu)
        self.O.combine_register(self.ora, f, s)

    def compare(self, rel=1e-12, exact_amp=False):
        """Keys bit-exact; amplitudes within rel * max|a| (or bit-exact).
        Returns the max relative amplitude error."""
        ids = self.ps.System.active_ids()
        assert ids == self.O.active_ids()
        gk, ga = self.O.canonical(*self.gpu.download(), ids)
        ok, oa = self.O.canonical(*self.ora.get(), ids)
        assert gk.shape == ok.shape, f"entry count {gk.shape[0]} != oracle {ok.shape[0]}"
        if not np.array_equal(gk, ok):
            bad = np.nonzero((gk != ok).any(axis=1))[0][:5]
            raise AssertionError(f"keys differ at rows {bad}: gpu {gk[bad]} oracle {ok[bad]}")
        scale = max(float(np.max(np.abs(oa))) if oa.size else 0.0, 1e-300)
        err = float(np.max(np.abs(ga - oa))) / scale if oa.size else 0.0
        mode = self.ps.get_fwht_arithmetic()
        AMP_ERRORS.setdefault(mode, []).append(err)
        if exact_amp and not self.relaxed:
            assert np.array_equal(ga.view(np.float64), oa.view(np.float64)), f"amplitudes not bit-exact (rel {err})"
        assert err <= rel, f"amplitude rel error {err} > {rel}"
        return err


@pytest.fixture
def dual():
    return Dual()
