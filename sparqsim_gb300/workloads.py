"""Seeded synthetic workloads built on the operator API.

RegisterCircuit: the register circuit at scale (a 20-bit, b 32-bit, c 32-bit
plus a 32-bit scratch t). From |0>, each of L layers is

    Hadamard_Int(a, h)                    # split: 1 -> 2^h, or merge 2^2h -> 2^h
    b ^= QRAM[a]                          # 2^20-word table of seeded uint32
    t ^= a*b; c += t; t ^= a*b            # c += a*b mod 2^32
    phase exp(i theta_l) on bit 0 of c    # theta_l seeded uniform in [0, 2 pi)
    Hadamard_Int(a, h)                    # split: fan-out to the 2^2h peak

with the five elementwise operators of a layer fused into one launch.

NoisyTrajectories: n instances of the register circuit (registers a, b, c of
16 bits) with independent Pauli X/Z noise, each instance with its own Hadamard
width h_t, so that the support of instance t alternates between 2^h_t and
2^(2 h_t) entries. Layer l of one instance is

    Hadamard_Int(a, h_t)                  # 2^(2h) -> 2^h (merge) or 1 -> 2^h
    b ^= QRAM[a]                          # 2^16-word table of seeded uint16
    c ^= a * b mod 2^16                   # Mul_UInt_UInt(a, b, c)
    phase exp(i theta_l) on bit 0 of c
    Pauli X then Z masks on a, b, c       # each bit with probability p
    Hadamard_Int(a, h_t)                  # 2^h -> 2^(2h) (split)

The batched form holds every instance in one state, with a register `t`
(instance id) and a register `w` (its width h_t), and runs each layer as one
Hadamard_Int_Batched, one fused elementwise launch and one more
Hadamard_Int_Batched. The plain form runs instance by instance, each in its
own state, with the same operators. Instance t of the batched result is
bit-identical to the plain run of instance t: no operator mixes instances.
"""
from __future__ import annotations

import math

import numpy as np

from . import core
from .core import QRAMCircuit_qutrit, SparseState, System
from .operators import Fused, Hadamard_Int, Hadamard_Int_Batched, Mul_UInt_UInt, NoiseTable, PauliNoise, Phase_Bool, \
    QRAMLoad

REG_BITS = 16


class RegisterCircuit:
    A_BITS, B_BITS, C_BITS, T_BITS = 20, 32, 32, 32
    TABLE_BITS = 20
    SEED = 20261203

    def __init__(self, h: int = 12, layers: int = 10, seed: int = SEED):
        self.h, self.layers = int(h), int(layers)
        rng = np.random.default_rng(seed)
        self.table = rng.integers(0, 1 << 32, 1 << self.TABLE_BITS, dtype=np.uint64)
        self.thetas = rng.uniform(0.0, 2 * math.pi, self.layers)
        self.qram = None

    def build(self):
        """Declares a, b, c, t (ids 0..3, the register table cleared first) and
        the operators."""
        System.clear()
        for name, w in (("a", self.A_BITS), ("b", self.B_BITS), ("c", self.C_BITS), ("t", self.T_BITS)):
            System.add_register(name, core.UnsignedInteger, w)
        self.qram = QRAMCircuit_qutrit(self.TABLE_BITS, 32, self.table)
        self.H = Hadamard_Int("a", self.h)
        self.mid = [self.mid_ops(self.qram, th) for th in self.thetas]
        return self

    @staticmethod
    def mid_ops(qram, theta: float):
        from .operators import Add_UInt_UInt_InPlace
        return Fused([QRAMLoad(qram, "a", "b"), Mul_UInt_UInt("a", "b", "t"), Add_UInt_UInt_InPlace("t", "c"),
                      Mul_UInt_UInt("a", "b", "t"), Phase_Bool("c", 0, float(theta))])

    def ops(self, layers: int | None = None):
        """The operator sequence of the first `layers` layers."""
        out = []
        for layer in range(self.layers if layers is None else layers):
            out += [self.H, self.mid[layer], self.H]
        return out

    def run(self, st: SparseState, count: bool = False, reset: bool = True, layers: int | None = None) -> int:
        """One step from |0> (`reset`); returns the update count when count=True."""
        if reset:
            st.reset()
        upd = 0
        for layer in range(self.layers if layers is None else layers):
            n0 = st.size() if count else 0
            self.H(st)
            n1 = st.size() if count else 0
            self.mid[layer](st)
            self.H(st)
            if count:
                n2 = st.size()
                upd += max(n0, n1) + 5 * n1 + max(n1, n2)
        return upd


class NoisyTrajectories:
    def __init__(self, n_traj: int = 4096, layers: int = 6, p: float = 1e-3, h_min: int = 4, h_max: int = 8,
                 seed: int = 20261203):
        if not 1 <= h_min <= h_max <= 8:
            raise ValueError("Hadamard widths must lie in 1..8")
        self.n_traj, self.layers, self.p = int(n_traj), int(layers), float(p)
        self.t_bits = max(1, math.ceil(math.log2(max(self.n_traj, 2))))
        self.h_max = int(h_max)
        rng = np.random.default_rng(seed)
        self.widths = rng.integers(h_min, h_max + 1, self.n_traj).astype(np.uint64)
        self.table = rng.integers(0, 1 << REG_BITS, 1 << REG_BITS, dtype=np.uint64)
        self.thetas = rng.uniform(0.0, 2 * math.pi, self.layers)
        self.masks = []
        for _ in range(self.layers):
            m = np.zeros((self.n_traj, 6), dtype=np.uint64)
            for j in range(6):
                bits = rng.random((self.n_traj, REG_BITS)) < self.p
                m[:, j] = (bits.astype(np.uint64) << np.arange(REG_BITS, dtype=np.uint64)).sum(axis=1)
            self.masks.append(m)
        self._built = None

    # ------------------------------------------------------------- registers
    def declare(self, batched: bool) -> None:
        System.clear()
        System.add_register("t", core.UnsignedInteger, self.t_bits)
        if batched:
            System.add_register("w", core.UnsignedInteger, 4)
        for name in ("a", "b", "c"):
            System.add_register(name, core.UnsignedInteger, REG_BITS)

    def _layer_ops(self):
        qram = QRAMCircuit_qutrit(REG_BITS, REG_BITS, self.table)
        noise = [NoiseTable(m) for m in self.masks]
        mids = [Fused([QRAMLoad(qram, "a", "b"), Mul_UInt_UInt("a", "b", "c"), Phase_Bool("c", 0, float(th)),
                       PauliNoise("t", ["a", "b", "c"], noise[l])]) for l, th in enumerate(self.thetas)]
        return qram, noise, mids

    # --------------------------------------------------------------- batched
    def build_batched(self):
        self.declare(batched=True)
        qram, noise, mids = self._layer_ops()
        H = Hadamard_Int_Batched("a", "w", self.h_max)
        self._built = ("batched", qram, noise, mids, H)
        return self

    def initial_batched(self):
        """One |t, h_t, 0, 0, 0> entry of amplitude 1 per instance."""
        t = np.arange(self.n_traj, dtype=np.uint64)
        z = np.zeros(self.n_traj, dtype=np.uint64)
        regs = np.stack([t, self.widths, z, z, z], axis=1)
        return regs, np.ones(self.n_traj, dtype=np.complex128)

    def run_batched(self, st: SparseState, count: bool = False, upload: bool = True) -> int:
        kind, _, _, mids, H = self._built
        assert kind == "batched"
        if upload:
            st.upload(*self.initial_batched())
        return self._run(st, lambda: H, mids, count)

    # ----------------------------------------------------------------- plain
    def build_plain(self):
        self.declare(batched=False)
        qram, noise, mids = self._layer_ops()
        Hs = {int(h): Hadamard_Int("a", int(h)) for h in np.unique(self.widths)}
        self._built = ("plain", qram, noise, mids, Hs)
        return self

    def run_plain(self, st: SparseState, traj: int, count: bool = False) -> int:
        kind, _, _, mids, Hs = self._built
        assert kind == "plain"
        st.upload(np.array([[traj, 0, 0, 0]], dtype=np.uint64), np.ones(1, dtype=np.complex128))
        H = Hs[int(self.widths[traj])]
        return self._run(st, lambda: H, mids, count)

    @staticmethod
    def _run(st, get_h, mids, count):
        upd = 0
        for mid in mids:
            H = get_h()
            n0 = st.size() if count else 0
            H(st)
            n1 = st.size() if count else 0
            mid(st)
            H(st)
            if count:
                n2 = st.size()
                upd += max(n0, n1) + 4 * n1 + max(n1, n2)
        return upd
