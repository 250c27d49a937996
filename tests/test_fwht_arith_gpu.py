"""Accuracy of the two FWHT arithmetics against exact rational arithmetic.

'reference' runs the reference's FP64 butterflies (a0 +- a1) * sqrt2inv stage
by stage (hadamard.cpp:44-59,100-131) and is bit-identical to the oracle.
'exact-sum' puts a group's amplitudes on one integer grid of spacing
2^(E - F) (E: smallest power of two above every component, F = 62 - n), sums
exactly and rounds each output once, so its error is bounded by
    |y - y_exact| <= (members / 2^(n/2)) * 2^(E - F - 1) + ulp(y) / 2.
Both are checked here on groups whose amplitudes span six decades."""
from __future__ import annotations

from fractions import Fraction

import numpy as np
import pytest

import sparqsim_gb300 as ps

pytestmark = pytest.mark.gpu

U = ps.UnsignedInteger


def _exact_fwht(xs):
    """Exact H^{(x)n} of a list of Fractions (unnormalised)."""
    v = list(xs)
    h = 1
    while h < len(v):
        for i in range(0, len(v), 2 * h):
            for j in range(i, i + h):
                a, b = v[j], v[j + h]
                v[j], v[j + h] = a + b, a - b
        h *= 2
    return v


@pytest.mark.parametrize("n,members", [(12, 4096), (12, 1500), (7, 128), (7, 40), (4, 16)])
def test_fwht_error_bound(n, members):
    rng = np.random.default_rng(1000 * n + members)
    ps.System.add_register("a", U, n)
    ps.System.add_register("b", U, 3)
    t = np.sort(rng.choice(1 << n, members, replace=False))
    mags = 10.0 ** rng.uniform(-6, 0, (members, 2))
    amps = (mags[:, 0] * rng.choice([-1, 1], members)) + 1j * (mags[:, 1] * rng.choice([-1, 1], members))
    regs = np.stack([t, np.full(members, 5)], axis=1).astype(np.uint64)
    # exact result (n even: 2^(n/2) scale; odd n compared after the same scale)
    re = [Fraction(0)] * (1 << n)
    im = [Fraction(0)] * (1 << n)
    for i, ti in enumerate(t):
        re[int(ti)] = Fraction(float(amps[i].real))
        im[int(ti)] = Fraction(float(amps[i].imag))
    yr, yi = _exact_fwht(re), _exact_fwht(im)
    scale = 2.0 ** (-(n // 2)) * (2 ** -0.5 if n & 1 else 1.0)
    exact = np.array([float(a) * scale for a in yr]) + 1j * np.array([float(b) * scale for b in yi])
    emax = max(np.frexp(np.abs(amps.real))[1].max(), np.frexp(np.abs(amps.imag))[1].max())  # |x| < 2^emax
    grid = 2.0 ** (emax - (62 - n) - 1)  # half the grid spacing
    errs = {}
    for arith in ("reference", "exact-sum"):
        ps.set_fwht_arithmetic(arith)
        ps.set_clearzero_default_eps(0.0)
        st = ps.SparseState()
        st.upload(regs, amps)
        ps.Hadamard_Int("a", n)(st)
        out_regs, out_amps = st.download()
        got = np.zeros(1 << n, dtype=np.complex128)
        got[out_regs[:, 0].astype(np.int64)] = out_amps
        assert np.all(out_regs[:, 1] == 5)
        err = np.abs(got - exact)
        errs[arith] = err.max() / np.abs(exact).max()
        if arith == "exact-sum":
            bound = members * scale * grid * 2 + np.spacing(np.abs(exact)) * 2  # re and im parts
            assert np.all(err <= bound), f"exact-sum error above its bound: {(err / bound).max()}"
    assert errs["exact-sum"] < 1e-13 and errs["reference"] < 1e-13, errs
    ps.set_clearzero_default_eps(1e-14)
