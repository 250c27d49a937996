"""The Poiseuille QDA benchmark's classical side (CPU): the analytic condition
number, the Thomas solution, the residual definitions and the step budget,
each against a direct numpy statement (PoiseuilleQDABench.cu:57-88,164-228).
The GPU run of the driver is in test_qda_gpu.py."""
from __future__ import annotations

import math

import numpy as np
import pytest

from sparqsim_gb300 import poiseuille as P

ALPHA, BETA = 2.2666666666564934, -1.0


def _A(n, alpha=ALPHA, beta=BETA):
    return alpha * np.eye(n) + beta * (np.eye(n, k=1) + np.eye(n, k=-1))


def test_analytic_kappa():
    for n in (4, 37, 64):
        assert P.analytic_kappa(ALPHA, BETA, n) == pytest.approx(np.linalg.cond(_A(n)), rel=1e-10)
    # the benchmark's alpha is chosen for kappa = 16 as n grows
    assert P.analytic_kappa(ALPHA, BETA, 1 << 20) == pytest.approx(16.0, rel=1e-6)


def test_thomas_reference():
    for n in (2, 5, 100):
        x = np.linalg.solve(_A(n), np.ones(n) / math.sqrt(n))
        assert np.allclose(P.thomas_reference(ALPHA, BETA, n), x / np.linalg.norm(x), atol=1e-13)


def test_residuals_definitions():
    n = 32
    xref = P.thomas_reference(ALPHA, BETA, n)
    out = np.zeros(4 * n, dtype=np.complex128)
    out[n:2 * n] = 0.6 * xref
    out[0] = 0.8
    rd, ro, succ, fid = P.residuals(out, n, ALPHA, BETA, xref)
    assert rd < 1e-7 and ro < 1e-7  # y = A x is parallel to b
    assert succ == pytest.approx(0.36, abs=1e-14) and fid == pytest.approx(1.0, abs=1e-14)
    rng = np.random.default_rng(3)
    out[n:2 * n] = rng.normal(size=n) + 1j * rng.normal(size=n)
    rd, ro, succ, fid = P.residuals(out, n, ALPHA, BETA, xref)
    x = out[n:2 * n] / np.linalg.norm(out[n:2 * n])
    y = _A(n) @ x
    b = np.ones(n) / math.sqrt(n)
    proj = np.vdot(b, y)
    assert ro == pytest.approx(math.sqrt(np.linalg.norm(y) ** 2 - abs(proj) ** 2), rel=1e-12)
    assert rd == pytest.approx(math.sqrt(max(2 - 2 * proj.real / np.linalg.norm(y), 0)), rel=1e-12)
    assert fid == pytest.approx(abs(np.dot(xref, x)) ** 2, rel=1e-12)
    assert succ == pytest.approx(np.linalg.norm(out[n:2 * n]) ** 2, rel=1e-14)
    # an empty solution block: NaN residuals, zero success probability
    out[n:2 * n] = 0
    rd, ro, succ, fid = P.residuals(out, n, ALPHA, BETA, xref)
    assert math.isnan(rd) and math.isnan(ro) and math.isnan(fid) and succ == 0.0


def test_step_budget_and_cli_defaults():
    assert P.step_budget(1.1, 16.0, 10 ** 9) == (40568, 40568)
    assert P.step_budget(0.1, 16.0, 10 ** 9) == (3688, 3688)
    assert P.step_budget(1.1, 16.0, 41) == (40568, 40)
    assert P.step_budget(1.1, 16.0, 1) == (40568, 2)
    a = P.parser().parse_args([])
    assert (a.steprate, a.p, a.nqubit, a.alpha, a.beta, a.logEvery, a.tol, a.czEps) == \
        (1.1, 1.3, 20, ALPHA, BETA, 250, 1e-6, 1e-14)
