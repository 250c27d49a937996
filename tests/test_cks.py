"""The CKS solver's classical side (CPU): the quantised tridiagonal matrix and
its combined table, the walk spectrum, the stock and least-squares LCU
coefficients, and the angle lookup table's coverage
(SparQ_Algorithm/include/hamiltonian_simulation_tridiagonal.h,
src/hamiltonian_simulation.cpp:40-100, Experiments/CKS/CKSPoiseuilleBench.cu)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from sparqsim_gb300 import cks

ALPHA, BETA = 2.2666666666564934, -1.0


def test_quantised_matrix_and_combined_table():
    mat, spec = cks.make_tridiagonal_matrix_spec(ALPHA, BETA, 16, 32)
    lam = ALPHA + 2.0
    assert spec.alpha_enc == math.floor(ALPHA / lam * 2.0 ** 32)
    assert spec.beta_enc == math.floor(1.0 / lam * 2.0 ** 32)
    assert (spec.sparse_offset, spec.addr_mask, spec.k_width) == (64, 127, 32)
    assert mat.get_sparsity_offset() == 64
    # windows: interior rows {j-1..j+2}, clamped at both ends
    assert [spec.window_base(j) for j in (0, 1, 2, 13, 14, 15, 1000)] == [0, 0, 1, 12, 12, 12, 12]
    for j in range(16):
        row = [spec.value_of(j, s) for s in range(4)]
        cols = [spec.col_of(j, s) for s in range(4)]
        for s in range(4):
            want = spec.alpha_enc if cols[s] == j else spec.beta_enc if abs(cols[s] - j) == 1 else 0
            assert row[s] == want
            assert spec.combined_mem(4 * j + s) == row[s]
            assert spec.combined_mem(64 + 4 * j + s) == cols[s]
            assert spec.combined_mem(128 + 4 * j + s) == row[s]  # masked to 8n words
    with pytest.raises(ValueError):
        cks.make_tridiagonal_matrix_spec(ALPHA, BETA, 12, 32)


def test_walk_spectrum_is_the_quantised_matrix_spectrum():
    for n in (8, 16, 64):
        _, spec = cks.make_tridiagonal_matrix_spec(ALPHA, BETA, n, 32)
        A = (spec.alpha_enc * np.eye(n) + spec.beta_enc * (np.eye(n, k=1) + np.eye(n, k=-1))) / (2.0 ** 32 * 4)
        ev = np.linalg.eigvalsh(A)
        m, M = cks.walk_spectrum(spec)
        assert m == pytest.approx(ev.min() * (1 - 1e-12), rel=1e-12)
        assert M == pytest.approx(ev.max() * (1 + 1e-12), rel=1e-12)


def test_stock_coefficients():
    c = cks.ChebyshevPolynomialCoefficient(40)  # exact binomial tail for b <= 100
    for j in (0, 3, 10, 39):
        want = 4 * sum(math.comb(80, 40 + i) for i in range(j + 1, 41)) / 4.0 ** 40
        assert c.coef(j) == pytest.approx(want, rel=1e-12)
    big = cks.ChebyshevPolynomialCoefficient(1435)
    assert big.coef(7) == 2 * math.erfc(7.5 / math.sqrt(1435))
    assert [c.sign(j) for j in range(4)] == [False, True, False, True]
    assert [c.step(j) for j in range(3)] == [1, 3, 5]


def test_inverse_coefficients_fit_one_over_x():
    _, spec = cks.make_tridiagonal_matrix_spec(ALPHA, BETA, 16, 32)
    m, M = cks.walk_spectrum(spec)
    inv = cks.ChebyshevInverseCoefficients(m, M, 640)
    assert inv.coef.shape == (641,) and inv.a == pytest.approx(np.abs(inv.coef).sum())
    x = np.linspace(m, M, 997)
    t = np.arccos(np.clip(x, -1, 1))
    approx = np.cos(np.outer(t, 2 * np.arange(641) + 1)) @ inv.coef
    assert np.max(np.abs(approx * x - 1)) < 1e-6


def test_angle_table_covers_every_table_word():
    mat, spec = cks.make_tridiagonal_matrix_spec(ALPHA, BETA, 16, 32)
    dense, extra = mat.oracle_values()
    words = {spec.combined_mem(i) for i in range(8 * 16)}
    assert all(w < dense or w in extra for w in words)
    assert extra == sorted({spec.alpha_enc, spec.beta_enc})
