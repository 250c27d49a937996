"""The learned output-size model: its FP64 oracle pinned by finite
differences (CPU), the GPU forward/backward/Adam kernels against that oracle,
training on sizes logged by the split operators, and what the trained model
gains over the method without it at identical results."""
from __future__ import annotations

import re

import numpy as np
import pytest

from oracle import mlp_oracle as M

ROOT_HEADER = __import__("pathlib").Path(__file__).resolve().parent.parent / "include" / "sparq_gb300.h"


def test_header_constants_match():
    from sparqsim_gb300 import predictor as P
    h = ROOT_HEADER.read_text()
    assert int(re.search(r"#define SQ_PRED_FEATURES (\d+)", h).group(1)) == P.FEATURES == M.IN
    assert int(re.search(r"#define SQ_PRED_PARAMS (\d+)", h).group(1)) == P.PARAMS == M.PARAMS


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(scale=0.2, size=M.PARAMS)
    x = rng.normal(size=(7, M.IN))
    t = rng.normal(size=(7, M.OUT))
    _, g = M.loss_and_grad(p, x, t)
    idx = rng.choice(M.PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(M.PARAMS)
        e[i] = h
        num = (M.loss_and_grad(p + e, x, t)[0] - M.loss_and_grad(p - e, x, t)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, num, g[i])


def _random_problem(seed, n):
    rng = np.random.default_rng(seed)
    p = (rng.normal(scale=0.15, size=M.PARAMS)).astype(np.float32)
    x = rng.normal(size=(n, M.IN)).astype(np.float32)
    t = rng.normal(size=(n, M.OUT)).astype(np.float32)
    return p, x, t


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle():
    from sparqsim_gb300 import predictor as P
    p, x, t = _random_problem(5, 300)
    P.set_params(p)
    loss, g = P.gradient(x, t)
    ref_loss, ref_g = M.loss_and_grad(p.astype(np.float64), x, t)
    assert abs(loss - ref_loss) <= 1e-5 * abs(ref_loss)
    scale = np.abs(ref_g).max()
    assert np.abs(g - ref_g).max() <= 1e-5 * scale, np.abs(g - ref_g).max() / scale  # FP32 sums of 300 rows
    y = P.predict(x)
    ref_y, _ = M.forward(p.astype(np.float64), x)
    assert np.abs(y - ref_y).max() <= 1e-5 * np.abs(ref_y).max()


@pytest.mark.gpu
def test_gpu_adam_matches_oracle():
    """Full-batch steps: each minibatch holds every row, so the GPU update
    equals the oracle's up to FP32 rounding."""
    from sparqsim_gb300 import predictor as P
    p, x, t = _random_problem(6, 64)
    P.set_params(p)
    P.train(x, t, epochs=5, batch=64, lr=1e-3, seed=1)
    got = P.get_params()
    q = p.astype(np.float64)
    m = np.zeros_like(q)
    v = np.zeros_like(q)
    for step in range(1, 6):
        _, g = M.loss_and_grad(q, x, t)
        q, m, v = M.adam(q, g, m, v, step, 1e-3)
    assert np.abs(got - q).max() <= 2e-5 * np.abs(q).max(), np.abs(got - q).max()


@pytest.mark.gpu
def test_training_reduces_loss():
    from sparqsim_gb300 import predictor as P
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, size=(2000, M.IN)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.abs(x[:, 3]) - 0.5], axis=1).astype(np.float32)
    P.reset(seed=2)
    before, _ = P.gradient(x, t)
    P.train(x, t, epochs=60, batch=128, lr=2e-3, seed=3)
    after, _ = P.gradient(x, t)
    assert after < 0.2 * before, (before, after)


def _collapse_circuit(ps, h, groups, seed):
    """H(a, h) on `groups` singleton entries (fan-out to groups * 2^h), a key
    change outside a (drops the cached group ranges), then H(a, h) again: full
    groups that merge back to `groups` entries."""
    rng = np.random.default_rng(seed)
    ps.System.clear()
    ps.System.add_register("a", ps.UnsignedInteger, 12)
    ps.System.add_register("b", ps.UnsignedInteger, 20)
    ps.System.add_register("c", ps.UnsignedInteger, 8)
    b = rng.choice(1 << 20, groups, replace=False).astype(np.uint64)
    regs = np.stack([rng.integers(0, 1 << 12, groups).astype(np.uint64) & ~np.uint64((1 << h) - 1), b,
                     np.zeros(groups, dtype=np.uint64)], axis=1)
    amps = rng.normal(size=groups) + 1j * rng.normal(size=groups)
    st = ps.SparseState()
    st.upload(regs, amps / np.linalg.norm(amps))
    H = ps.Hadamard_Int("a", h)
    H(st)
    ps.Add_ConstUInt_InPlace("c", 5)(st)
    return st, H


@pytest.mark.gpu
def test_trained_model_gain():
    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native
    from sparqsim_gb300 import predictor as P

    def run_heldout(model_on):
        P.enable(model_on)
        st, H = _collapse_circuit(ps, 8, 6000, seed=99)
        _native.profile_reset()
        _native.profile_enable(True)
        H(st)
        _native.profile_enable(False)
        prof = _native.profile_read()
        regs, amps = st.download()
        order = np.lexsort(regs.T[::-1])
        return prof, regs[order], amps[order]

    try:
        ps.set_group_strategy("hash")
        P.set_single_pass_limit(1 << 16)   # the fully populated bound of the held-out merge exceeds this
        P.set_hash_groups_hint(1024)       # and its group count exceeds the table's default sizing
        # log sizes from a family of circuits, train, predict
        P.clear_log()
        P.log(True)
        for h in (6, 7, 9, 10):
            for groups in (1500, 3000, 5000, 9000, 12000):
                if groups << h > 6_000_000:
                    continue
                for seed in range(3):
                    st, H = _collapse_circuit(ps, h, groups, seed=100 * h + groups + seed)
                    H(st)
        P.log(False)
        x, t = P.read_log()
        assert x.shape[0] >= 40
        P.reset(seed=4)
        P.train(x, t, epochs=400, batch=32, lr=3e-3, seed=5)
        base_prof, base_regs, base_amps = run_heldout(False)
        over0 = P.stats()["single_pass_overflows"]
        prof, regs, amps = run_heldout(True)
        assert P.stats()["single_pass_overflows"] == over0      # the predicted capacity held
        # identical results either way
        assert np.array_equal(regs, base_regs)
        assert np.array_equal(amps.view(np.float64), base_amps.view(np.float64))
        assert regs.shape[0] == 6000
        # without the model: count pass + scan + write pass, and a hash table retry
        single = ("emit_hadamard_single_pass", "emit_hadamard_merge")  # named by the groups' shape
        assert "emit_hadamard_count" in base_prof and not any(k in base_prof for k in single)
        assert base_prof["hash_insert"][0] == 2
        # with it: one emit pass and one table
        assert any(k in prof for k in single) and "emit_hadamard_count" not in prof
        assert prof["hash_insert"][0] == 1
        emit_ms = lambda pr: sum(v[1] for k, v in pr.items() if k.startswith(("emit_", "scan_counts", "hash_insert")))
        print(f"model gain: grouping+emit {emit_ms(base_prof):.3f} ms -> {emit_ms(prof):.3f} ms")
    finally:
        P.enable(False)
        P.log(False)
        P.set_single_pass_limit(0)
        P.set_hash_groups_hint(0)
        ps.set_group_strategy("autotune")


@pytest.mark.gpu
@pytest.mark.parametrize("h, groups, members", [(8, 600, 60), (12, 64, 600)])
def test_underpredicted_single_pass_falls_back_to_exact(dual, h, groups, members):
    """The size model predicts far too few outputs (its last bias set to
    2^-16 of the input size): the single pass overflows its capacity, writes
    nothing past it, counts an overflow, and the exact count -> scan -> write
    path gives the oracle's entries bit for bit, as the run without the model
    does."""
    import sparqsim_gb300 as ps
    from sparqsim_gb300 import predictor as P

    U = ps.UnsignedInteger
    dual.reg("a", U, 12)
    dual.reg("b", U, 20)
    rng = np.random.default_rng(h * 1000 + groups)
    b = rng.choice(1 << 20, groups, replace=False).astype(np.uint64)
    regs = np.stack([np.concatenate([rng.choice(1 << h, members, replace=False) for _ in range(groups)]),
                     np.repeat(b, members)], axis=1).astype(np.uint64)
    amps = rng.normal(size=len(regs)) + 1j * rng.normal(size=len(regs))
    amps /= np.linalg.norm(amps)
    assert len(regs) >= 1 << 15  # the model is consulted from 2^15 entries
    params = np.zeros(P.PARAMS, dtype=np.float32)
    params[-1] = -1.0  # log2(outputs / N) / 16 = -1
    results = {}
    try:
        ps.set_group_strategy("hash")
        P.set_single_pass_limit(1 << 16)  # the fully populated bound exceeds this
        for model_on in (True, False):
            P.set_params(params)
            P.enable(model_on)
            dual.start(regs, amps)
            over0 = P.stats()["single_pass_overflows"]
            dual.apply(ps.Hadamard_Int("a", h))
            over1 = P.stats()["single_pass_overflows"]
            assert over1 == over0 + (1 if model_on else 0)
            assert dual.gpu.size() > 4200  # more than the predicted capacity
            dual.compare(exact_amp=True)
            results[model_on] = dual.gpu.download()
    finally:
        P.enable(False)
        P.set_single_pass_limit(0)
        ps.set_group_strategy("autotune")
    # the same entries either way (their order follows the hash grouping's)
    (rk, ra), (bk, ba) = results[True], results[False]
    ro, bo = np.lexsort(rk.T[::-1]), np.lexsort(bk.T[::-1])
    assert np.array_equal(rk[ro], bk[bo]) and np.array_equal(ra[ro].view(np.float64), ba[bo].view(np.float64))
