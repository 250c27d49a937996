"""The Poiseuille QDA linear-solver benchmark on the GB300 engine.

Same contract as the reference's production driver
(Experiments/QDA/QDA_Poiseuille/PoiseuilleQDABench.cu:100-290): the 1D Poisson
matrix A = tridiag(beta, alpha, beta), b = ones(n) / sqrt(n), the walk
W_s (qda.WalkS) over s = i / steps for steps = ceil(rate * 2305 * kappa)
(made even), ClearZero(czEps) and Normalize after every step, and at every
log point the GetOutput read-out with the residuals res_dir, res_opt, the
success probability and the fidelity with the classical (Thomas) solution.
Writes `residual_curve.csv` and `qda_summary.json` into --outdir and stops
early once res_dir < tol.

    python -m sparqsim_gb300.poiseuille --nqubit 16 --maxSteps 1000 --outdir out
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

STEP_CONSTANT = 2305


def analytic_kappa(alpha: float, beta: float, n: int) -> float:
    """max/min of |alpha + 2 beta cos(pi k / (n + 1))|, k = 1..n
    (PoiseuilleQDABench.cu:57-65)."""
    k = np.arange(1, n + 1, dtype=np.float64)
    lam = np.abs(alpha + 2.0 * beta * np.cos(np.pi * k / float(n + 1)))
    return float(lam.max() / lam.min())


def thomas_reference(alpha: float, beta: float, n: int) -> np.ndarray:
    """Unit-norm solution of tridiag(beta, alpha, beta) x = ones / sqrt(n) by
    the Thomas recurrence (PoiseuilleQDABench.cu:67-88)."""
    bi = 1.0 / math.sqrt(n)
    cp = np.empty(max(n - 1, 1))
    dp = np.empty(n)
    cp[0] = beta / alpha
    dp[0] = bi / alpha
    for i in range(1, n):
        m = alpha - beta * cp[i - 1]
        if i < n - 1:
            cp[i] = beta / m
        dp[i] = (bi - beta * dp[i - 1]) / m
    x = np.empty(n)
    x[n - 1] = dp[n - 1]
    for i in range(n - 2, -1, -1):
        x[i] = dp[i] - cp[i] * x[i + 1]
    return x / math.sqrt(float(np.dot(x, x)))


def residuals(out: np.ndarray, n: int, alpha: float, beta: float, xref: np.ndarray):
    """(res_dir, res_opt, success probability, fidelity) of a GetOutput vector
    (PoiseuilleQDABench.cu:193-228): the block out[n:2n) normalised to x,
    y = A x; res_dir = sqrt(2 - 2 <y/|y|, b>), res_opt = sqrt(|y|^2 - |<b, y>|^2),
    succP = |out[n:2n)|^2, fid = |<xref, x>|^2; NaN residuals when the block
    is empty."""
    blk = out[n:2 * n]
    blk_nrm2 = float(np.sum(blk.real ** 2 + blk.imag ** 2))
    blk_nrm = math.sqrt(blk_nrm2)
    if not blk_nrm > 1e-300:
        return math.nan, math.nan, blk_nrm2, math.nan
    x = blk / blk_nrm
    y = alpha * x
    y[:-1] += beta * x[1:]
    y[1:] += beta * x[:-1]
    y_nrm2 = float(np.sum(y.real ** 2 + y.imag ** 2))
    y_nrm = math.sqrt(y_nrm2)
    bnorm_inv = 1.0 / math.sqrt(n)
    proj_re = bnorm_inv * float(np.sum(y.real))
    proj_im = bnorm_inv * float(np.sum(y.imag))
    rd = math.sqrt(max(2.0 - 2.0 * proj_re / y_nrm, 0.0))
    ro = math.sqrt(max(y_nrm2 - (proj_re * proj_re + proj_im * proj_im), 0.0))
    fr = float(np.dot(xref, x.real))
    fi = float(np.dot(xref, x.imag))
    return rd, ro, blk_nrm2, fr * fr + fi * fi


def step_budget(step_rate: float, kappa: float, max_steps: int) -> tuple[int, int]:
    """(budget, steps): budget = ceil(rate * 2305 * kappa); steps = the budget
    capped at max_steps, made even, at least 2 (PoiseuilleQDABench.cu:164-168)."""
    budget = int(math.ceil(step_rate * STEP_CONSTANT * kappa))
    steps = min(budget, max_steps)
    if steps % 2 == 1:
        steps -= 1
    return budget, max(steps, 2)


def _fmt(v: float):
    return None if math.isnan(v) else v


def run(args) -> dict:
    import sparqsim_gb300 as ps
    from . import qda

    if args.logEvery % 2 == 1:
        args.logEvery += 1  # 2-step periodicity: log points on valid solution blocks
    n = 1 << args.nqubit
    kappa_analytic = analytic_kappa(args.alpha, args.beta, n)
    kappa = args.kappa if args.kappa > 0 else kappa_analytic
    os.makedirs(args.outdir, exist_ok=True)
    xref = thomas_reference(args.alpha, args.beta, n)
    print(f"[INFO] n={n} nqubit={args.nqubit} kappa={kappa:.17g} (analytic={kappa_analytic:.17g}) "
          f"rate={args.steprate:.17g} alpha={args.alpha:.17g} beta={args.beta:.17g} p={args.p:.17g}", flush=True)
    print(f"[INFO] outdir={args.outdir} log_every={args.logEvery} tol={args.tol:.17g}", flush=True)

    ps.System.clear()
    ps.set_clearzero_default_eps(args.czEps)  # the walk's own ClearZero calls follow the same threshold
    state = ps.SparseState(capacity=1 << 20)

    class Peak(qda.Runner):
        """Tracks the largest entry count seen (System::max_system_size)."""

        def __init__(self, st):
            super().__init__(st)
            self.peak = 0

        def op(self, o, dag=False):
            super().op(o, dag)
            self.peak = max(self.peak, self.state.size())

    run_ = Peak(state)
    for name, typ, width in (("main", ps.UnsignedInteger, args.nqubit), ("anc_UA", ps.UnsignedInteger, 4),
                             ("anc_4", ps.Boolean, 1), ("anc_3", ps.Boolean, 1), ("anc_2", ps.Boolean, 1),
                             ("anc_1", ps.Boolean, 1)):
        ps.AddRegister(name, typ, width)(state)
    enc_b = qda.StatePrepHadamard("main")
    enc_b.apply(run_)  # |b>: uniform superposition over main
    enc_A = qda.BlockEncodingTridiagonal("main", "anc_UA", args.alpha, args.beta)
    getoutput = qda.GetOutput("main", "anc_UA", "anc_4", "anc_3", "anc_2", "anc_1", False)

    budget, steps = step_budget(args.steprate, kappa, args.maxSteps)
    print(f"[INFO] steps budget={steps} (StepConstant={STEP_CONSTANT})", flush=True)
    curve = []
    termination = "fixed_step_budget"
    t0 = time.perf_counter()
    t_extract = 0.0
    with open(os.path.join(args.outdir, "residual_curve.csv"), "w") as cf:
        cf.write("step,res_dir,res_opt,success_prob,fidelity\n")
        for i in range(steps):
            qda.WalkS(enc_A, enc_b, "main", "anc_UA", "anc_1", "anc_2", "anc_3", "anc_4", i / steps, kappa,
                      args.p).apply(run_)
            run_.op(ps.ClearZero(args.czEps))
            run_.op(ps.Normalize())
            if (i + 1) % args.logEvery == 0 or i == steps - 1:
                te = time.perf_counter()
                out, _ = getoutput(state)
                rd, ro, succ, fid = residuals(out, n, args.alpha, args.beta, xref)
                t_extract += time.perf_counter() - te
                curve.append((i + 1, rd, ro, succ, fid))
                cf.write(f"{i + 1},{rd:.17g},{ro:.17g},{succ:.17g},{fid:.17g}\n")
                cf.flush()
                wall = time.perf_counter() - t0
                print(f"{time.strftime('%Y-%m-%d %H:%M:%S')} | step {i + 1:7d}/{steps} res_dir={rd:.6e} "
                      f"res_opt={ro:.6e} succP={succ:.4f} fid={fid:.6f} wall={wall:.1f}s max_sys={run_.peak}",
                      flush=True)
                if not math.isnan(rd) and rd < args.tol:
                    termination = f"residual_below_tol({args.tol:g})"
                    break
    wall = time.perf_counter() - t0
    last = curve[-1] if curve else (0, math.nan, math.nan, math.nan, math.nan)
    summary = {
        "engine": "qda (GB300 sparse-state engine: WalkS + GetOutput post-selected read-out)",
        "backend": "CUDA sm_103a (sparqsim_gb300)",
        "dimension": n, "nqubit": args.nqubit, "kappa": kappa, "kappa_analytic": kappa_analytic,
        "eps": 0.01, "alpha": args.alpha, "beta": args.beta, "p": args.p, "clearzero_eps": args.czEps,
        "problem": "1D Poisson tridiagonal, b=ones/sqrt(n)",
        "step_budget": budget, "steps_executed": last[0], "step_rate": args.steprate,
        "step_constant": STEP_CONSTANT, "termination": termination, "tol": args.tol,
        "final_res_dir": _fmt(last[1]), "final_res_opt": _fmt(last[2]),
        "final_success_prob": _fmt(last[3]), "final_fidelity_vs_classical": _fmt(last[4]),
        "wall_time_s": wall, "time_per_step_s": wall / max(1, last[0]), "extract_time_s": t_extract,
        "max_system_size": run_.peak,
    }
    with open(os.path.join(args.outdir, "qda_summary.json"), "w") as f:
        json.dump(summary, f, indent=2)
    print(f"[OK] steps={last[0]} final_res_dir={last[1]:.6e} fid={last[4]:.6f} wall={wall:.1f}s -> {args.outdir}",
          flush=True)
    return summary


def parser() -> argparse.ArgumentParser:
    """The reference driver's options and defaults (PoiseuilleQDABench.cu:103-129)."""
    ap = argparse.ArgumentParser("poiseuille", description="QDA linear-solver benchmark (tridiagonal Poiseuille "
                                                           "case) on the GB300 engine")
    ap.add_argument("-s", "--steprate", type=float, default=1.1, help="steps = ceil(rate*2305*kappa)")
    ap.add_argument("--p", type=float, default=1.3, help="walk parameter p")
    ap.add_argument("--nqubit", type=int, default=20, help="main register qubit count (dimension = 2^nq)")
    ap.add_argument("--alpha", type=float, default=2.2666666666564934, help="tridiagonal diagonal coefficient")
    ap.add_argument("--beta", type=float, default=-1.0, help="tridiagonal sub-diagonal coefficient")
    ap.add_argument("--kappa", type=float, default=0.0, help="override the analytic condition number")
    ap.add_argument("--logEvery", type=int, default=250, help="steps between residual log points (even)")
    ap.add_argument("--tol", type=float, default=1e-6, help="res_dir convergence threshold")
    ap.add_argument("--maxSteps", type=int, default=10 ** 9, help="hard cap on executed steps")
    ap.add_argument("--outdir", default=".", help="output directory")
    ap.add_argument("--czEps", type=float, default=1e-14, help="ClearZero pruning threshold")
    return ap


def main(argv=None) -> int:
    run(parser().parse_args(argv))
    return 0


if __name__ == "__main__":
    sys.exit(main())
