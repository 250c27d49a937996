"""The Poiseuille CKS linear-solver benchmark on the GB300 engine.

Same contract as the reference's driver (Experiments/CKS/CKSPoiseuilleBench.cu:
139-420): A = tridiag(beta, alpha, beta) quantised to ds bits, b = ones(n) /
sqrt(n) prepared as a uniform Hadamard plus the parity phase D (the walk
implements |A| = D A D), the first walk step, then one Chebyshev LCU term per
Step() (stock or least-squares 1/x coefficients on the exact walk spectrum).
Every `--logEvery` terms the LCU state is post-selected (non-destructively),
D is undone on the read-out and res_dir, res_opt, the success probability and
the fidelity with the Thomas solution are logged; the run stops once
res_dir < tol. Writes `residual_curve.csv` (step = 2j + 1 walk steps) and
`qda_summary.json`.

    python -m sparqsim_gb300.cks_bench --nqubit 4 --J 640 --outdir out
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

from .poiseuille import analytic_kappa, residuals, thomas_reference


def residual_metrics(m: np.ndarray, n: int, alpha: float, beta: float, xref: np.ndarray):
    """(res_dir, res_opt, fid, |m|^2) of the read-out m (CKSPoiseuilleBench.cu:98-136)."""
    out = np.zeros(2 * n, dtype=np.complex128)
    out[n:] = m
    rd, ro, blk2, fid = residuals(out, n, alpha, beta, xref)
    return rd, ro, fid, blk2


def read_out(state, input_reg: str, n: int, dphase: bool) -> np.ndarray:
    """Amplitudes of the post-selected state by input-register value, with
    D = diag((-1)^i) undone (CKSPoiseuilleBench.cu:341-345)."""
    from .core import System
    regs, amps = state.download()
    m = np.zeros(n, dtype=np.complex128)
    if len(amps):
        idx = regs[:, System.resolve(input_reg)].astype(np.int64)
        sign = np.where((idx & 1) & (1 if dphase else 0), -1.0, 1.0)
        m[idx] = amps * sign
    return m


def _fmt(v: float):
    return None if math.isnan(v) else v


def run(args) -> dict:
    import sparqsim_gb300 as ps
    from . import cks

    n = 1 << args.nqubit
    kappa_analytic = analytic_kappa(args.alpha, args.beta, n)
    kappa = args.kappa if args.kappa > 0 else 16.0
    os.makedirs(args.outdir, exist_ok=True)
    ps.System.clear()
    mat, spec = cks.make_tridiagonal_matrix_spec(args.alpha, args.beta, n, args.ds)
    xref = thomas_reference(args.alpha, args.beta, n)
    m_spec, M_spec = cks.walk_spectrum(spec)
    print(f"[INFO] n={n} nqubit={args.nqubit} kappa={kappa:.17g} (analytic={kappa_analytic:.17g}) eps={args.eps:g} "
          f"ds={args.ds} nnz_col={mat.nnz_col}", flush=True)
    print(f"[INFO] alpha_enc={spec.alpha_enc} beta_enc={spec.beta_enc}", flush=True)
    print(f"[INFO] Ahat spectrum [{m_spec:.9f}, {M_spec:.9f}] (kappa_interval={M_spec / m_spec:.6f})", flush=True)

    obj = cks.LCU_Container_NoiseFree_Tridiagonal(mat, spec, kappa, args.eps, checks=not args.noChecks)
    if args.coef == "true":
        inv = cks.ChebyshevInverseCoefficients(m_spec, M_spec, args.J)
        print(f"[INFO] true coefficients: J={inv.J} sum|d|={inv.a:.6e}", flush=True)
        obj.set_inverse_coefficients(inv)
    dphase = bool(args.dphase)
    input_reg = obj.GetInputVecReg()
    st = obj.step_state
    ps.Hadamard_Int(input_reg, obj.quantum_walk_obj.get_init_size())(st)
    if dphase:
        cks.TridiagParityPhase(input_reg)(st)
    ps.ClearZero()(st)
    obj.quantum_walk_obj.FirstStep(obj.run)
    print(f"[INFO] state size after FirstStep = {st.size()}", flush=True)

    curve = []
    termination = "full_lcu_expansion"
    t0 = time.perf_counter()
    t_extract = 0.0
    j = 0
    with open(os.path.join(args.outdir, "residual_curve.csv"), "w") as cf:
        cf.write("step,res_dir,res_opt,success_prob,fidelity\n")
        while obj.Step():
            j += 1
            last_term = j == obj.j0 + 1 or j == args.maxTerms
            if j % args.logEvery == 0 or last_term:
                te = time.perf_counter()
                state, p_succ = obj.PartialTrace_Nondestructive()
                m = read_out(state, input_reg, n, dphase)
                rd, ro, fid, _ = residual_metrics(m, n, args.alpha, args.beta, xref)
                t_extract += time.perf_counter() - te
                curve.append((j, rd, ro, p_succ, fid))
                cf.write(f"{2 * j + 1},{rd:.17g},{ro:.17g},{p_succ:.17g},{fid:.17g}\n")
                cf.flush()
                wall = time.perf_counter() - t0
                print(f"{time.strftime('%Y-%m-%d %H:%M:%S')} | term {j:5d}/{obj.j0} (walk {2 * j + 1:5d}) "
                      f"res_dir={rd:.6e} res_opt={ro:.6e} succP={p_succ:.6e} fid={fid:.8f} wall={wall:.1f}s "
                      f"max_sys={obj.max_system_size}", flush=True)
                if not math.isnan(rd) and rd < args.tol:
                    termination = f"residual_below_tol({args.tol:g})"
                    break
            if j == args.maxTerms:
                termination = f"max_terms({args.maxTerms})"
                break
    wall = time.perf_counter() - t0
    last = curve[-1] if curve else (0, math.nan, math.nan, math.nan, math.nan)
    summary = {
        "engine": "cks (GB300 sparse-state engine: tridiagonal QRAM-free walk + Chebyshev LCU)",
        "backend": "CUDA sm_103a (sparqsim_gb300)",
        "dimension": n, "nqubit": args.nqubit, "kappa": kappa, "kappa_analytic": kappa_analytic,
        "eps": args.eps, "alpha": args.alpha, "beta": args.beta, "ds": args.ds, "coef_mode": args.coef,
        "J": args.J if args.coef == "true" else 0, "dphase": int(dphase),
        "problem": "1D Poisson tridiagonal, b=ones/sqrt(n)",
        "lcu_terms": obj.j0 + 1, "walk_steps": 2 * (obj.j0 + 1), "terms_executed": j,
        "termination": termination, "tol": args.tol,
        "final_res_dir": _fmt(last[1]), "final_res_opt": _fmt(last[2]),
        "final_success_prob": _fmt(last[3]), "final_fidelity_vs_classical": _fmt(last[4]),
        "wall_time_s": wall, "time_per_term_s": wall / max(1, j), "extract_time_s": t_extract,
        "max_system_size": obj.max_system_size,
    }
    with open(os.path.join(args.outdir, "qda_summary.json"), "w") as f:
        json.dump(summary, f, indent=2)
    print(f"[OK] terms={j} walk_steps={2 * j + 1} final_res_dir={last[1]:.6e} fid={last[4]:.8f} wall={wall:.1f}s "
          f"-> {args.outdir}", flush=True)
    return summary


def parser() -> argparse.ArgumentParser:
    """The reference driver's options and defaults (CKSPoiseuilleBench.cu:140-172)."""
    ap = argparse.ArgumentParser("cks_bench", description="CKS (Chebyshev LCU quantum walk) linear-solver benchmark "
                                                          "(tridiagonal Poiseuille case) on the GB300 engine")
    ap.add_argument("--nqubit", type=int, default=20, help="main register qubit count (dimension = 2^nq)")
    ap.add_argument("--alpha", type=float, default=2.2666666666564934, help="tridiagonal diagonal coefficient")
    ap.add_argument("--beta", type=float, default=-1.0, help="tridiagonal sub-diagonal coefficient")
    ap.add_argument("--kappa", type=float, default=0.0, help="override condition number (default 16)")
    ap.add_argument("--eps", type=float, default=0.01, help="CKS target precision")
    ap.add_argument("--ds", type=int, default=32, help="matrix element quantization bits")
    ap.add_argument("--coef", choices=("true", "stock"), default="true", help="LCU coefficient family")
    ap.add_argument("--J", type=int, default=640, help="truncation for true coefficients")
    ap.add_argument("--dphase", type=int, default=1, help="apply the D-transform sign handling")
    ap.add_argument("--logEvery", type=int, default=64, help="LCU terms between log points")
    ap.add_argument("--tol", type=float, default=1e-6, help="res_dir convergence threshold")
    ap.add_argument("--outdir", default=".", help="output directory")
    ap.add_argument("--noChecks", action="store_true", help="skip the NaN / normalisation checks inside T")
    ap.add_argument("--maxTerms", type=int, default=0, help="stop after this many LCU terms (0: no cap)")
    return ap


def main(argv=None) -> int:
    run(parser().parse_args(argv))
    return 0


if __name__ == "__main__":
    sys.exit(main())
