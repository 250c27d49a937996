"""bench.py — sparse-entry updates/s of the register circuit at scale on one GB300.

Workload ("register circuit at scale", a 20-bit, b 32-bit, c 32-bit plus a
32-bit scratch t): from |0>, L = 10 layers of
    Hadamard_Int(a, h=12)                         # split: 4096 -> 2^24 entries (merge on layers >= 2)
    QRAMLoad(T, a, b)                             # b ^= T[a], T = 2^20 seeded uniform uint32 words
    Mul_UInt_UInt(a, b, t); Add_UInt_UInt_InPlace(t, c); Mul_UInt_UInt(a, b, t)   # c += a*b mod 2^32
    Phase_Bool(c, 0, theta_l)                     # theta_l seeded uniform in [0, 2*pi)
    Hadamard_Int(a, h=12)                         # split: fan-out to the 2^24-entry peak
The five elementwise operators of a layer run as one fused launch. One step
is the whole circuit from |0>. `updates` = sum over operator applications of
max(N_in, N_out) (elementwise operators count N each).

Arms: default = the GB300 engine; `--impl reference` = the CPU restatement of
the reference's operator path (the reference itself does not build here)
on the host cores, one steady-state layer per step in P concurrent processes.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "sparse-entry updates/s (register circuit at scale)"
UNIT = "updates/s"
A_BITS, B_BITS, C_BITS, T_BITS = 20, 32, 32, 32
TABLE_BITS = 20
SEED = 20261203


def workload_config(h: int, layers: int) -> dict:
    return {
        "workload": (f"register circuit at scale: a{A_BITS}/b{B_BITS}/c{C_BITS} (+t{T_BITS} scratch), {layers} layers of "
                     f"[Hadamard_Int(a,{h}); b^=QRAM[a] (2^{TABLE_BITS}-word uint32 table); c+=a*b mod 2^32; "
                     f"phase exp(i*theta_l) on c bit 0; Hadamard_Int(a,{h})], peak 2^{2 * h} entries, complex128"),
        "hadamard_bits": h,
        "layers": layers,
        "peak_entries": 1 << (2 * h),
        "l2_policy": "inputs larger than L2: the 2^24-entry state is 0.54 GB (L2 129 MB), no flush needed",
        "seed": SEED,
    }


def circuit_inputs(h: int, layers: int):
    import numpy as np
    rng = np.random.default_rng(SEED)
    table = rng.integers(0, 1 << 32, 1 << TABLE_BITS, dtype=np.uint64)
    thetas = rng.uniform(0.0, 2 * math.pi, layers)
    return table, thetas


# ---------------------------------------------------------------------- GB300 arm
def sample_clocks_start(path: Path):
    q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "20"],
                             stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except Exception:
        return None, None


def sample_clocks_wait(path: Path, timeout_s: float = 3.0) -> None:
    """Wait until the sampler has written its first line (nvidia-smi start-up)."""
    t0 = time.time()
    while time.time() - t0 < timeout_s:
        try:
            if path.stat().st_size > 0:
                return
        except OSError:
            pass
        time.sleep(0.02)


def sample_clocks_stop(p, f, path: Path, device: int, window=None):
    """Median SM clock and the throttle reasons seen, over the samples taken
    inside `window` = (start, end) host times (all samples when None)."""
    import datetime
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    sm, mx, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in path.read_text().splitlines():
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 10 or not parts[1].isdigit() or int(parts[1]) != device:
            continue
        if window is not None:
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            if not window[0] <= ts <= window[1]:
                continue
        try:
            sm.append(float(parts[2]))
            mx = max(mx, float(parts[3]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[6:10]):
            if v.lower() == "active":
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
            "window": "timed region" if window is not None else "whole run"}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(kernel)
    except Exception:
        return None


def _canonical_rows(regs, amps):
    """Entries sorted by (a, b, c, t): two 64-bit sort words, a << 32 | b and
    c << 32 | t (a has 20 bits)."""
    import numpy as np
    k0 = (regs[:, 0] << np.uint64(32)) | regs[:, 1]
    k1 = (regs[:, 2] << np.uint64(32)) | regs[:, 3]
    order = np.lexsort((k1, k0))
    return k0[order], k1[order], amps[order]


def cpu_baseline_and_parity(ps, circ, layers_sample: int = 2):
    """The oracle (the CPU restatement of the reference path), one thread, on
    the first `layers_sample` layers of the same full-size circuit, timed;
    then the GPU engine over the same layers from |0>, in the headline
    (exact-sum) and in the reference butterfly arithmetic, compared with the
    oracle's state: keys bit-exact, amplitudes relative to the largest."""
    import numpy as np
    from oracle import oracle as O
    O.clear()
    for rid in ps.System.active_ids():
        O.add_register(int(ps.System.type_of(rid)), ps.System.size_of(rid))
    O.register_qram(circ.qram)
    ost = O.OracleState()
    t0 = time.perf_counter()
    upd = 0
    for layer in range(layers_sample):
        n0 = ost.size()
        O.apply(ost, circ.H.spec())
        n1 = ost.size()
        O.apply(ost, circ.mid[layer].spec())
        O.apply(ost, circ.H.spec())
        n2 = ost.size()
        upd += max(n0, n1) + 5 * n1 + max(n1, n2)
    dt = time.perf_counter() - t0
    ok0, ok1, oa = _canonical_rows(*ost.get())
    del ost
    O.clear()
    parity = {"layers": layers_sample, "entries": int(len(oa)), "oracle": "CPU restatement of the reference path"}
    scale = float(np.max(np.abs(oa))) if len(oa) else 1.0
    arith0 = ps.get_fwht_arithmetic()
    for arith in ("exact-sum", "reference"):
        ps.set_fwht_arithmetic(arith)
        st = ps.SparseState(capacity=max(len(oa), 1))
        circ.run(st, layers=layers_sample)
        gk0, gk1, ga = _canonical_rows(*st.download())
        del st
        same = len(ga) == len(oa) and bool(np.array_equal(gk0, ok0) and np.array_equal(gk1, ok1))
        err = float(np.max(np.abs(ga - oa))) / scale if same and len(oa) else None
        if arith == "exact-sum":
            parity.update(keys_equal=same, max_rel_amp_err=err, fwht_arithmetic=arith, tolerance=1e-12,
                          ok=bool(same and err is not None and err <= 1e-12))
        else:
            parity["reference_arithmetic"] = {
                "keys_equal": same,
                "amps_bit_exact": bool(same and np.array_equal(ga.view(np.float64), oa.view(np.float64)))}
    ps.set_fwht_arithmetic(arith0)
    return upd, dt, parity


def run_cks(args, ext) -> dict:
    """The reference's CKS benchmark (CKSPoiseuilleBench: A = tridiag(-1,
    2.2666666666564934, -1) quantised to 32 bits, b = ones / sqrt(n) with the
    parity phase D, least-squares 1/x coefficients with J = 640, kappa 16) at
    n = 2^cks_bits: FirstStep and one untimed LCU term, then `--cks-terms`
    terms timed, each two walk steps and the add_systems merge into the
    accumulator, device time with CUDA events."""
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native, cks
    n_bits, terms = args.cks_bits, args.cks_terms
    n = 1 << n_bits
    ps.System.clear()
    mat, spec = cks.make_tridiagonal_matrix_spec(2.2666666666564934, -1.0, n, 32)
    obj = cks.LCU_Container_NoiseFree_Tridiagonal(mat, spec, 16.0, 0.01)
    obj.set_inverse_coefficients(cks.ChebyshevInverseCoefficients(*cks.walk_spectrum(spec), 640))
    st = obj.step_state
    ps.Hadamard_Int(obj.GetInputVecReg(), n_bits)(st)
    cks.TridiagParityPhase(obj.GetInputVecReg())(st)
    ps.ClearZero()(st)
    t0 = time.perf_counter()
    obj.quantum_walk_obj.FirstStep(obj.run)
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    obj.Step()
    obj.Step()
    torch.cuda.synchronize()
    _native.profile_reset()
    _native.profile_enable(True)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    if args.cuda_profiler_range == "cks":
        torch.cuda.profiler.start()
    s.record(ext)
    for _ in range(terms):
        obj.Step()
    e.record(ext)
    e.synchronize()
    if args.cuda_profiler_range == "cks":
        torch.cuda.profiler.stop()
    wall = time.perf_counter() - t0
    _native.profile_enable(False)
    prof = _native.profile_read()
    ms = s.elapsed_time(e)
    tot = sum(v[1] for v in prof.values()) or 1.0
    kernels = {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:10]}
    out = {
        "workload": (f"CKS walk of the reference's CKSPoiseuilleBench: n=2^{n_bits}, tridiagonal 1D Poisson "
                     f"matrix quantised to 32 bits, least-squares 1/x coefficients (J=640), kappa 16; LCU terms "
                     f"2..{1 + terms} timed (two walk steps and one add_systems merge each)"),
        "terms_timed": terms, "entries_walk_state": st.size(), "entries_accumulator": obj.current_state.size(),
        "peak_walk_entries": obj.max_system_size, "first_step_s": first_s,
        "s_per_term": ms / terms / 1e3, "wall_s_per_term": wall / terms,
        "kernels": kernels, "kernel_s_per_term": tot / terms / 1e3, "roofline": leg_roofline(prof),
    }
    if n_bits == 20:
        out["reference_published"] = {"s_per_term": 4.2, "entries_after_first_step": 20971512,
                                      "hardware": "1x A800-SXM4-80GB",
                                      "source": "docs/verification/v1e-cks-direct-oracle-linsolver.md:116-118"}
        out["speedup_vs_published"] = 4.2 / (ms / terms / 1e3)
    return out


def run_cks_qram(args, ext) -> dict:
    """Config 5's CKS solve through the QRAM walk: an N = 2^cks_qram_bits
    symmetric banded matrix (half bandwidth 4, off-diagonals uniform in
    [-1, 1], the diagonal set for kappa ~ 100) as a SparseMatrix in QRAM
    (24-bit elements), least-squares 1/x coefficients of Chebyshev degree
    201 (J = 100) on the encoded matrix's Gershgorin interval, b uniform. The
    reference's T rotates by the element's magnitude (its angle ignores the
    sign), so the walk encodes |A|. Timed: `--cks-qram-terms` LCU terms after
    FirstStep and one term, plain, then with the size model trained on the
    split sizes logged by an untimed repeat of the same terms (learned); the
    two accumulators are compared (same entries, amplitudes within 1e-12)."""
    import numpy as np
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native, cks, cks_qram
    from sparqsim_gb300 import predictor as P
    n_bits, terms = args.cks_qram_bits, args.cks_qram_terms
    n = 1 << n_bits
    A = cks_qram.banded_symmetric(n, 4, 100.0, seed=SEED + n_bits)

    def solve(learned: bool, log: bool):
        ps.System.clear()
        mat = cks_qram.SparseMatrix(A, 24)
        # Gershgorin interval of the encoded matrix |A| / (max|A| nnz_col)
        absA_rows = np.asarray(abs(A).sum(axis=1)).ravel()
        diag = np.abs(A.diagonal())
        scale = mat.amax * mat.nnz_col
        lo = max(float(np.min(2 * diag - absA_rows)) / scale, 1e-3 / scale)
        hi = float(np.max(absA_rows)) / scale
        obj = cks_qram.LCU_Container_NoiseFree(mat, 100.0, 0.01, checks=False)
        obj.set_inverse_coefficients(cks.ChebyshevInverseCoefficients(lo, hi, 100))
        st = obj.step_state
        ps.Hadamard_Int(obj.GetInputVecReg(), n_bits)(st)
        ps.ClearZero()(st)
        P.log(log)  # the untimed first steps log their split sizes too
        t0 = time.perf_counter()
        obj.quantum_walk_obj.FirstStep(obj.run)
        obj.Step()
        obj.Step()
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        P.enable(learned)
        pred0 = P.stats()["predictions"]
        over0 = P.stats()["single_pass_overflows"]
        if not log:
            _native.profile_reset()
            _native.profile_enable(True)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(ext)
        for _ in range(terms):
            obj.Step()
        e.record(ext)
        e.synchronize()
        _native.profile_enable(False)
        P.log(False)
        P.enable(False)
        st_ = P.stats()
        return (obj, mat, s.elapsed_time(e), setup_s, _native.profile_read(),
                st_["predictions"] - pred0, st_["single_pass_overflows"] - over0)

    obj, mat, ms, setup_s, prof, _, _ = solve(False, False)
    plain_r, plain_a = obj.current_state.download()
    peak = obj.max_system_size
    walk_entries = obj.step_state.size()
    del obj
    P.clear_log()
    solve(False, True)  # logs the split sizes of the same terms
    x_log, t_log = P.read_log()
    learned = None
    if x_log.shape[0] >= 8:
        P.reset(seed=31)
        loss = P.train(x_log, t_log, epochs=200, batch=64, lr=2e-3, seed=32)
        obj2, _, lms, _, _, preds, overs = solve(True, False)
        lr, la = obj2.current_state.download()
        same = len(la) == len(plain_a)
        diff = None
        if same:
            o1, o2 = np.lexsort(plain_r.T[::-1]), np.lexsort(lr.T[::-1])
            same = bool(np.array_equal(plain_r[o1], lr[o2]))
            if same:
                diff = float(np.max(np.abs(plain_a[o1] - la[o2])) / max(np.max(np.abs(plain_a)), 1e-300))
        learned = {"s_per_term": lms / terms / 1e3, "training_rows": int(x_log.shape[0]), "final_loss": loss,
                   "predictions": preds, "overflows": overs, "same_entries_as_plain": same,
                   "max_rel_amp_diff_vs_plain": diff}
        del obj2
    tot = sum(v[1] for v in prof.values()) or 1.0
    kernels = {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:10]}
    return {
        "workload": (f"CKS through the QRAM walk: N=2^{n_bits} symmetric banded matrix (half bandwidth 4, "
                     "off-diagonals U[-1,1], kappa ~100) as a SparseMatrix in QRAM (24-bit elements, "
                     f"nnz_col {mat.nnz_col}), least-squares 1/x coefficients of degree 201 (J=100); LCU terms "
                     f"3..{2 + terms} timed (two walk steps and one add_systems merge each)"),
        "terms_timed": terms, "s_per_term": ms / terms / 1e3, "projected_degree_201_solve_s": ms / terms / 1e3 * 101,
        "setup_s": setup_s, "entries_walk_state": walk_entries, "peak_walk_entries": peak,
        "key_words": ps.System.key_words(), "kernels": kernels, "kernel_s_per_term": tot / terms / 1e3,
        "roofline": leg_roofline(prof), "learned": learned,
        "note": "the reference's QRAM T rotates by the element's magnitude (GetQWRotateAngle_Int_Int_Int "
                "then CondRot_Fixed_Bool), so a signed matrix is walked as |A|",
    }


def leg_roofline(prof: dict) -> dict:
    """The kernel with the largest device time in a leg's profile: its
    algorithmic bytes per launch over its event-timed duration, against the
    measured HBM copy peak."""
    dom = max(prof, key=lambda k_: prof[k_][1])
    n_l, d_ms, d_bytes = prof[dom]
    peak, kind = measured_peak_hbm()
    achieved = d_bytes / (d_ms / 1e3) / 1e9 if d_ms > 0 else 0.0
    return {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": kind, "traffic": ncu_traffic(dom),
            "alg_bytes_per_launch": d_bytes / max(n_l, 1), "avg_launch_ms": d_ms / max(n_l, 1)}


def replica_max(ms: float, device: str) -> float:
    """The slowest replica's time: all-reduce MAX over the ranks, then a barrier
    (independent circuits per GPU, no exchange on the data path)."""
    import torch
    import torch.distributed as dist
    tt = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(tt.item())


def replica_value(world: int, updates_per_step: int, steps: int, t_max_ms: float) -> float:
    """Whole-job updates/s: every replica runs the same circuit, timed by the slowest."""
    return world * updates_per_step * steps / (t_max_ms / 1e3)


def run_trajectories(args, ext) -> dict:
    """Batched noisy trajectories (4096 instances, a/b/c 16-bit, per-instance
    Hadamard width h_t in [4, 8], Pauli X/Z at p = 1e-3 per bit per layer,
    6 layers): the batched form, the plain GPU form (one state per instance)
    on a sample of instances, and the oracle on a smaller sample."""
    import numpy as np
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300.workloads import NoisyTrajectories
    wl = NoisyTrajectories(n_traj=args.trajectories, layers=6, p=1e-3, h_min=4, h_max=8, seed=SEED)
    wl.build_batched()
    st = ps.SparseState(capacity=1 << 20)
    from sparqsim_gb300 import predictor as P
    P.log(True)  # untimed runs: their split sizes join the size model's training log
    upd = wl.run_batched(st, count=True)
    peak_hint = st.size()
    for _ in range(2):
        wl.run_batched(st)
    P.log(False)
    steps = max(2, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(ext)
    for _ in range(steps):
        wl.run_batched(st)
    e.record(ext)
    e.synchronize()
    batched_ms = s.elapsed_time(e) / steps
    batched_wall = (time.perf_counter() - t0) / steps
    # per-kernel device time of one more batched run (CUDA events on the library stream)
    from sparqsim_gb300 import _native
    _native.profile_reset()
    _native.profile_enable(True)
    wl.run_batched(st)
    _native.profile_enable(False)
    tprof = _native.profile_read()
    ttot = sum(v[1] for v in tprof.values()) or 1.0
    traj_kernels = {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / ttot, 4),
                        "alg_GBps": round(v[2] / (v[1] / 1e3) / 1e9, 1) if v[1] > 0 else 0}
                    for k, v in sorted(tprof.items(), key=lambda kv: -kv[1][1])[:8]}
    eager_n, eager_norm = st.size(), st.norm_sq()
    # batched + learned: the size model, trained on the split sizes logged so
    # far in this run (register circuit and these trajectories), sizes the
    # hash tables and single passes of the same batched runs
    learned = None
    x_log, t_log = P.read_log()
    if x_log.shape[0] >= 16:
        P.reset(seed=11)
        loss = P.train(x_log, t_log, epochs=200, batch=64, lr=2e-3, seed=12)
        P.enable(True)
        pred0, over0 = P.stats()["predictions"], P.stats()["single_pass_overflows"]
        wl.run_batched(st)
        torch.cuda.synchronize()
        s.record(ext)
        for _ in range(steps):
            wl.run_batched(st)
        e.record(ext)
        e.synchronize()
        learned_ms = s.elapsed_time(e) / steps
        same = st.size() == eager_n and abs(st.norm_sq() - eager_norm) <= 1e-12 * eager_norm
        st_ = P.stats()
        P.enable(False)
        learned = {"value": upd / (learned_ms / 1e3), "unit": UNIT, "ms_per_step": learned_ms,
                   "training_rows": int(x_log.shape[0]), "final_loss": loss,
                   "predictions": st_["predictions"] - pred0, "overflows": st_["single_pass_overflows"] - over0,
                   "same_size_and_norm_as_without": same,
                   "note": "the size model trained on the split sizes logged earlier in this run, enabled for "
                           "the same batched runs; results are identical with it on or off"}
    # the same batched circuit replayed as one CUDA graph per run (one
    # recording pass, one capture; each run is the upload and one launch)
    init = wl.initial_batched()
    graph = ps.Graph(st, apply=lambda: wl.run_batched(st, upload=False), prepare=lambda: st.upload(*init))
    graph.replay()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.record(ext)
    for _ in range(steps):
        graph.replay()
    e.record(ext)
    e.synchronize()
    ps.synchronize()  # reports a replay whose sizes differed from the recording
    graph_ms = s.elapsed_time(e) / steps
    graph_wall = (time.perf_counter() - t0) / steps
    graph_same = st.size() == eager_n and abs(st.norm_sq() - eager_norm) <= 1e-12 * eager_norm
    del graph
    # plain GPU form: instance by instance, on a sample of instances
    n_sample = min(args.plain_sample, wl.n_traj)
    wl.build_plain()
    sp = ps.SparseState(capacity=1 << 17)
    upd_p = sum(wl.run_plain(sp, t, count=True) for t in range(n_sample))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.record(ext)
    for t in range(n_sample):
        wl.run_plain(sp, t)
    e.record(ext)
    e.synchronize()
    plain_s = time.perf_counter() - t0
    plain_ev_s = s.elapsed_time(e) / 1e3
    # the oracle, one thread, plain form, on a smaller sample
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.clear()
        for rid in ps.System.active_ids():
            O.add_register(int(ps.System.type_of(rid)), ps.System.size_of(rid))
        _, qram, noise, mids, Hs = wl._built
        O.register_qram(qram)
        for nt in noise:
            O.register_qram(nt.table)
        n_cpu = min(args.cpu_sample, wl.n_traj)
        upd_c = 0
        t0 = time.perf_counter()
        for t in range(n_cpu):
            ost = O.OracleState()
            ost.set(np.array([[t, 0, 0, 0]], dtype=np.uint64), np.ones(1, dtype=np.complex128))
            H = Hs[int(wl.widths[t])]
            for mid in mids:
                n0 = ost.size()
                O.apply(ost, H.spec())
                n1 = ost.size()
                O.apply(ost, mid.spec())
                O.apply(ost, H.spec())
                upd_c += max(n0, n1) + 4 * n1 + max(n1, ost.size())
        cpu_s = time.perf_counter() - t0
        O.clear()
        cpu = {"value": upd_c / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"instances 0..{n_cpu - 1}, plain form, {upd_c} updates in {cpu_s:.1f} s, one thread"}
    batched_ups = upd / (batched_ms / 1e3)
    plain_ups = upd_p / plain_ev_s
    out = {
        "workload": (f"{wl.n_traj} noisy instances of the register circuit (a/b/c 16-bit, 2^16-word uint16 table), "
                     "Hadamard width h_t in [4,8] per instance, Pauli X/Z p=1e-3 per bit per layer, 6 layers, "
                     "support 2^h..2^2h per instance"),
        "updates_per_step": upd, "peak_entries": peak_hint,
        "batched": {"value": batched_ups, "unit": UNIT, "ms_per_step": batched_ms,
                    "wall_ms_per_step": batched_wall * 1e3},
        "batched_graph": {"value": upd / (graph_ms / 1e3), "unit": UNIT, "ms_per_step": graph_ms,
                          "wall_ms_per_step": graph_wall * 1e3, "same_size_and_norm_as_eager": graph_same,
                          "note": "the batched circuit recorded once and replayed as one CUDA graph launch per run; "
                                  "each run uploads the initial state first"},
        "plain_gpu": {"value": plain_ups, "unit": UNIT, "wall_value": upd_p / plain_s,
                      "sample": f"instances 0..{n_sample - 1}, {upd_p} updates in {plain_ev_s:.3f} s between CUDA "
                                f"events on the library stream ({plain_s:.3f} s wall clock); one state per instance, "
                                f"so each split's count read-back sits between the launches, as in any unbatched driver"},
        "kernels": traj_kernels,
        "batched_over_plain": batched_ups / plain_ups,
        "fwht_arithmetic": ps.get_fwht_arithmetic(),
    }
    if learned:
        out["batched_learned"] = learned
    if cpu:
        out["cpu"] = cpu
        out["batched_over_cpu"] = batched_ups / cpu["value"]
    best = max(batched_ups, learned["value"] if learned else 0.0)
    out["target"] = {"batched_learned_over_plain": best / plain_ups,
                     "batched_learned_over_cpu": best / cpu["value"] if cpu else None,
                     "goal": ">= 5x plain GPU, >= 20x the stated-core CPU"}
    return out


def run_qda(args, ext) -> dict:
    """The reference's QDA walk benchmark (PoiseuilleQDABench: the 1D Poisson
    matrix A = tridiag(beta, alpha, beta) with alpha = 2.2666666666564934,
    beta = -1, kappa = 16, b = ones / sqrt(n), p = 1.3, a step budget of
    ceil(1.1 * 2305 * 16) = 40568, clearzero eps 1e-14) at n = 2^qda_bits:
    `--qda-steps` walk steps of that schedule timed after `--qda-warm` (at least
    2) untimed ones, each followed by ClearZero and Normalize as there, and
    counted (sizes per operator, peak entries) in a separate untimed pass."""
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native, qda
    n_bits = args.qda_bits
    alpha, beta, kappa, p = 2.2666666666564934, -1.0, 16.0, 1.3
    total_steps, sample, warm = 40568, args.qda_steps, max(2, args.qda_warm)

    class Counting(qda.Runner):
        """Counts entries read or written per operator (max of the sizes
        before and after) and the peak entry count, the reference's
        System::max_system_size."""

        def __init__(self, state, count):
            super().__init__(state)
            self.count, self.updates, self.peak, self.sizes = count, 0, 0, []

        def op(self, o, dag=False):
            n0 = self.state.size() if self.count else 0
            super().op(o, dag)
            if self.count:
                n1 = self.state.size()
                self.updates += max(n0, n1)
                self.peak = max(self.peak, n0, n1)

    def walk(count, profile=False, bracket=False):
        ps.System.clear()
        ps.set_clearzero_default_eps(1e-14)  # the walk's own ClearZero calls use the bench's threshold
        run = Counting(ps.SparseState(capacity=1 << 22), False)
        qda.declare_registers(run, n_bits)
        run.op(ps.Hadamard_Int_Full("main_reg"))
        enc_A = qda.BlockEncodingTridiagonal("main_reg", "anc_UA", alpha, beta)
        enc_b = qda.StatePrepHadamard("main_reg")

        def step(n):
            qda.WalkS(enc_A, enc_b, *qda.REGS, n / total_steps, kappa, p).apply(run)
            run.op(ps.ClearZero(1e-14))
            run.op(ps.Normalize())
            if run.count:
                run.sizes.append(run.state.size())

        run.count = count
        for n in range(warm):
            step(n)
        run.updates = 0  # the timed steps' updates only; peak and sizes cover the whole walk
        torch.cuda.synchronize()
        if profile:
            _native.profile_reset()
            _native.profile_enable(True)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        if bracket:
            torch.cuda.profiler.start()
        s.record(ext)
        for n in range(warm, warm + sample):
            step(n)
        e.record(ext)
        e.synchronize()
        if bracket:
            torch.cuda.profiler.stop()
        if profile:
            _native.profile_enable(False)
        return run, s.elapsed_time(e), time.perf_counter() - t0

    counted, _, _ = walk(True)
    run, ms, wall = walk(False, bracket=args.cuda_profiler_range == "qda")
    walk(False, profile=True)  # per-kernel device time of the timed steps
    prof = _native.profile_read()
    tot = sum(v[1] for v in prof.values()) or 1.0
    kernels = {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:12]}
    ref_s_per_step = {16: 0.24, 20: 1.33}.get(n_bits)
    out = {
        "workload": (f"QDA walk of the reference's PoiseuilleQDABench: n=2^{n_bits}, A = tridiag(-1, "
                     f"{alpha}, -1) (kappa 16), b uniform, p={p}, schedule of {total_steps} steps; "
                     f"steps {warm}..{warm + sample - 1} timed"),
        "steps_timed": sample, "entries": run.state.size(), "peak_entries": counted.peak,
        "entries_after_each_step": counted.sizes,
        "updates": counted.updates, "value": counted.updates / (ms / 1e3), "unit": UNIT,
        "ms_per_walk_step": ms / sample, "wall_ms_per_walk_step": wall * 1e3 / sample,
        "projected_full_budget_s": ms / sample * total_steps / 1e3,
        "kernels": kernels, "kernel_ms_per_walk_step": tot / sample, "roofline": leg_roofline(prof),
    }
    if ref_s_per_step:
        out["reference_published"] = {"s_per_walk_step": ref_s_per_step, "hardware": "1x A800-SXM4-80GB",
                                      "source": "docs/verification/v1d-qda-linsolver-a800.md:48-52"}
        out["speedup_vs_published"] = ref_s_per_step / (ms / sample / 1e3)
    return out


def oracle_timed_runner():
    """A runner that applies each operator to a GPU state (which keeps the
    register table) and to an oracle state, timing only the oracle's calls;
    `updates` counts entries per operator as the GPU legs do (a fused
    program counts each of its operators)."""
    import sparqsim_gb300 as ps
    from oracle import oracle as O
    from sparqsim_gb300.qda import Runner

    class OracleTimed(Runner):
        def __init__(self, state, ost):
            super().__init__(state)
            self.ost, self.t, self.updates = ost, 0.0, 0

        def op(self, o, dag=False):
            (o.dag if dag else o)(self.state)
            n0 = self.ost.size()
            t0 = time.perf_counter()
            O.apply(self.ost, o.spec(dag and not o.self_adjoint))
            self.t += time.perf_counter() - t0
            self.updates += (len(o.items) if hasattr(o, "items") else 1) * max(n0, self.ost.size())

        def split(self, first, name, size):
            rid = super().split(first, name, size)
            f = ps.System.resolve(first)
            assert O.split_register(self.ost, f, size) == rid
            return rid

        def combine(self, first, second):
            f, s2 = ps.System.resolve(first), ps.System.resolve(second)
            super().combine(first, second)
            O.combine_register(self.ost, f, s2)

        def add_register(self, name, type_, size):
            rid = super().add_register(name, type_, size)
            assert O.add_register_sync(self.ost, int(type_), size) == rid
            return rid

        def remove_register(self, reg):
            rid = ps.System.resolve(reg)
            super().remove_register(reg)
            O.remove_register_sync(self.ost, rid)

    return OracleTimed


def run_qda_batched(args, ext) -> dict:
    """B walks of the PoiseuilleQDABench system (n = 2^qda_bits) with step
    budgets 40568 + 2000 t, t < B, side by side in one state (a log2 B-bit
    instance register in uniform superposition; each walk's R_s by
    CondRot_General_Bool on it; ClearZero at 1e-14 / B, where each walk's
    |a|^2 is 1/B of its own), against the plain form: the walk of the last
    budget alone in its own state, over the same steps. Steps
    `--qda-warm`..+`--qda-steps` timed with CUDA events in both, updates
    counted in separate untimed passes; the last walk of the batch is checked
    against the plain walk (same basis entries, amplitudes times sqrt B).
    The oracle times walk steps 0 and 1 of the plain walk on one host core."""
    import numpy as np
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native, qda
    B, n_bits = args.qda_batch, args.qda_bits
    alpha, kappa, p = 2.2666666666564934, 16.0, 1.3
    budgets = [40568 + 2000 * t for t in range(B)]
    warm, k = max(2, args.qda_warm), args.qda_steps
    inst_bits = max(1, (B - 1).bit_length())
    if B != 1 << inst_bits:
        raise ValueError("--qda-batch: a power of two (>= 2)")

    class Counting(qda.Runner):
        def __init__(self, state):
            super().__init__(state)
            self.count, self.updates, self.peak = False, 0, 0

        def op(self, o, dag=False):
            n0 = self.state.size() if self.count else 0
            super().op(o, dag)
            if self.count:
                n1 = self.state.size()
                self.updates += max(n0, n1)
                self.peak = max(self.peak, n0, n1)

    def walk(batched, count, profile=False):
        ps.System.clear()
        nb = len(budgets) if batched else 1
        eps = 1e-14 / nb
        ps.set_clearzero_default_eps(eps)
        st = ps.SparseState(capacity=1 << 22)
        run = Counting(st)
        qda.declare_registers(run, n_bits)
        if batched:
            run.add_register("inst", ps.UnsignedInteger, inst_bits)
            run.op(ps.Hadamard_Int_Full("inst"))
        run.op(ps.Hadamard_Int_Full("main_reg"))
        enc_A = qda.BlockEncodingTridiagonal("main_reg", "anc_UA", alpha, -1.0)
        enc_b = qda.StatePrepHadamard("main_reg")

        def step(n):
            s = [n / b for b in budgets] if batched else n / budgets[-1]
            qda.WalkS(enc_A, enc_b, *qda.REGS, s, kappa, p, inst_reg="inst" if batched else None).apply(run)
            run.op(ps.ClearZero(eps))
            run.op(ps.Normalize())

        for n in range(warm):
            step(n)
        run.count = count
        torch.cuda.synchronize()
        if profile:
            _native.profile_reset()
            _native.profile_enable(True)
        ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev[0].record(ext)
        for n in range(warm, warm + k):
            step(n)
        ev[1].record(ext)
        ev[1].synchronize()
        if profile:
            _native.profile_enable(False)
        ps.set_clearzero_default_eps(1e-14)
        return st, run, ev[0].elapsed_time(ev[1])

    _, plain_c, _ = walk(False, True)
    sp, _, plain_ms = walk(False, False)
    from sparqsim_gb300 import predictor as P
    P.clear_log()
    P.log(True)  # the counted pass (untimed) logs its split sizes for the size model
    _, batch_c, _ = walk(True, True)
    P.log(False)
    walk(True, False, profile=True)  # per-kernel device time of the batched steps
    prof = _native.profile_read()
    tot = sum(v[1] for v in prof.values()) or 1.0
    batch_kernels = {kk: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4)}
                     for kk, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:12]}
    sb, _, batch_ms = walk(True, False)
    # batched + learned: the size model trained on those sizes sizes the same
    # batched walk's splits (results identical with it on or off)
    learned = None
    x_log, t_log = P.read_log()
    if x_log.shape[0] >= 16:
        P.reset(seed=21)
        loss = P.train(x_log, t_log, epochs=200, batch=64, lr=2e-3, seed=22)
        P.enable(True)
        pred0, over0 = P.stats()["predictions"], P.stats()["single_pass_overflows"]
        sl, _, learned_ms = walk(True, False)
        st_ = P.stats()
        P.enable(False)
        same = sl.size() == sb.size() and abs(sl.norm_sq() - sb.norm_sq()) <= 1e-12 * sb.norm_sq()
        del sl
        learned = {"value": batch_c.updates / (learned_ms / 1e3), "unit": UNIT, "ms_per_walk_step": learned_ms / k,
                   "training_rows": int(x_log.shape[0]), "final_loss": loss,
                   "predictions": st_["predictions"] - pred0,
                   "overflows": st_["single_pass_overflows"] - over0, "same_size_and_norm_as_without": same}
    pr, pa = sp.download()
    br, ba = sb.download()
    ncol = len(qda.REGS)
    sel = br[:, ncol] == B - 1
    br, ba = br[sel][:, :ncol], ba[sel] * math.sqrt(B)
    pr = pr[:, :ncol]
    same_keys = len(pr) == len(br)
    diff = None
    if same_keys:
        o1, o2 = np.lexsort(pr.T[::-1]), np.lexsort(br.T[::-1])
        same_keys = bool(np.array_equal(pr[o1], br[o2]))
        if same_keys:
            diff = float(np.max(np.abs(pa[o1] - ba[o2])))
    plain_ups = plain_c.updates / (plain_ms / 1e3)
    batch_ups = batch_c.updates / (batch_ms / 1e3)
    out = {
        "workload": (f"{B} QDA walks of the PoiseuilleQDABench system at n=2^{n_bits} (kappa 16, p={p}) with "
                     f"step budgets {budgets[0]}..{budgets[-1]} (+2000 each) in one state, told apart by a "
                     f"{inst_bits}-bit instance register; steps {warm}..{warm + k - 1} of each timed"),
        "batched": {"value": batch_ups, "unit": UNIT, "updates": batch_c.updates, "ms_per_walk_step": batch_ms / k,
                    "peak_entries": batch_c.peak, "entries": sb.size(), "kernels": batch_kernels,
                    "kernel_ms_per_walk_step": tot / k, "roofline": leg_roofline(prof)},
        "plain_gpu": {"value": plain_ups, "unit": UNIT, "updates": plain_c.updates, "ms_per_walk_step": plain_ms / k,
                      "peak_entries": plain_c.peak, "entries": sp.size(),
                      "sample": f"the walk of budget {budgets[-1]} alone in its own state, the same steps, "
                                "CUDA events on the library stream"},
        "batched_learned": learned,
        "batched_over_plain": batch_ups / plain_ups,
        "batched_s_per_walk_step_per_walk": batch_ms / k / B / 1e3,
        "last_walk_vs_plain": {"same_basis_entries": same_keys, "max_abs_amp_diff": diff,
                               "note": "the batch's last walk (amplitudes times sqrt B) against the plain walk of "
                                       "the same budget after the timed steps"},
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        OracleTimed = oracle_timed_runner()
        ps.System.clear()
        O.clear()
        st = ps.SparseState(capacity=1 << 22)
        run = OracleTimed(st, O.OracleState())
        qda.declare_registers(run, n_bits)
        for rid in ps.System.active_ids():
            assert O.add_register_sync(run.ost, int(ps.System.type_of(rid)), ps.System.size_of(rid)) == rid
        run.op(ps.Hadamard_Int_Full("main_reg"))
        enc_A = qda.BlockEncodingTridiagonal("main_reg", "anc_UA", alpha, -1.0)
        enc_b = qda.StatePrepHadamard("main_reg")
        run.t, run.updates = 0.0, 0
        for n in range(2):
            qda.WalkS(enc_A, enc_b, *qda.REGS, n / budgets[-1], kappa, p).apply(run)
            run.op(ps.ClearZero(1e-14))
            run.op(ps.Normalize())
        O.clear()
        cpu = {"value": run.updates / run.t, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"walk steps 0 and 1 at n=2^{n_bits} ({run.updates} updates in {run.t:.2f} s), one thread"}
        out["cpu"] = cpu
    best = max(batch_ups, learned["value"] if learned else 0.0)
    out["target"] = {"batched_learned_over_plain": best / plain_ups,
                     "batched_learned_over_cpu": best / out["cpu"]["value"] if "cpu" in out else None,
                     "goal": ">= 5x plain GPU, >= 20x the stated-core CPU"}
    return out


def run_qda_config3(args, ext) -> dict:
    """The QDA solve of the banded system through the QRAM encodings: A =
    N x N symmetric, half bandwidth 4 (bandwidth 8), off-diagonals uniform in
    [-1, 1], the diagonal set for lambda_max / lambda_min = 50; b standard
    normal, normalised; A through Block_Encoding_via_QRAM (U_L, U_R on its
    quantised column tree), b through State_Prep_via_QRAM; a schedule of 2000
    walk steps. Timed: `--qda3-steps` steps at n = `--qda3-bits` after two
    untimed ones (device time, CUDA events), projected to the 2000-step
    solve; solved: all 2000 steps at n = `--qda3-solve-bits`, fidelity
    against the FP64 solve. The oracle times one walk step at the solved
    size on one host core."""
    import numpy as np
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native
    from sparqsim_gb300 import qram_encoding as Q
    from sparqsim_gb300.qda import Runner
    total = 2000

    class Counting(Runner):
        def __init__(self, state):
            super().__init__(state)
            self.count, self.updates, self.peak, self.ops, self.launches = False, 0, 0, 0, 0

        def op(self, o, dag=False):
            n0 = self.state.size() if self.count else 0
            super().op(o, dag)
            k = len(o.items) if hasattr(o, "items") else 1  # a fused program counts its operators
            self.ops += k
            self.launches += 1
            if self.count:
                n1 = self.state.size()
                self.updates += k * max(n0, n1)
                self.peak = max(self.peak, n0, n1)

    def problem(n_bits):
        rng = np.random.default_rng(SEED + n_bits)
        A = Q.banded_spd(1 << n_bits, 4, 50.0, seed=SEED + n_bits)
        return Q.QDAviaQRAM(A, rng.normal(size=1 << n_bits))

    # timed steps at the larger size
    n = args.qda3_bits
    solver = problem(n)
    ps.System.clear()
    st = ps.SparseState(capacity=1 << 22)
    run = Counting(st)
    solver.start(run)
    for i in range(2):
        solver.step(run, i, total)
    run.count = True
    k = args.qda3_steps
    for i in range(2, 2 + k):  # counted pass (sizes), untimed
        solver.step(run, i, total)
    ups, peak = run.updates, run.peak
    run.count = False
    ps.System.clear()
    st = ps.SparseState(capacity=1 << 22)
    run = Counting(st)
    solver.start(run)
    for i in range(2):
        solver.step(run, i, total)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _native.profile_reset()
    _native.profile_enable(True)
    t0 = time.perf_counter()
    s.record(ext)
    ops0, launches0 = run.ops, run.launches
    for i in range(2, 2 + k):
        solver.step(run, i, total)
    e.record(ext)
    e.synchronize()
    wall = time.perf_counter() - t0
    _native.profile_enable(False)
    prof = _native.profile_read()
    ms = s.elapsed_time(e) / k
    tot = sum(v[1] for v in prof.values()) or 1.0
    kernels = {kk: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4)}
               for kk, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:10]}
    out = {
        "workload": (f"QDA via QRAM: N=2^{n} banded SPD (half bandwidth 4, off-diagonals U[-1,1], kappa(A) 50), "
                     "b ~ N(0,1); A by Block_Encoding_via_QRAM, b by State_Prep_via_QRAM (exponent 20, data 50 "
                     f"bits, rational 51 bits); walk steps 2..{1 + k} of a 2000-step schedule timed"),
        "n_bits": n, "kappa_matrix": solver.kappa_matrix, "kappa_walk": solver.kappa,
        "ms_per_walk_step": ms, "wall_ms_per_walk_step": wall * 1e3 / k, "operators_per_walk_step": (run.ops - ops0) / k,
        "operator_calls_per_walk_step": (run.launches - launches0) / k,
        "projected_solve_s": ms * total / 1e3, "updates": ups, "value": ups / (ms * k / 1e3), "unit": UNIT,
        "peak_entries": peak, "entries": st.size(), "kernels": kernels, "roofline": leg_roofline(prof),
    }
    # the whole 2000-step solve at the smaller size: fidelity
    ns = args.qda3_solve_bits
    solver = problem(ns)
    ps.System.clear()
    st = ps.SparseState()
    run = Runner(st)
    solver.start(run)
    torch.cuda.synchronize()
    s.record(ext)
    t0 = time.perf_counter()
    for i in range(total):
        solver.step(run, i, total)
    e.record(ext)
    e.synchronize()
    solve_wall = time.perf_counter() - t0
    x, prob, fid = solver.read_out(st)
    out["solve"] = {"n_bits": ns, "steps": total, "s": s.elapsed_time(e) / 1e3, "wall_s": solve_wall,
                    "fidelity_vs_fp64_solve": fid, "success_probability": prob, "kappa_walk": solver.kappa,
                    "kappa_matrix": solver.kappa_matrix}
    # the oracle: the state preparation and the first walk steps at N =
    # 2^qda3_cpu_bits (the GPU runs beside it to keep the register table;
    # only the oracle's calls are timed)
    if not args.no_cpu_baseline:
        from oracle import oracle as O

        OracleTimed = oracle_timed_runner()
        nc = args.qda3_cpu_bits
        solver = problem(nc)
        ps.System.clear()
        O.clear()
        O.register_qram(solver.tree_A.qram)
        O.register_qram(solver.tree_b.qram)
        st = ps.SparseState()
        run = OracleTimed(st, O.OracleState())
        solver.start(run)
        steps = 0
        while run.t < 10.0 and steps < 400:  # about 10 s of oracle time
            solver.step(run, steps, total)
            steps += 1
        out["cpu_baseline"] = {"value": run.updates / run.t, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"state preparation and walk steps 0-{steps - 1} at N=2^{nc} "
                                         f"({run.updates} updates in {run.t:.2f} s), one thread"}
        O.clear()
    return out


def run_gb300(args, rank: int, world: int, local_rank: int):
    import numpy as np
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native

    torch.cuda.set_device(local_rank)
    _native.call("sq_init", local_rank)
    ps.set_fwht_arithmetic(args.fwht_arithmetic)
    ps.set_group_strategy(args.group_strategy)
    h, L = args.hadamard_bits, args.layers
    from sparqsim_gb300.workloads import RegisterCircuit
    circ = RegisterCircuit(h, L, seed=SEED).build()
    table = circ.table
    st = ps.SparseState(capacity=1 << (2 * h))
    sp = ctypes_void_p()
    _native.call("sq_get_stream", __import__("ctypes").byref(sp))
    ext = torch.cuda.ExternalStream(sp.value)

    # the split sizes of every leg are logged for the size model (host memory)
    from sparqsim_gb300 import predictor as P
    P.clear_log()
    P.log(True)
    # untimed: count updates (deterministic), warm up
    updates = circ.run(st, count=True)
    final_n = st.size()
    for _ in range(max(args.warmup - 1, 0)):
        circ.run(st)
    P.log(False)  # logging computes key sketches: never inside a timed region
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()

    # raw samples in a scratch file; their summary goes into the JSON line
    clocks_path = Path(tempfile.gettempdir()) / f"sparqsim_clocks_rank{rank}_{os.getpid()}.csv"
    cp, cf = sample_clocks_start(clocks_path) if rank == 0 else (None, None)
    if cp is not None:
        sample_clocks_wait(clocks_path)
    launches0 = ps.launch_count()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.time()
    start.record(ext)
    for _ in range(args.steps):
        circ.run(st)
    end.record(ext)
    end.synchronize()
    torch.cuda.synchronize()
    eager_ms = start.elapsed_time(end)
    # the same steps, each replayed as one CUDA graph launch (the circuit is
    # recorded once and captured once; a replay re-runs every kernel with no
    # host round trip between them, and its counts are checked on the device)
    graph = ps.Graph(st, apply=lambda: circ.run(st, reset=False), prepare=st.reset)
    graph.replay()
    torch.cuda.synchronize()
    launches0 = ps.launch_count()
    start.record(ext)
    for _ in range(args.steps):
        graph.replay()
    end.record(ext)
    end.synchronize()
    ps.synchronize()  # a replay whose counts differed from the recording is reported here
    w1 = time.time()
    ms = start.elapsed_time(end)
    launches = ps.launch_count() - launches0
    clocks = sample_clocks_stop(cp, cf, clocks_path, local_rank, (w0, w1)) if rank == 0 else None
    graph_same = st.size() == final_n
    del graph

    t_max, t_eager = ms, eager_ms
    if world > 1:
        t_max = replica_max(ms, "cuda")
        t_eager = replica_max(eager_ms, "cuda")
    ms_per_step = t_max / args.steps
    value = replica_value(world, updates, args.steps, t_max)
    eager = {"value": replica_value(world, updates, args.steps, t_eager), "unit": UNIT,
             "ms_per_step": t_eager / args.steps,
             "note": "the same steps issued operator by operator (host reads of the split sizes between them)"}

    # the same steps in the other butterfly arithmetic (same keys; amplitudes
    # bit-identical to the reference in 'reference', within 1e-12 in 'exact-sum')
    other = "reference" if args.fwht_arithmetic == "exact-sum" else "exact-sum"
    other_ms = None
    if not args.skip_other_arithmetic:
        ps.set_fwht_arithmetic(other)
        circ.run(st)
        torch.cuda.synchronize()
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        other_steps = max(1, min(args.steps, 20))
        s2.record(ext)
        for _ in range(other_steps):
            circ.run(st)
        e2.record(ext)
        e2.synchronize()
        other_ms = s2.elapsed_time(e2) / other_steps
        ps.set_fwht_arithmetic(args.fwht_arithmetic)

    # end to end through the public API: every step uploads its inputs (the
    # QRAM table and the initial state) from pinned host memory and downloads
    # its final state into pinned host memory. Two states and two host buffers
    # alternate, so that a step's download (host link, about 190 GB/s here)
    # overlaps the next step's circuit; the clock stops when the last download
    # has landed.
    k = ps.System.key_words()
    host_keys = [torch.empty(final_n * k, dtype=torch.int64, pin_memory=True) for _ in range(2)]
    host_amps = [torch.empty(final_n * 2, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    init_keys = torch.zeros(k, dtype=torch.int64, pin_memory=True)
    init_amp = torch.tensor([1.0, 0.0], dtype=torch.float64).pin_memory()
    host_table = torch.from_numpy(table.view(np.int64)).pin_memory()
    s2 = ps.SparseState(capacity=final_n)
    states = [st, s2]
    graphs = [ps.Graph(st, apply=lambda: circ.run(st, reset=False), prepare=st.reset),
              ps.Graph(s2, apply=lambda: circ.run(s2, reset=False), prepare=s2.reset)]
    e2e_steps = max(2, min(args.steps, 20))

    def e2e_loop(engine, nsteps):
        ps.set_download_engine(engine)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(nsteps):
            s_i = states[i % 2]
            circ.qram.write(host_table.data_ptr())  # the step's table, in place (the graphs read it there)
            _native.call("sq_state_upload_packed", s_i._h, 1, init_keys.data_ptr(), init_amp.data_ptr())
            graphs[i % 2].launch()
            s_i.download_packed_async(host_keys[i % 2].data_ptr(), host_amps[i % 2].data_ptr())
        for s_i in states:
            s_i.wait()
        ps.synchronize()
        ps.set_download_engine("sm")
        return (time.perf_counter() - t0) / nsteps

    # which engine moves the downloads is tuned here, untimed: the copy
    # engine's rate into pinned memory differs between systems (84 to 190
    # GB/s measured) and has dropped to a quarter within one run, the SM
    # stores' much less; two interleaved rounds of each, and the timed loop
    # runs on the engine whose slower round was the faster
    rounds = [{e: world * updates / e2e_loop(e, 6) for e in ("sm", "copy", "split")} for _ in range(2)]
    calib = {e: min(r[e] for r in rounds) for e in rounds[0]}
    engine = max(calib, key=calib.get) if args.download_engine == "auto" else args.download_engine
    e2e_s = e2e_loop(engine, e2e_steps)
    del graphs
    # the downloaded result is the state the circuit produced
    gk = host_keys[(e2e_steps - 1) % 2].view(k, final_n)
    assert int(torch.count_nonzero(host_amps[(e2e_steps - 1) % 2])) > 0 and gk.shape[1] == final_n
    h2d = k * 8 + 16 + (1 << TABLE_BITS) * 8
    d2h = final_n * (8 * k + 16)
    e2e_value = world * updates / e2e_s

    # profiled step: per-kernel device time with events on the library stream
    _native.profile_reset()
    _native.profile_enable(True)
    circ.run(st)
    _native.profile_enable(False)
    prof = _native.profile_read()
    total_ms = sum(v[1] for v in prof.values())
    dom = max(prof, key=lambda k_: prof[k_][1])
    n_l, d_ms, d_bytes = prof[dom]
    peak, peak_kind = measured_peak_hbm()
    achieved = d_bytes / (d_ms / 1e3) / 1e9 if d_ms > 0 else 0.0
    traffic = ncu_traffic(dom)
    kernels = {name: {"launches": v[0], "ms": round(v[1], 4), "share": round(v[1] / total_ms, 4) if total_ms else 0,
                      "alg_GBps": round(v[2] / (v[1] / 1e3) / 1e9, 1) if v[1] > 0 else 0}
               for name, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    at_scale = elementwise_at_scale(circ, st, peak, peak_kind)

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (complex128 amplitudes), u64 keys", "data": "synthetic (seeded table and angles)",
        "config": dict(workload_config(h, L), updates_per_step=updates, final_entries=final_n,
                       parallelism="replicas" if world > 1 else "single GPU"),
        "gpu_launches": launches,
        "execution": ("each step replayed as one CUDA graph of the circuit (recorded and captured once, counts "
                      "checked on the device); the eager form is reported beside it"),
        "graph_final_size_matches": graph_same,
        "eager": eager,
        "fwht_arithmetic": args.fwht_arithmetic,
        f"{other}_arithmetic": ({"value": world * updates / (other_ms / 1e3), "unit": UNIT, "ms_per_step": other_ms}
                                if other_ms else None),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "download_engine": engine,
                "engine_calibration": {e: [round(r[e], 1) for r in rounds] for e in calib},
                "note": "public API: QRAM table written in place and initial state uploaded from pinned host "
                        "memory, the circuit launched as one CUDA graph, final packed state downloaded into pinned "
                        "host memory, each step; two states alternate so that a step's download overlaps the next "
                        "step's circuit; wall clock until the last download has landed; the download engine is "
                        "the one whose slower of two interleaved untimed calibration runs was the faster "
                        "(engine_calibration: both runs of each)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": traffic, "alg_bytes_per_launch": d_bytes / max(n_l, 1),
                     "avg_launch_ms": d_ms / max(n_l, 1)},
        "kernels": kernels,
        "elementwise_at_scale": at_scale,
    }
    if clocks:
        result["clocks"] = clocks
    # the oracle on the first two layers of the same circuit: the CPU baseline
    # (timed on this host, one thread) and the parity of this kernel
    # configuration (K = 2 key words, 2^24 entries, both butterfly arithmetics)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        upd, dt, parity = cpu_baseline_and_parity(ps, circ)
        result["cpu_baseline"] = {"value": upd / dt, "unit": UNIT, "cores": 1, "kind": "port",
                                  "sample": f"first 2 of {args.layers} layers of the same full-size circuit, "
                                            f"{upd} updates in {dt:.1f} s, one thread"}
        result["parity"] = parity
    if args.trajectories and rank == 0:
        result["batched_trajectories"] = run_trajectories(args, ext)
    if args.qda_steps and rank == 0:
        result["qda_walk"] = run_qda(args, ext)
        if args.qda_batch > 1:
            result["qda_walk"]["batched"] = run_qda_batched(args, ext)
            result["qda_walk"]["target"] = result["qda_walk"]["batched"].pop("target")
    if args.cks_terms and rank == 0:
        result["cks_walk"] = run_cks(args, ext)
    if args.qda3_steps and rank == 0:
        result["qda_config3"] = run_qda_config3(args, ext)
    if args.cks_qram_terms and rank == 0:
        result["cks_qram"] = run_cks_qram(args, ext)
    return result


def elementwise_at_scale(circ, st, peak: float, peak_kind: str, reps: int = 10) -> dict:
    """The layer's fused elementwise program (b ^= QRAM[a], t = a*b,
    c += t, t = a*b, phase on c bit 0: one launch) applied to the state the
    last split left (2^24 entries, 0.54 GB). In the circuit the program runs
    on the 4096 entries between a merge and a split, so it is timed here at
    full size: per launch it reads and writes both key words and the
    amplitude (64 B per entry) and gathers from the 4 MB table, which stays
    in L2."""
    from sparqsim_gb300 import _native
    n = st.size()
    _native.profile_reset()
    _native.profile_enable(True)
    for i in range(reps):
        circ.mid[i % len(circ.mid)](st)
    _native.profile_enable(False)
    n_l, ms, nbytes = _native.profile_read()["elementwise_program"]
    achieved = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    return {"entries": n, "launches": n_l, "avg_launch_ms": ms / max(n_l, 1),
            "alg_bytes_per_launch": nbytes / max(n_l, 1), "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
            "updates_per_s": 5 * n * n_l / (ms / 1e3) if ms > 0 else 0.0}


def profile_case(args) -> None:
    """Small cases of single kernels for ncu (no JSON line): see --profile-case."""
    import torch

    import sparqsim_gb300 as ps
    from sparqsim_gb300 import _native
    _native.call("sq_init", 0)
    if args.profile_case == "elementwise":
        from sparqsim_gb300.workloads import RegisterCircuit
        circ = RegisterCircuit(args.hadamard_bits, 2, seed=SEED).build()
        st = ps.SparseState(capacity=1 << (2 * args.hadamard_bits))
        circ.run(st, layers=1)  # program_kernel launch 1 runs on 2^h entries; the state then holds 2^2h
        for _ in range(3):
            circ.mid[0](st)  # program_kernel launches 2..4 on the full state
        print("elementwise case:", st.size(), "entries")
    else:
        from sparqsim_gb300.workloads import NoisyTrajectories
        w = NoisyTrajectories(n_traj=args.trajectories, layers=6).build_batched()
        st = ps.SparseState(capacity=1 << 26)
        w.run_batched(st)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        w.run_batched(st)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print("trajectories case:", st.size(), "entries")
    ps.synchronize()


def ctypes_void_p():
    import ctypes
    return ctypes.c_void_p()


# ---------------------------------------------------------------------- reference arm
def _ref_worker(h, steps, warmup, barrier, out_q, idx):
    try:
        table, thetas = circuit_inputs(h, 10)
        from oracle import oracle as O  # noqa: F401  (CPU restatement, this process only)
        # setup: layer 1 of the circuit (|0> -> 2^{2h} entries), untimed
        res = _ref_layers(h, table, thetas, 1 + warmup, steps, barrier)
        out_q.put((idx, res))
    except Exception as e:  # report, do not hang the parent
        out_q.put((idx, ("error", repr(e))))


def _ref_layers(h, table, thetas, untimed_layers, timed_layers, barrier):
    import ctypes
    from oracle import oracle as O
    from sparqsim_gb300._native import OP, SqInstr
    from sparqsim_gb300.core import SqCond
    O.clear()
    a, b, c, t = (O.add_register(1, w) for w in (A_BITS, B_BITS, C_BITS, T_BITS))
    q = O.Qram(TABLE_BITS, 32, table)
    st = O.OracleState()
    nocond = SqCond()

    def ins(op, regs, imm=(), cc=()):
        x = SqInstr()
        x.op = OP[op]
        for i, r in enumerate(regs):
            x.reg[i] = r
        for i, v in enumerate(imm):
            x.imm[i] = v
        for i, v in enumerate(cc):
            x.c[i] = v
        return x

    def layer(th):
        n0 = st.size()
        O._chk(O.lib().sqo_hadamard_int(st.h, a, h, ctypes.byref(nocond)))
        n1 = st.size()
        qi = ins("QRAM_LOAD", [a, b])
        qi.qram = q.h
        prog = [qi, ins("MUL_UINT_UINT", [a, b, t]), ins("ADD_UINT_UINT_INPLACE", [t, c]),
                ins("MUL_UINT_UINT", [a, b, t]), ins("PHASE_BOOL", [c], [0], [math.cos(th), math.sin(th)])]
        arr = (SqInstr * len(prog))(*prog)
        O._chk(O.lib().sqo_apply(st.h, arr, len(prog)))
        O._chk(O.lib().sqo_hadamard_int(st.h, a, h, ctypes.byref(nocond)))
        n2 = st.size()
        return max(n0, n1) + 5 * n1 + max(n1, n2)

    for i in range(untimed_layers):
        layer(float(thetas[i % len(thetas)]))
    barrier.wait()
    t0 = time.perf_counter()
    upd = 0
    for i in range(timed_layers):
        upd += layer(float(thetas[(untimed_layers + i) % len(thetas)]))
    return upd, time.perf_counter() - t0


def run_reference(args):
    h = args.hadamard_bits
    ncpu = os.cpu_count() or 1
    try:
        avail_gb = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE") / 2**30
    except Exception:
        avail_gb = 16.0
    per_proc_gb = 4.0 * (1 << (2 * h)) / (1 << 24)
    P = max(1, min(ncpu, int(avail_gb * 0.6 / max(per_proc_gb, 0.1))))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(P + 1)
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(h, args.steps, args.warmup, barrier, q, i)) for i in range(P)]
    for p in procs:
        p.start()
    barrier.wait()
    t0 = time.perf_counter()
    results = [q.get() for _ in procs]
    wall = time.perf_counter() - t0
    for p in procs:
        p.join()
    errs = [r for _, r in results if isinstance(r, tuple) and r and r[0] == "error"]
    if errs:
        print(json.dumps({"impl": "reference", "unavailable": f"CPU restatement failed: {errs[0][1]}"}))
        return
    upd = sum(r[0] for _, r in results)
    value = upd / wall
    sample = (f"{P} concurrent single-thread processes, each {args.steps} steady-state layers (2^{2 * h} -> "
              f"2^{h} -> 2^{2 * h} entries) of the full-size circuit after {1 + args.warmup} untimed layers")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (complex128 amplitudes), u64 registers", "data": "synthetic",
        "config": workload_config(h, 10),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": P, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)  # about 1 s of timed work: several clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--hadamard-bits", type=int, default=12)
    ap.add_argument("--layers", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--download-engine", default="auto", choices=["auto", "sm", "copy", "split"],
                    help="how the end-to-end loop's downloads into pinned memory are moved "
                         "(auto: the fastest in an untimed six-step run of each)")
    ap.add_argument("--skip-other-arithmetic", action="store_true",
                    help="do not also time the other Hadamard butterfly arithmetic")
    ap.add_argument("--trajectories", type=int, default=4096,
                    help="instances in the batched noisy-trajectory leg (0 skips it)")
    ap.add_argument("--plain-sample", type=int, default=256, help="instances timed in the plain GPU form")
    ap.add_argument("--cpu-sample", type=int, default=16, help="instances timed in the oracle")
    ap.add_argument("--qda-steps", type=int, default=10, help="QDA walk steps timed (0 skips)")
    ap.add_argument("--qda-batch", type=int, default=8, help="QDA walks batched in one state (0 or 1 skips)")
    ap.add_argument("--qda-bits", type=int, default=16, help="main register of the QDA walk (16 or 20)")
    ap.add_argument("--qda-warm", type=int, default=200,
                    help="untimed QDA walk steps before the timed ones (200: the state has grown to the size the "
                         "reference's published per-step times are quoted at)")
    ap.add_argument("--cks-terms", type=int, default=3, help="CKS LCU terms timed (0 skips)")
    ap.add_argument("--qda3-steps", type=int, default=3, help="QDA-via-QRAM walk steps timed (0 skips)")
    ap.add_argument("--qda3-bits", type=int, default=10, help="N = 2^bits of the timed QDA-via-QRAM walk")
    ap.add_argument("--qda3-cpu-bits", type=int, default=8, help="N = 2^bits of the oracle's QDA-via-QRAM sample")
    ap.add_argument("--qda3-solve-bits", type=int, default=4, help="N = 2^bits of the 2000-step QDA-via-QRAM solve")
    ap.add_argument("--cks-bits", type=int, default=20, help="main register of the CKS walk")
    ap.add_argument("--cks-qram-terms", type=int, default=2, help="LCU terms of the QRAM CKS walk timed (0 skips)")
    ap.add_argument("--cks-qram-bits", type=int, default=18, help="N = 2^bits of the QRAM CKS walk")
    ap.add_argument("--fwht-arithmetic", default="exact-sum", choices=["exact-sum", "reference"],
                    help="Hadamard butterfly arithmetic of the headline run (the other one is timed too)")
    ap.add_argument("--cuda-profiler-range", default="none", choices=["none", "qda", "cks"],
                    help="bracket the timed QDA steps or CKS terms with cudaProfilerStart/Stop "
                         "(for ncu --profile-from-start off)")
    ap.add_argument("--group-strategy", default="autotune", choices=["autotune", "hash", "sort"],
                    help="how split operators group entries (autotune: timed per shape class)")
    ap.add_argument("--profile-case", default="none", choices=["none", "elementwise", "trajectories"],
                    help="run only a small case for an ncu capture and exit: 'elementwise' = one layer of the "
                         "register circuit, then the layer's fused program three times on its 2^24 entries; "
                         "'trajectories' = the batched trajectories (--trajectories instances) twice, the second "
                         "run inside cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.profile_case != "none":
        profile_case(args)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    result = run_gb300(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
