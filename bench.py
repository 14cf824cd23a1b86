#!/usr/bin/env python
"""Benchmark of the DMRG/TDVP inner loop: two-site H_eff*x throughput.

Workload (the H_eff*x microbenchmark configuration): x[D,2,2,D], L[D,5,D],
R[D,5,D] iid N(0,1) from a fixed numpy seed, L and R symmetrised in (a, a'),
the Heisenberg Schur MPO W[5,2,5,2] with its exact zero pattern; D = 2048
(the largest size of the set) unless --D is given.  A step is one
H_eff*x = ac2_prime(x, W, W, L, R) with the environments prepared once (as
inside a Lanczos solve).  Algorithmic flops per step: F2 = 4 w d^2 D^3 +
4 w^2 d^3 D^2 (the reference's dense pairwise order, derivatives.jl:21).

Arms:
  default            this library (libfmpt) at --precision (default fp64_tc: the
                     FP64-accurate form, FP64 products emulated exactly on the
                     BF16 tensor cores by the Ozaki scheme); also reports every
                     precision form (fp64, fp64_tc, tf32x3, tf32, bf16) at D in
                     {256..2048} with its relative Frobenius error against the
                     plain FP64 form, and the DMRG, U(1), TDVP1 and gradient
                     sections beside the hot path.
  --impl reference   the reference's algorithm on the host cores: the numpy
                     restatement of ac2_prime in the reference's pairwise
                     order (OpenBLAS, all host threads).  The reference itself
                     is Julia and cannot run on this machine.
  --config3          the J1-J2 L=100 D=1024 mixed-vs-FP64 DMRG comparison, both ramps.
  --config5          the differentiable TDVP1 run as configured (100 steps).

Multi-GPU: the path does not shard (each sweep is sequential over bonds), so
--gpus N under torchrun runs N independent replicas; value = all replicas'
flops over the slowest replica's time.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DMRG sweep s & H_eff·x TFLOP/s, mixed vs FP64 on one GB300 at ΔE≤1e-8"
# DRAM bytes (read + write) per tc_gemm launch from one ncu capture of this workload
# (dram__bytes_read.sum + dram__bytes_write.sum of the third step of
# `bench.py --steps 2 --warmup 3`, averaged over its GEMM 1 and GEMM 2)
NCU_TRAFFIC = {("bf16", 2048): {"bytes_per_launch": (88.77e6 + 134.09e6 + 334.29e6 + 106.94e6) / 2,
                                "gemm1_bytes": 88.77e6 + 134.09e6, "gemm2_bytes": 334.29e6 + 106.94e6,
                                "algorithmic_operand_bytes": {"gemm1": 76.0e6, "gemm2": 210.0e6}},
               # dram__bytes_read + write of the two oz_gemm_pair launches of one application
               # (ncu --set full, D=2048); the digit planes the GEMMs read are 0.68 GB (GEMM 1)
               # and 1.89 GB (GEMM 2), the FP64 output tile's epilogue passes add their
               # read-modify-write
               ("fp64_tc", 2048): {"bytes_per_launch": (19.81e9 + 6.05e9 + 24.01e9 + 4.75e9) / 2,
                                   "gemm1_bytes": 19.81e9 + 6.05e9, "gemm2_bytes": 24.01e9 + 4.75e9,
                                   "algorithmic_digit_plane_bytes": {"gemm1": 0.68e9,
                                                                     "gemm2": 1.89e9}}}
UNIT = "TFLOP/s"
W_MPO, D_PHYS = 5, 2
OZ_PRODUCTS = 45          # BF16 digit products per FP64 multiply-add of the fp64_tc GEMM


def flops_ac2(D, w=W_MPO, d=D_PHYS):
    return 4 * w * d * d * D ** 3 + 4 * w * w * d ** 3 * D ** 2


def workload(D, seed=2024):
    from finitemptools_gb300.utilities import heisenberg_xxz_mpo
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((D, 2, 2, D))
    L = rng.standard_normal((D, W_MPO, D))
    L = 0.5 * (L + L.transpose(2, 1, 0))
    R = rng.standard_normal((D, W_MPO, D))
    R = 0.5 * (R + R.transpose(2, 1, 0))
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    return x, L, R, W


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [q.strip() for q in line.split(",")]
                if len(p) < 8:
                    continue
                try:
                    sm.append(float(p[0]))
                    mx = float(p[1])
                except ValueError:
                    continue
                for nm, v in zip(names, p[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(D, budget_s=12.0):
    """The oracle's ac2_prime (numpy, reference pairwise order) on the host:
    repeated full applications at D until about budget_s seconds."""
    import oracle as O
    x, L, R, W = workload(D)
    O.ac2_prime(x, W, W, L, R)              # warm BLAS threads
    n, t0 = 0, time.perf_counter()
    while True:
        O.ac2_prime(x, W, W, L, R)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 20:
            break
    return {"value": flops_ac2(D) * n / el / 1e12, "unit": UNIT, "cores": os.cpu_count(),
            "kind": "port",
            "sample": "%d full two-site H_eff*x applications at D=%d, float64, numpy/OpenBLAS "
                      "with all %d host threads, %.1f s" % (n, D, os.cpu_count(), el)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    D = args.D
    x, L, R, W = workload(D)
    # bound the run: estimate one step, shrink the per-step sample if needed
    t0 = time.perf_counter()
    O.ac2_prime(x, W, W, L, R)
    est = time.perf_counter() - t0
    steps = args.steps + args.warmup
    frac = 1.0
    if est * steps > 150.0:
        frac = max(150.0 / (est * steps), 1.0 / D)
    nb = max(1, int(round(D * frac)))
    Rs = R[:nb]                               # right-environment bra rows b' of the sample
    f_step = (flops_ac2(D) - 2 * 4 * W_MPO * D ** 3) + 2 * 4 * W_MPO * D * D * nb
    for _ in range(args.warmup):
        O.ac2_prime(x, W, W, L, Rs)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.ac2_prime(x, W, W, L, Rs)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    v = f_step / (ms / 1e3) / 1e12
    sample = ("two-site H_eff*x at D=%d, float64, numpy/OpenBLAS on %d host threads%s" %
              (D, os.cpu_count(), "" if nb == D else
               ", output columns b' sampled: %d of %d per step" % (nb, D)))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_dict(args, "fp64"),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_dmrg_sweeps(mpo, e_ed, e_gpu, budget_s=40.0):
    """The oracle's FP64 DMRG2 (numpy, the reference's algorithm step for step) on the
    XXZ chain L=20: seeded D=8 start (the GPU run's seed), right-canonicalised, 4 sweeps
    at D=64, cutoff 1e-10, Lanczos 30 vectors / tol 1e-12, on all host cores; stops early
    past budget_s."""
    import oracle as O
    from finitemptools_gb300.utilities import FiniteMPO
    rng = np.random.default_rng(20)
    st, _ = O.canonicalize(O.randommps(20, 2, 8, rng), normalize=True)
    env = O.environments(FiniteMPO(mpo, 20), st)
    times, t_all = [], time.perf_counter()
    for _ in range(4):
        t0 = time.perf_counter()
        Es, _ = O.dmrg2_sweep(env, O.MPSTruncation(64, 1e-10), 30, 1e-12)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget_s:
            break
    E = float(Es[-1])
    return {"sweep_s": times, "E_last_bond": E, "dE_rel_vs_ed": abs(E - e_ed) / abs(e_ed),
            "dE_rel_vs_gpu_fp64": abs(E - e_gpu) / abs(e_gpu), "threads": os.cpu_count(),
            "note": "numpy/OpenBLAS with all host threads; E is the last Ritz value"}


def config3_j1j2(h, fm, run, full=False, L=100, window=20):
    """J1-J2 L=100 (J1=1, J2=0.3), cutoff 1e-9, D ramp 64 -> 256 -> 1024 from a seeded D=16
    state.  (At J2=0.5 the ground state is an exact dimer product and keeps D<=3, so the
    D=1024 stage runs at J2=0.3.)
      mixed: 3xTF32 contractions and environment updates, FP64 Lanczos reorthogonalisation,
             the FP64 density-matrix split with tail refinement;
      fp64:  the plain form -- FP64-accurate contractions (the tensor-core FP64 engine) and
             the reference's SVD split (gesvd).
    Always: the mixed ramp with two D=1024 sweeps (the second one timed: sweep_s_mixed) and,
    from that converged state, the same window of `window` consecutive centre bonds run in
    both forms (state restored in between): window_s_mixed / window_s_fp64.
    full=True adds the plain form's own ramp from the same start (64, 256, then two D=1024
    sweeps, the second timed: sweep_s_fp64) and the relative difference of the two
    FP64-evaluated ground-state energies."""
    import time as _t
    from finitemptools_gb300 import algorithms as A
    hj = fm.j1j2_heisenberg_mpo(1.0, 0.3)
    mpo = fm.FiniteMPO(hj, L)
    alg_mx = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(1024, 1e-9),
                      precision="tf32x3", reorth=True, svd="dm")
    alg_64 = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(1024, 1e-9),
                      precision="fp64_tc", svd="gesvd")
    env, tmx = run(L, hj, [(64, 1), (256, 1), (1024, 2)], "tf32x3", "dm", True, 1e-9, 16, 5)
    E_mx = float(fm.expectation(env.mps, mpo))
    res = {"J2": 0.3, "cutoff": 1e-9, "ramp_sweeps_s_mixed": tmx, "sweep_s_mixed": tmx[-1],
           "Dmax_mixed": fm.bond_dimension(env.mps), "E_mixed_fp64_eval": E_mx}
    # the window: left-sweep bond bodies at sites s0 .. s0+window-1 from the converged state
    s0 = L // 2 - window // 2
    env.precision = alg_mx.env_precision
    for site in range(1, s0):
        A._dmrg2_bond_left(env, site, alg_mx)
    keep_mps = {i: env.mps[i].copy() for i in range(s0, s0 + window + 1)}
    keep_env = {i: env.hstorage[i] for i in range(s0 + 1, s0 + window + 1)}
    shapes = [list(env.mps[i].shape) for i in range(s0, s0 + window)]
    times = {}
    for name, alg in (("mixed", alg_mx), ("fp64", alg_64)):
        env.precision = alg.env_precision
        h.synchronize()
        t0 = _t.perf_counter()
        for site in range(s0, s0 + window):
            A._dmrg2_bond_left(env, site, alg)
        h.synchronize()
        times[name] = _t.perf_counter() - t0
        for i, v in keep_mps.items():
            env.mps[i] = v.copy()
        for i, v in keep_env.items():
            env.hstorage[i] = v
    res.update({"window_sites": [s0, s0 + window - 1], "window_site_shapes": shapes,
                "window_s_mixed": times["mixed"], "window_s_fp64": times["fp64"],
                "window_speedup_fp64_over_mixed": times["fp64"] / times["mixed"]})
    del env, keep_mps, keep_env
    if full:
        # the same ramp as the mixed form (one D=1024 sweep only reaches about D=500)
        env64, t64 = run(L, hj, [(64, 1), (256, 1), (1024, 2)], "fp64_tc", "gesvd", False, 1e-9,
                         16, 5)
        E_64 = float(fm.expectation(env64.mps, mpo))
        res.update({"ramp_sweeps_s_fp64": t64, "sweep_s_fp64": t64[-1],
                    "Dmax_fp64": fm.bond_dimension(env64.mps), "E_fp64": E_64,
                    "dE_rel_mixed_vs_fp64": abs(E_mx - E_64) / abs(E_64),
                    "sweep_speedup_fp64_over_mixed": t64[-1] / tmx[-1]})
        del env64
    return res


def config3_equal_D(h, fm, run, eps=1e-12, L=100):
    """The config-3 comparison at equal bond dimension.  At cutoff 1e-9 the reference's
    gesvd truncation keeps about 500 states of the FP64 J1-J2 ground state, while the
    3xTF32 Ritz vectors carry a noise floor near 1e-7 of their largest singular value that
    the same cutoff keeps, up to D=1024.  Both forms are therefore run here with cutoff
    `eps`, which neither reaches, so that both ramps (64 -> 256 -> 1024, two sweeps at
    1024, from the same seeded D=16 state) end at D=1024; the second D=1024 sweep of each
    is timed, and the FP64-evaluated energies are compared."""
    hj = fm.j1j2_heisenberg_mpo(1.0, 0.3)
    mpo = fm.FiniteMPO(hj, L)
    envm, tm = run(L, hj, [(64, 1), (256, 1), (1024, 2)], "tf32x3", "dm", True, eps, 16, 5)
    Em = float(fm.expectation(envm.mps, mpo))
    Dm = fm.bond_dimension(envm.mps)
    del envm
    env64, t64 = run(L, hj, [(64, 1), (256, 1), (1024, 2)], "fp64_tc", "gesvd", False, eps, 16, 5)
    E64 = float(fm.expectation(env64.mps, mpo))
    D64 = fm.bond_dimension(env64.mps)
    del env64
    return {"cutoff": eps, "J2": 0.3, "ramp_sweeps_s_mixed": tm, "ramp_sweeps_s_fp64": t64,
            "sweep_s_mixed": tm[-1], "sweep_s_fp64": t64[-1], "Dmax_mixed": Dm, "Dmax_fp64": D64,
            "sweep_speedup_fp64_over_mixed": t64[-1] / tm[-1], "E_mixed_fp64_eval": Em,
            "E_fp64": E64, "dE_rel_mixed_vs_fp64": abs(Em - E64) / abs(E64)}


def dmrg_section(h, fm, budget_s=150.0, full3=False, only3=False):
    """DMRG sweep seconds, plain FP64 vs the mixed form (3xTF32 contractions and
    environment updates, FP64 Lanczos reorthogonalisation, FP64 density-matrix
    split), each energy evaluated in FP64 as <psi|H|psi> of the final state.
      xxz_L20: XXZ L=20, Delta=1, D=64, cutoff 1e-10, 4 sweeps from a seeded D=8
               right-canonical state; the exact energy is the ED fixture.
      xxz_L20_D64_dmrg1s: the same chain and start with DMRG1S + OptimalExpansion, FP64,
               6 sweeps.
      j1j2_L100_D1024: J1-J2 L=100, J1=1, J2=0.3, cutoff 1e-9, ramp 64 -> 256 -> 1024 in
               the mixed form (two sweeps at 1024, the second timed), then the same window
               of 20 centre bonds run in both forms from that converged state (config3_j1j2).
               `--config3` adds both forms' full ramps, as configured and at equal D.
               (At J2=0.5 the ground state is an exact dimer product and keeps D<=3,
               so the D=1024 stage runs at J2=0.3.)"""
    import time as _t
    from finitemptools_gb300 import algorithms as A
    from finitemptools_gb300.auxiliary import scal
    out = {}
    t_start = _t.perf_counter()
    with open(os.path.join(ROOT, "tests", "golden", "exact_energies.json")) as f:
        e_ed = json.load(f)["xxz_L20_J1_Jzz1_hz0"]

    def run(L, mpo, stages, prec, svd, reorth, eps, D0, seed, driver="python"):
        rng = np.random.default_rng(seed)
        psi = fm.randommps(L, 2, D0, rng, handle=h)
        fm.canonicalize_(psi, normalize=True)
        env = fm.environments(fm.FiniteMPO(mpo, L), psi)
        times = []
        for D, n in stages:
            alg = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(D, eps),
                           precision=prec, reorth=reorth, svd=svd, driver=driver)
            for _ in range(n):
                h.synchronize()
                t0 = _t.perf_counter()
                fm.sweep_(env, alg)
                h.synchronize()
                times.append(_t.perf_counter() - t0)
        return env, times

    if only3:
        return {"as_configured": config3_j1j2(h, fm, run, full=True),
                "equal_D": config3_equal_D(h, fm, run)}
    hx = fm.heisenberg_xxz_mpo(1.0, 1.0, 0.0)
    env64, t64 = run(20, hx, [(64, 4)], "fp64", "gesvd", False, 1e-10, 8, 20)
    envmx, tmx = run(20, hx, [(64, 4)], "tf32x3", "dm", True, 1e-10, 8, 20)
    # the same FP64 sweeps through the whole-sweep entry point (fmpt_dmrg2_sweep)
    envdv, tdv = run(20, hx, [(64, 4)], "fp64", "gesvd", False, 1e-10, 8, 20, driver="device")
    E64 = float(fm.expectation(env64.mps, fm.FiniteMPO(hx, 20)))
    Emx = float(fm.expectation(envmx.mps, fm.FiniteMPO(hx, 20)))
    Edv = float(fm.expectation(envdv.mps, fm.FiniteMPO(hx, 20)))
    out["xxz_L20_D64"] = {"sweep_s_fp64": t64, "sweep_s_mixed": tmx, "E_fp64": E64,
                          "E_mixed_fp64_eval": Emx, "dE_rel_mixed_vs_fp64": abs(Emx - E64) / abs(E64),
                          "E_ed": e_ed, "dE_rel_fp64_vs_ed": abs(E64 - e_ed) / abs(e_ed),
                          "sweep_s_fp64_device_driver": tdv,
                          "ms_per_bond_fp64": [1e3 * t / 37 for t in t64],
                          "ms_per_bond_fp64_device_driver": [1e3 * t / 37 for t in tdv],
                          "E_fp64_device_driver_equal": Edv == E64}
    del envdv
    # the same 4 FP64 sweeps (same seed, start and truncation) by the oracle's DMRG2 on the
    # host cores: the CPU run this workload is checked against
    out["xxz_L20_D64"]["cpu_reference"] = cpu_dmrg_sweeps(hx, e_ed, E64)
    # DMRG1S with OptimalExpansion (the reference's default ground-state algorithm), same
    # chain, start and truncation as the FP64 DMRG2 run above, with the reference's
    # expansion and with the capped one
    res1 = {}
    for cap in (False, True):
        rng = np.random.default_rng(20)
        psi1 = fm.randommps(20, 2, 8, rng, handle=h)
        fm.canonicalize_(psi1, normalize=True)
        env1 = fm.environments(fm.FiniteMPO(hx, 20), psi1)
        alg1 = fm.DMRG1S(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(64, 1e-10),
                         expan=fm.OptimalExpansion(cap=cap), verbosity=0)
        t1s = []
        for _ in range(6):
            h.synchronize()
            t0 = _t.perf_counter()
            fm.sweep_(env1, alg1)
            h.synchronize()
            t1s.append(_t.perf_counter() - t0)
        E1 = float(fm.expectation(env1.mps, fm.FiniteMPO(hx, 20)))
        res1["capped_expansion" if cap else "reference_expansion"] = {
            "sweep_s_fp64": t1s, "E_fp64": E1, "dE_rel_vs_ed": abs(E1 - e_ed) / abs(e_ed),
            "Dmax": fm.bond_dimension(env1.mps)}
        del env1, psi1
    res1["E_ed"] = e_ed
    res1["note"] = ("reference expansion: once D saturates, truncating [B ; V1 NR] (all singular "
                    "values 1) drops part of the state and the energy stalls; capped: at most "
                    "D_max - D new directions (not in the reference)")
    out["xxz_L20_D64_dmrg1s"] = res1
    if _t.perf_counter() - t_start > budget_s:
        return out
    out["j1j2_L100_J2_0.3_D1024"] = config3_j1j2(h, fm, run, full=full3)
    if _t.perf_counter() - t_start > budget_s:
        return out
    # XX chain (Delta = 0), L=200, D=256, against the free-fermion closed form
    hxx = fm.heisenberg_xxz_mpo(1.0, 0.0, 0.0)
    envx, tx = run(200, hxx, [(64, 2), (256, 3)], "tf32x3", "dm", True, 1e-9, 16, 7)
    Exx = float(fm.expectation(envx.mps, fm.FiniteMPO(hxx, 200)))
    with open(os.path.join(ROOT, "tests", "golden", "exact_energies.json")) as f:
        e_ff = json.load(f)["xx_L200_free_fermion"]
    out["xx_L200_D256"] = {"sweep_s_mixed": tx, "E_mixed_fp64_eval": Exx, "E_free_fermion": e_ff,
                           "dE_rel_vs_free_fermion": abs(Exx - e_ff) / abs(e_ff),
                           "Dmax": fm.bond_dimension(envx.mps)}
    del envx
    if _t.perf_counter() - t_start > budget_s:
        return out
    return out


def u1_section(h, fm, budget_s=150.0):
    """U(1) block-sparse DMRG2 (charge = number of up spins, total Sz = 0): the
    grouped persistent FP64 engine, graph-captured Lanczos, autotuned tiles and
    the batched density-matrix sector split.
      xxz_L20: parity with exact diagonalisation (same fixture as the dense path).
      heisenberg_L64: D ramp 64 -> 256 -> 1024 (cutoff 1e-14, 10 Lanczos vectors),
               two timed sweeps at D=1024; the centre bond's H_eff*x in the
               block-sparse form vs the dense FP64 form on the same (charge-sorted)
               tensors, and vs the oracle's block-by-block numpy restatement on the
               host cores (the reference's symmetric CPU path cannot run here)."""
    import time as _t
    from finitemptools_gb300 import DeviceTensor as DT
    from finitemptools_gb300.u1 import (U1ExpectationCache, U1HeffOp, u1_pack2, u1_randommps,
                                        u1_twosite, u1_unpack2)
    out = {}
    t_start = _t.perf_counter()
    with open(os.path.join(ROOT, "tests", "golden", "exact_energies.json")) as f:
        e_ed = json.load(f)["xxz_L20_J1_Jzz1_hz0"]
    hx = fm.heisenberg_xxz_mpo(1.0, 1.0, 0.0)

    profile = []

    def sweeps(m, D, n, eps, kmax):
        alg = fm.DMRG2(eig_maxiter=kmax, eig_tol=1e-12, trunc=fm.MPSTruncation(D, eps), svd="dm",
                       verbosity=0)
        ts, Es = [], []
        for _ in range(n):
            dims0 = m.mps.bond_dimensions()
            h.synchronize()
            t0 = _t.perf_counter()
            E, _ = fm.sweep_(m, alg)
            h.synchronize()
            ts.append(_t.perf_counter() - t0)
            Es.append(E[-1])
            dims1 = m.mps.bond_dimensions()
            # the work of a bond grows as D^3: sum of D^3 over the bonds before and after
            profile.append({"D": D, "s": ts[-1], "Dmax_before": max(dims0),
                            "Dmax_after": max(dims1),
                            "sum_D3_before": float(sum(float(d) ** 3 for d in dims0)),
                            "sum_D3_after": float(sum(float(d) ** 3 for d in dims1))})
        return ts, Es

    psi = u1_randommps(20, 10, 8, rng=20, handle=h)
    m = U1ExpectationCache(hx, psi)
    t20, _ = sweeps(m, 64, 4, 1e-10, 30)
    E20 = float(fm.expectation(psi, hx))
    out["xxz_L20_Sz0_D64"] = {"sweep_s": t20, "E": E20, "E_ed": e_ed,
                              "dE_rel_vs_ed": abs(E20 - e_ed) / abs(e_ed)}
    del m, psi
    if _t.perf_counter() - t_start > budget_s:
        return out
    L, N = 64, 32
    psi = u1_randommps(L, N, 16, rng=64, handle=h)
    m = U1ExpectationCache(hx, psi)
    # cutoff 1e-14: the bond dimension, not the cutoff, limits the state (at 1e-10
    # the L=64 ground state stops growing near D=200)
    tramp, _ = sweeps(m, 64, 1, 1e-14, 10)
    t2, _ = sweeps(m, 256, 1, 1e-14, 10)
    tramp += t2
    t1024, E1024 = sweeps(m, 1024, 2, 1e-14, 10)
    E = float(fm.expectation(psi, hx))
    site = L // 2
    Vl, Vm, Vr = psi.spaces[site], psi.spaces[site + 1], psi.spaces[site + 2]
    qp = psi.qphys
    x = u1_twosite(psi[site], psi[site + 1], Vl, Vm, Vr, qp, qp)
    op = U1HeffOp(m.hstorage[site], m.hstorage[site + 2], m.mpo[site], m.mpo[site + 1], Vl, Vr,
                  qp, qp, m.qw[site], m.qw[site + 1], m.qw[site + 2])
    y = DT((op.n,), np.float64, h)
    h.profile(True)
    for _ in range(3):
        op(x, y)
    h.profile_read(4)
    for _ in range(10):
        op(x, y)
    n_g, ms_g = h.profile_read(4)
    h.profile(False)
    ms_u1 = ms_g / max(n_g, 1)
    X = u1_unpack2(x, Vl, Vr, qp, qp)
    dop = fm.HeffOp("ac2", m.hstorage[site], m.hstorage[site + 2], W1=m.mpo[site],
                    W2=m.mpo[site + 1])
    Y = DT(X.shape, np.float64, h)
    dop(X, Y)
    h.synchronize()
    t0 = _t.perf_counter()
    for _ in range(3):
        dop(X, Y)
    h.synchronize()
    ms_dense = (_t.perf_counter() - t0) / 3 * 1e3
    yd = u1_pack2(Y, Vl, Vr, qp, qp).numpy()
    yu = y.numpy()
    lz = {}
    for g in (False, True):
        h.set_graphs(g)
        op.lanczos(x, 10, 1e-12)
        h.synchronize()
        t0 = _t.perf_counter()
        op.lanczos(x, 10, 1e-12)
        h.synchronize()
        lz["graph" if g else "host_loop"] = (_t.perf_counter() - t0) * 1e3
    h.set_graphs(True)
    cpu_ms = None
    try:   # the oracle's block-by-block restatement on the host cores (baseline leg)
        from oracle.u1 import Leg, ac2_prime_blocks
        Lh, Rh, Xh = m.hstorage[site].numpy(), m.hstorage[site + 2].numpy(), X.numpy()
        vl, vr = Leg(zip(Vl.charges, Vl.dims)), Leg(zip(Vr.charges, Vr.dims))
        t0 = _t.perf_counter()
        ac2_prime_blocks(Xh, m.mpo[site], m.mpo[site + 1], Lh, Rh, vl, vr, list(qp), list(qp),
                         m.qw[site], m.qw[site + 2])
        cpu_ms = (_t.perf_counter() - t0) * 1e3
    except Exception as e:     # noqa: BLE001 -- the baseline is optional in the report
        cpu_ms = "unavailable: %s" % e
    out["heisenberg_L64_Sz0_D1024"] = {
        "ramp_sweeps_s": tramp, "sweep_s_D1024": t1024, "E_last_sweeps": E1024, "E": E,
        "bond_dims_max": max(psi.bond_dimensions()),
        "centre_leg_sectors": len(Vm.charges), "centre_block_dims": list(Vm.dims),
        "heff_block_sparse_ms": ms_u1, "heff_block_sparse_flops": op.flops(),
        "heff_block_sparse_gflops": op.flops() / (ms_u1 * 1e-3) / 1e9,
        "heff_tile": op.tile(), "heff_dense_fp64_ms": ms_dense,
        "heff_speedup_vs_dense_fp64": ms_dense / ms_u1,
        "heff_rel_diff_vs_dense": float(np.linalg.norm(yu - yd) / np.linalg.norm(yd)),
        "lanczos10_ms": lz, "heff_cpu_oracle_blocks_ms": cpu_ms,
        "tuning_entries_timed": h.tuning_info(),
        "sweep_profile": profile[-4:],
        "note": "sweeps: DMRG2 svd=dm (batched density-matrix sector split), eig_maxiter 10, "
                "cutoff 1e-14"}
    return out


def cublas_same_shapes(D, stream, reps=10):
    """cuBLAS (torch.matmul, bf16 operands, FP32 accumulation) on the two GEMM shapes of
    the BF16 two-site H_eff*x at bond dimension D: GEMM 1 M = 4D, N = 5D, K = D and
    GEMM 2 M = 4D, N = D, K = 5D (w=5, d=2), each timed with CUDA events after a
    warm-up; a yardstick for the hand-written tcgen05 GEMM on the same problems."""
    import torch
    out = {}
    for name, (M, N, K) in (("gemm1", (4 * D, W_MPO * D, D)), ("gemm2", (4 * D, D, W_MPO * D))):
        a = torch.randn(M, K, device="cuda", dtype=torch.bfloat16)
        b = torch.randn(K, N, device="cuda", dtype=torch.bfloat16)
        for _ in range(3):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            torch.matmul(a, b)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"M": M, "N": N, "K": K, "ms": ms, "tflops": 2.0 * M * N * K / (ms / 1e3) / 1e12}
        del a, b
    return out


def next_rows_section(h, fm):
    """The paths beside the hot path, each timed once on synthetic inputs:
      ed_xxz_L20: exact_diagonalization of the XXZ chain L=20 (Delta=1) through the
          device ac_prime at the centre (n = 2^20, environments 512 and 1024 wide),
          num=2, tol 1e-10; E0 against the ED fixture; the host numpy ac_prime of
          the oracle timed on the same centre (2 applications) for comparison.
      excited_xxz_L20_D64: projected DMRG2 for the first excited state (ground state
          from 4 DMRG2 sweeps at D=64 as the projector, 4 projected sweeps), E1
          against the device ED value above.
      tebd_bond_D256: one layer of 19 two-site gates exp(-i 0.05 h) (TFI bonds) on
          a random right-canonical complex MPS, L=20, D=256 kept, in the gesvd and
          density-matrix forms; the oracle's numpy bond update timed on 2 bonds."""
    import time as _t
    import oracle as O
    from oracle import core as OC
    from oracle import tebd as OT
    out = {}
    with open(os.path.join(ROOT, "tests", "golden", "exact_energies.json")) as f:
        e_ed = json.load(f)["xxz_L20_J1_Jzz1_hz0"]
    hx = fm.heisenberg_xxz_mpo(1.0, 1.0, 0.0)
    # --- exact diagonalisation on the device
    h.synchronize()
    t0 = _t.perf_counter()
    vals, states = fm.exact_diagonalization(hx, len=20, num=2, rng=np.random.default_rng(1),
                                            tol=1e-10, handle=h)
    h.synchronize()
    t_ed = _t.perf_counter() - t0
    psi = states[0]
    left, right, Wc = fm.init_h_center(hx, psi)
    op = fm.HeffOp("ac", left, right, W1=Wc)
    x = psi[psi.center]
    op(x)
    h.synchronize()
    t0 = _t.perf_counter()
    for _ in range(5):
        op(x)
    h.synchronize()
    t_apply = (_t.perf_counter() - t0) / 5
    Ln, Rn, xn = left.numpy(), right.numpy(), x.numpy()
    t0 = _t.perf_counter()
    for _ in range(2):
        OC.ac_prime(xn, np.asarray(Wc), Ln, Rn)
    t_apply_cpu = (_t.perf_counter() - t0) / 2
    out["ed_xxz_L20"] = {"s_total": t_ed, "E0": vals[0], "E1": vals[1], "E0_fixture": e_ed,
                         "dE0_rel": abs(vals[0] - e_ed) / abs(e_ed),
                         "centre_shape": list(x.shape), "ms_per_apply_gpu_fp64": 1e3 * t_apply,
                         "ms_per_apply_cpu_numpy": 1e3 * t_apply_cpu,
                         "apply_speedup": t_apply_cpu / t_apply}
    del op, left, right, states, psi
    # --- first excited state by projected DMRG2
    rng = np.random.default_rng(20)
    g = fm.randommps(20, 2, 8, rng, handle=h)
    fm.canonicalize_(g, normalize=True)
    envg = fm.environments(fm.FiniteMPO(hx, 20), g)
    alg = fm.DMRG2(eig_maxiter=20, eig_tol=1e-12, trunc=fm.MPSTruncation(64, 1e-10), verbosity=0)
    for _ in range(4):
        fm.sweep_(envg, alg)
    st = fm.randommps(20, 2, 8, np.random.default_rng(21), handle=h)
    fm.canonicalize_(st, normalize=True)
    envx = fm.environments(fm.FiniteMPO(hx, 20), st, [envg.mps])
    tx = []
    for _ in range(4):
        h.synchronize()
        t0 = _t.perf_counter()
        Es, _ = fm.sweep_(envx, alg)
        h.synchronize()
        tx.append(_t.perf_counter() - t0)
    out["excited_xxz_L20_D64"] = {"sweep_s": tx, "E1_dmrg": Es[-1], "E1_device_ed": vals[1],
                                  "dE1_rel": abs(Es[-1] - vals[1]) / abs(vals[1])}
    del envx, envg
    # --- TEBD bond updates at D=256
    L, D = 20, 256
    Z = np.diag([-1.0, 1.0])
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    import scipy.linalg
    G = scipy.linalg.expm(-0.05j * (-np.kron(Z, Z) - 0.5 * (np.kron(np.eye(2), X) +
                                                             np.kron(X, np.eye(2)))))
    mps, sv = O.canonicalize(O.randommps(L, 2, D, np.random.default_rng(256),
                                         dtype=np.complex128), normalize=True)
    sv[0], sv[L] = np.ones(1), np.ones(1)
    layer = fm.QuantumCircuit(fm.QuantumGate((i, i + 1), G) for i in range(1, L))
    res = {}
    for name, svd, meth in (("gesvd", "gesvd", "gesvd"), ("gesvdp", "gesvd", "gesvdp"),
                            ("gesvdj", "gesvd", "gesvdj"), ("dm", "dm", "gesvd")):
        h.set_svd_method(meth)
        psi_t = fm.FiniteMPS.from_numpy(mps, handle=h)
        for i in range(1, L + 2):
            psi_t.s[i] = fm.DeviceTensor.from_numpy(np.asarray(sv[i - 1], dtype=np.float64), h)
        centre = layer[L // 2 - 1]                                   # gate on (L/2, L/2+1)
        fm.apply_([centre], psi_t, trunc=fm.MPSTruncation(D, 1e-12), svd=svd)   # warm-up
        h.synchronize()
        t0 = _t.perf_counter()
        for _ in range(3):
            fm.apply_([centre], psi_t, trunc=fm.MPSTruncation(D, 1e-12), svd=svd)
        h.synchronize()
        t_c = (_t.perf_counter() - t0) / 3
        t0 = _t.perf_counter()
        fm.apply_(layer, psi_t, trunc=fm.MPSTruncation(D, 1e-12), svd=svd)
        h.synchronize()
        res[name] = (t_c, (_t.perf_counter() - t0) / len(layer))
    h.set_svd_method("gesvd")
    mo, so = [A.copy() for A in mps], list(sv)
    c = L // 2
    t0 = _t.perf_counter()
    for i in (c, c + 1):
        OT.apply_gate((i, i + 1), G, mo, so, O.MPSTruncation(D, 1e-12))
    t_cpu = (_t.perf_counter() - t0) / 2
    out["tebd_bond_D256"] = {
        "ms_per_centre_gate": {k: 1e3 * v[0] for k, v in res.items()},
        "ms_per_gate_layer_average": {k: 1e3 * v[1] for k, v in res.items()},
        "ms_per_centre_gate_cpu_numpy": 1e3 * t_cpu,
        "centre_speedup_gesvd": t_cpu / res["gesvd"][0],
        "note": "centre gate: theta 512 x 512 complex; the layer average includes the small "
                "edge bonds"}
    return out


def _tfi_start(fm, h, L=40, D=64, seed=40):
    """TFI chain h_i = 1 + 0.1 N(0,1) (seeded) and a random normalised complex MPS, D=64."""
    rng = np.random.default_rng(seed)
    hs = 1.0 + 0.1 * rng.standard_normal(L)
    psi = fm.randommps(L, 2, D, rng, dtype=np.complex128, handle=h)
    fm.canonicalize_(psi, normalize=True)
    return hs, psi


def tdvp_section(h, fm, nsteps=5):
    """One-site TDVP (algorithms/tdvp.jl:19-69): TFI L=40, complex128, D=64, dt=0.05
    (stepsize -0.05i), Krylov dimension 20, exptol 1e-8.  After one warm-up step, nsteps
    timed steps in the plain FP64 form and in the 3xTF32 form (complex data on the
    tensor cores through the real embedding; FP64 Krylov, QR and environment updates).
    CPU baseline: the oracle's tdvp1_sweep (numpy, the reference's algorithm step for
    step, all host threads) for ONE step from the state after the warm-up step, and the
    device's FP64 step from that same state; <Z_20> of both after that step."""
    import time as _t
    import oracle as O
    from finitemptools_gb300.utilities import FiniteMPO
    L, Z = 40, np.diag([-1.0, 1.0])
    res = {}
    start = None
    for prec in ("fp64", "tf32x3"):
        hs, psi = _tfi_start(fm, h)
        envt = fm.environments(fm.FiniteMPO(fm.tfi_mpo(hs), L), psi)
        alg = fm.TDVP1(stepsize=-0.05j, D=64, exptol=1e-8, krylovdim=20, precision=prec)
        fm.sweep_(envt, alg)                             # first step (bond growth, warm-up)
        if prec == "fp64":
            start = [A.numpy() for A in envt.mps]
            h.synchronize()
            t0 = _t.perf_counter()
        fm.sweep_(envt, alg)                             # second step (fp64: timed alone)
        if prec == "fp64":
            h.synchronize()
            t_one = _t.perf_counter() - t0
            z_one = float(np.real(fm.expectation_local(envt.mps, 20, Z)))
        h.synchronize()
        t0 = _t.perf_counter()
        for _ in range(nsteps):
            fm.sweep_(envt, alg)
        h.synchronize()
        res[prec] = ((_t.perf_counter() - t0) / nsteps,
                     float(np.real(fm.expectation_local(envt.mps, 20, Z))))
        del envt, psi
    env_o = O.environments(FiniteMPO(fm.tfi_mpo(hs), L), [A.copy() for A in start])
    t0 = _t.perf_counter()
    O.tdvp1_sweep(env_o, -0.05j, D=64, exptol=1e-8, krylovdim=20)
    t_cpu = _t.perf_counter() - t0
    z_cpu = float(np.real(O.single_site_expectation(env_o.mps, 20, Z)))
    return {"s_per_step_fp64_complex": res["fp64"][0], "steps_timed": nsteps,
            "s_per_step_tf32x3_complex": res["tf32x3"][0],
            "Z20_after_%d_steps_fp64" % (nsteps + 2): res["fp64"][1],
            "Z20_tf32x3_minus_fp64": res["tf32x3"][1] - res["fp64"][1],
            "cpu_reference": {"s_per_step": t_cpu, "threads": os.cpu_count(),
                              "speedup_gpu_fp64_over_cpu": t_cpu / t_one,
                              "gpu_fp64_s_same_step": t_one,
                              "Z20_cpu": z_cpu, "Z20_gpu_fp64": z_one,
                              "dZ20_gpu_vs_cpu": abs(z_one - z_cpu),
                              "note": "one step of the oracle's tdvp1_sweep (numpy/OpenBLAS, "
                                      "all host threads) and of the device FP64 form from the "
                                      "same state (after one warm-up step)"}}


def tdvp_grad_section(h, fm, nsteps=5, checkpoint=2, fd_sites=(20, 21, 1, 40),
                      mixed=True):
    """Config 5 (differentiable TDVP1): TFI L=40, h_i = 1 + 0.1 N(0,1) (seed 40), random
    normalised complex MPS D=64, dt=0.05 (stepsize -0.05i), Krylov dimension 20, exptol
    1e-8; gradient of <Z_20>(T) with respect to all 40 h_i by the device adjoint (MPS
    checkpoints every `checkpoint` steps, blocks recomputed in the reverse pass), checked
    against central differences (step 1e-5, FP64 device forward) on the fields
    `fd_sites` (1-based).  mixed: the same value and gradient with the Krylov
    exponentials of forward and adjoint in 3xTF32, and their errors against FP64."""
    import time as _t
    from finitemptools_gb300 import adjoint as AD
    L = 40
    hs, psi = _tfi_start(fm, h)
    Z = np.diag([-1.0, 1.0])
    alg = fm.TDVP1(stepsize=-0.05j, D=64, exptol=1e-8, krylovdim=20)

    def forward(hv):
        env = fm.environments(fm.tfi_mpo(hv), fm.FiniteMPS([A.copy() for A in psi.data]))
        for _ in range(nsteps):
            fm.sweep_(env, alg)
        return float(np.real(fm.expectation_local(env.mps, 20, Z)))

    h.synchronize()
    t0 = _t.perf_counter()
    v0 = forward(hs)
    h.synchronize()
    t_fwd = _t.perf_counter() - t0
    t0 = _t.perf_counter()
    val, g = AD.tfi_field_gradient(hs, psi, -0.05j, nsteps, 20, Z, checkpoint=checkpoint,
                                   exptol=1e-8, krylovdim=20)
    h.synchronize()
    t_grad = _t.perf_counter() - t0
    checks = {}
    for site in fd_sites:
        i = site - 1
        hp, hm = hs.copy(), hs.copy()
        hp[i] += 1e-5
        hm[i] -= 1e-5
        fd = (forward(hp) - forward(hm)) / 2e-5
        checks["h_%d" % site] = {"adjoint": float(g[i]), "central_fd": fd,
                                 "abs_err": abs(g[i] - fd),
                                 "rel_err": abs(g[i] - fd) / max(abs(fd), 1e-300)}
    out = {"steps": nsteps, "checkpoint": checkpoint, "blocks": -(-nsteps // checkpoint),
           "value_Z20": val, "value_forward_only": v0,
           "grad_norm": float(np.linalg.norm(g)), "grad": [float(x) for x in g],
           "s_forward": t_fwd, "s_value_and_gradient": t_grad,
           "gradient_over_forward": t_grad / t_fwd, "fd_checks": checks,
           "fd_max_abs_err_over_grad_norm": max(c["abs_err"] for c in checks.values()) /
           float(np.linalg.norm(g))}
    if mixed:
        h.synchronize()
        t0 = _t.perf_counter()
        v32, g32 = AD.tfi_field_gradient(hs, psi, -0.05j, nsteps, 20, Z, checkpoint=checkpoint,
                                         exptol=1e-8, krylovdim=20, precision="tf32x3")
        h.synchronize()
        out["tf32x3"] = {"s_value_and_gradient": _t.perf_counter() - t0,
                         "value_minus_fp64": v32 - val,
                         "grad_rel_err_vs_fp64": float(np.linalg.norm(g32 - g) /
                                                       np.linalg.norm(g))}
    return out


def ed_heff_case(args):
    """The device ED operator alone: ac_prime at the centre of an ExactFiniteMPS of the
    XXZ chain (L = args.ed_heff sites; at L=20 the centre is 512 x 2 x 1024 with
    environments 512 x 5 x 512 and 1024 x 5 x 1024), FP64, seeded random x.  Warm-up
    applications, then timed ones; its FP64 GEMMs are the process's only gemm_kernel
    launches after the environment build, which is what an ncu capture with
    -k regex:gemm_kernel -s <n> needs."""
    import time as _t
    import finitemptools_gb300 as fm
    h = fm.default_handle()
    L = args.ed_heff
    hx = fm.heisenberg_xxz_mpo()
    psi = fm.ExactFiniteMPS.random([2] * L, rng=np.random.default_rng(L), handle=h)
    left, right, Wc = fm.init_h_center(hx, psi)
    op = fm.HeffOp("ac", left, right, W1=Wc)
    x = psi[psi.center]
    y = fm.DeviceTensor(x.shape, np.float64, h)
    for _ in range(args.warmup):
        op(x, y)
    h.synchronize()
    t0 = _t.perf_counter()
    for _ in range(args.steps):
        op(x, y)
    h.synchronize()
    ms = 1e3 * (_t.perf_counter() - t0) / args.steps
    Dl, d, Dr = x.shape
    w = Wc.shape[0]
    # pairwise order of ac_prime (derivatives.jl:2-4): L.x, then W, then .R
    flops = 2.0 * Dl * w * Dl * d * Dr + 2.0 * Dl * w * d * w * d * Dr + 2.0 * Dl * d * w * Dr * Dr
    print(json.dumps({"case": "ed_heff", "L": L, "centre": list(x.shape), "w": w,
                      "ms_per_apply": ms, "gflop_per_apply": flops / 1e9,
                      "tflops": flops / (ms / 1e3) / 1e12}), flush=True)


def krylov_exp_case(args):
    """One Krylov exponential of TDVP1 alone: TFI L=40, complex128, D=64 after one FP64
    TDVP1 step (dt=0.05, stepsize -0.05i), the one-site operator at site 20 (w=3), 20
    Krylov vectors, exptol 1e-8 as _tdvp1_leftsweep passes it.  Warm-up calls, then timed
    ones; the timed calls sit between cudaProfilerStart/Stop, which is what an ncu run with
    --profile-from-start off needs."""
    import ctypes
    import finitemptools_gb300 as fm
    from finitemptools_gb300.derivatives import HeffOp
    h = fm.default_handle()
    L, site = 40, 20
    hs, psi = _tfi_start(fm, h, L=L)
    env = fm.environments(fm.FiniteMPO(fm.tfi_mpo(hs), L), psi)
    alg = fm.TDVP1(stepsize=-0.05j, D=64, exptol=1e-8, krylovdim=20, precision="fp64")
    fm.sweep_(env, alg)
    mps, mpo, hstore = env.mps, env.mpo, env.hstorage
    dt = alg.stepsize
    A = mps[site]
    op = HeffOp("ac", hstore[site], hstore[site + 1], W1=mpo[site], precision="fp64",
                dtype=A.dtype)
    tol = alg.exptol / abs(dt / 2)
    for _ in range(max(1, args.warmup)):
        op.exponentiate(dt / 2, A, tol, alg.krylovdim)
    h.synchronize()
    import time as _t
    cuda = ctypes.CDLL("libcuda.so.1")           # cuProfilerStart/Stop: process-wide
    # the exponential reads its Hessenberg matrix back to the host once per Arnoldi cycle,
    # so a host clock around synchronised calls times it as well as device events would
    cuda.cuProfilerStart()
    t0 = _t.perf_counter()
    for _ in range(args.steps):
        op.exponentiate(dt / 2, A, tol, alg.krylovdim)
    h.synchronize()
    ms = (_t.perf_counter() - t0) * 1e3 / args.steps
    cuda.cuProfilerStop()
    print(json.dumps({"case": "krylov_exp", "L": L, "site": site, "shape": list(A.shape),
                      "krylovdim": alg.krylovdim, "ms_per_exponential": ms,
                      "calls": args.steps}), flush=True)


def u1_heff_case(args):
    """The block-sparse two-site H_eff*x alone: legs of the centre bond of an L=64,
    total-Sz=0 chain with bond dimension D (sector dimensions from the product-state
    counts), iid N(0,1) allowed blocks of L, R and x (seeded), Heisenberg MPO, the
    32x32 tile forced (no tuning launches).  Warm-up applications, then timed ones;
    the only grouped launches of the process are these, which is what an ncu capture
    with -k regex:grouped_kernel -s <warmup> needs."""
    import finitemptools_gb300 as fm
    from finitemptools_gb300 import DeviceTensor as DT
    from finitemptools_gb300.u1 import U1HeffOp, mpo_channel_charges, random_u1_tensors
    h = fm.default_handle()
    h.set_tuning(1)
    L, N, D = 64, 32, args.u1_heff
    _, spaces = random_u1_tensors(L, N, D, (0, 1), 1)
    site = L // 2
    Vl, Vr = spaces[site - 1], spaces[site + 1]
    Ws = fm.heisenberg_xxz_mpo().site_tensors(L)
    qw = mpo_channel_charges(Ws, (0, 1))
    rng = np.random.default_rng(64)

    def env(V, q):
        bq = V.basis_charges()
        mask = bq[:, None, None] == bq[None, None, :] + np.asarray(q)[None, :, None]
        return DT.from_numpy(rng.standard_normal((V.dim, len(q), V.dim)) * mask, h)

    Lm, Rm = env(Vl, qw[site]), env(Vr, qw[site + 2])
    op = U1HeffOp(Lm, Rm, Ws[site - 1], Ws[site], Vl, Vr, (0, 1), (0, 1), qw[site], qw[site + 1],
                  qw[site + 2])
    x = DT.from_numpy(rng.standard_normal(op.n), h)
    y = DT((op.n,), np.float64, h)
    for _ in range(args.warmup):
        op(x, y)
    h.synchronize()
    h.profile(True)
    for _ in range(args.steps):
        op(x, y)
    n, ms = h.profile_read(4)
    h.profile(False)
    ms = ms / max(n, 1)
    print(json.dumps({"case": "u1_heff", "L": L, "D": D, "left_leg": list(Vl.dims),
                      "right_leg": list(Vr.dims), "n_packed": op.n, "flops": op.flops(),
                      "ms": ms, "gflops": op.flops() / (ms * 1e-3) / 1e9, "tile": op.tile(),
                      "launches": n}), flush=True)


def config_dict(args, prec):
    return {"workload": "two-site H_eff*x (ac2_prime), Heisenberg Schur MPO w=5, "
                        "x[D,2,2,D], L/R[D,5,D] iid N(0,1) symmetrised",
            "D": args.D, "w": W_MPO, "d": D_PHYS, "precision": prec,
            "flops_per_step": flops_ac2(args.D), "seed": 2024,
            "l2": "L2 flushed (256 MB write) between timed steps",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--D", type=int, default=2048)
    ap.add_argument("--precision", default="fp64_tc",
                    choices=["fp64_tc", "fp64", "tf32x3", "tf32", "bf16"])
    ap.add_argument("--no-table", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-dmrg", action="store_true")
    ap.add_argument("--no-u1", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--no-next", action="store_true")
    ap.add_argument("--config3", action="store_true",
                    help="only the J1-J2 L=100 D=1024 mixed-vs-FP64 comparison with both forms' "
                         "full ramps (sweep times and energies of both), printed as JSON")
    ap.add_argument("--config5", action="store_true",
                    help="only the differentiable TDVP1 run as configured: TFI L=40, D=64, "
                         "100 steps, checkpoint every 10, gradient of <Z_20> with respect to "
                         "all 40 fields, central differences on h_20, h_21, h_1, h_40")
    ap.add_argument("--ed-heff", type=int, default=0, metavar="L",
                    help="time the exact-diagonalisation operator of an L-site XXZ chain alone")
    ap.add_argument("--krylov-exp", action="store_true",
                    help="one TDVP1 Krylov exponential (TFI L=40 D=64, site 20) alone")
    ap.add_argument("--u1-heff", type=int, default=0, metavar="D",
                    help="only time the block-sparse H_eff*x of an L=64, Sz=0 centre bond "
                         "with bond dimension D (profiling case) and exit")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.u1_heff:
        return u1_heff_case(args)
    if args.krylov_exp:
        return krylov_exp_case(args)
    if args.ed_heff:
        return ed_heff_case(args)

    import torch
    import finitemptools_gb300 as fm
    from finitemptools_gb300 import DeviceTensor as DT
    from finitemptools_gb300._native import lib, PREC

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    # one explicit stream shared by torch (events, L2 flush) and libfmpt
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    h = fm.Handle(local)
    h.set_stream(stream.cuda_stream)

    if args.config3:
        res = dmrg_section(h, fm, full3=True, only3=True)
        print(json.dumps({"config3": res}), flush=True)
        return
    if args.config5:
        res = tdvp_grad_section(h, fm, nsteps=100, checkpoint=10, fd_sites=(20, 21, 1, 40),
                                mixed=False)
        print(json.dumps({"config5": res}), flush=True)
        return
    D, prec = args.D, args.precision
    x, L, R, W = workload(D)
    xd, Ld, Rd = DT.from_numpy(x, h), DT.from_numpy(L, h), DT.from_numpy(R, h)
    op = fm.HeffOp("ac2", Ld, Rd, W1=W, W2=W, precision=prec)
    y = DT(x.shape, np.float64, h)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()

    for _ in range(args.warmup):
        op(xd, out=y)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        h.profile(True)
        h.profile_read(0), h.profile_read(1), h.profile_read(2), h.profile_read(3)
        n_launch0 = h.launch_count()
        for k in range(args.steps):
            flush.zero_()                      # evict L2 before every step (not timed)
            ev[k][0].record(stream)
            op(xd, out=y)
            ev[k][1].record(stream)
        barrier()
        n_launch = h.launch_count() - n_launch0
        tc_n, tc_ms = h.profile_read(0)
        mid_n, mid_ms = h.profile_read(2)
        cv_n, cv_ms = h.profile_read(3)
        h.profile(False)
        time.sleep(0.25)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_ms = sum(step_ms)
    if pg:
        t = torch.tensor([tot_ms], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        tot_ms = float(t[0])
    F = flops_ac2(D)
    value = F * args.steps * ws / (tot_ms / 1e3) / 1e12
    clocks = clk.summary()

    # ---- roofline of the dominant kernel (the tcgen05 GEMM: 2 launches per step,
    # each 2*w*d^2*D^3 algorithmic flops)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    if prec == "bf16":
        peak, peak_note = peaks.get("bf16_tflops", 1900.0), "bf16_tflops (burst) of measured"
    elif prec == "fp64_tc":
        # the FP64-accurate GEMM forms 45 BF16 digit products per FP64 multiply-add: the FP64
        # rate it can reach is the measured BF16 peak / 45
        peak = peaks.get("bf16_tflops", 1900.0) / OZ_PRODUCTS
        peak_note = "bf16_tflops (burst) of measured / %d digit products" % OZ_PRODUCTS
    elif prec in ("tf32", "tf32x3"):
        peak = peaks.get("bf16_tflops", 1900.0) / 2
        peak_note = "half of measured bf16_tflops (dense TF32 rate is half of BF16)"
    else:
        peak, peak_note = None, None
    roof = None
    if tc_n:
        per_launch = 2 * W_MPO * D_PHYS ** 2 * D ** 3
        achieved = per_launch / (tc_ms / tc_n / 1e3) / 1e12
        if prec == "tf32x3":
            achieved *= 1.0          # algorithmic flops only (3 products are not credited)
        kname = ("oz_gemm_pair (tcgen05 BF16 digit products of the FP64-accurate GEMM)"
                 if prec == "fp64_tc" else "tc_gemm (tcgen05 %s)" % prec)
        roof = {"bound": "tensor", "kernel": kname,
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None, "peak_source": peak_note,
                "traffic": NCU_TRAFFIC.get((prec, D)), "launches": tc_n,
                "avg_launch_ms": tc_ms / tc_n,
                "share_of_step": tc_ms / tot_ms if tot_ms else None,
                "other_kernels_ms_per_step": {"mpo_step": mid_ms / args.steps,
                                              "convert": cv_ms / args.steps}}
        if prec == "fp64_tc":
            roof["bf16_mma_tflops"] = achieved * OZ_PRODUCTS
            roof["unit_note"] = ("achieved: algorithmic FP64 flops (2 w d^2 D^3 per launch) per "
                                 "second; bf16_mma_tflops: the digit-product MMA work per second")
        if prec == "bf16" and rank == 0:
            roof["cublas_same_shapes"] = cublas_same_shapes(D, stream)

    # ---- end to end through the C ABI with host buffers (pinned)
    e2e = None
    if rank == 0 or ws > 1:
        hx = torch.from_numpy(x.ravel(order="F").copy()).pin_memory()
        hL = torch.from_numpy(L.ravel(order="F").copy()).pin_memory()
        hR = torch.from_numpy(R.ravel(order="F").copy()).pin_memory()
        hy = torch.empty(x.size, dtype=torch.float64).pin_memory()
        Wb = np.ascontiguousarray(W.ravel(order="F"))
        LIB = lib()

        def e2e_step():
            # host x/L/R in, host y out: fmpt_ac2_prime_host pipelines the copies (L, x, R
            # on a copy stream) with the conversions, GEMM 1 and the MPO step
            h.check(LIB.fmpt_ac2_prime_host(h.ptr, 0, PREC[prec], hx.data_ptr(), Wb.ctypes.data,
                                            Wb.ctypes.data, hL.data_ptr(), hR.data_ptr(),
                                            hy.data_ptr(), D, 2, 2, D, W_MPO, W_MPO, W_MPO))

        for _ in range(2):
            e2e_step()
        n_e2e = max(3, min(args.steps, 10))
        t_e2e = []
        for _ in range(n_e2e):
            flush.zero_()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            e2e_step()
            b.record(stream)
            torch.cuda.synchronize()
            t_e2e.append(a.elapsed_time(b))
        e_ms = sum(t_e2e) / len(t_e2e)
        e2e = {"value": F / (e_ms / 1e3) / 1e12, "unit": UNIT, "ms_per_step": e_ms,
               "h2d_bytes_per_step": (x.size + L.size + R.size) * 8,
               "d2h_bytes_per_step": x.size * 8,
               "path": "fmpt_ac2_prime_host through the C ABI: pinned host x/L/R in, y out"}

    # ---- every precision form at every size (D = 256 .. 2048), rank 0 only
    table = None
    if rank == 0 and not args.no_table:
        table = []
        for Dt in (256, 512, 1024, 2048):
            xt, Lt, Rt, Wt = workload(Dt, seed=7)
            xdt, Ldt, Rdt = DT.from_numpy(xt, h), DT.from_numpy(Lt, h), DT.from_numpy(Rt, h)
            ref = None
            for p in ("fp64", "fp64_tc", "tf32x3", "tf32", "bf16"):
                opt = fm.HeffOp("ac2", Ldt, Rdt, W1=Wt, W2=Wt, precision=p)
                yt = opt(xdt)
                reps = 2 if (p == "fp64" and Dt >= 1024) else 5
                for _ in range(1):
                    opt(xdt, out=yt)
                ts = []
                for _ in range(reps):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    opt(xdt, out=yt)
                    b.record(stream)
                    torch.cuda.synchronize()
                    ts.append(a.elapsed_time(b))
                ms = min(ts)
                yn = yt.numpy()
                if p == "fp64":
                    ref = yn
                    err = 0.0
                else:
                    err = float(np.linalg.norm(yn - ref) / np.linalg.norm(ref))
                table.append({"D": Dt, "dtype": p, "ms": ms,
                              "tflops": flops_ac2(Dt) / (ms / 1e3) / 1e12,
                              "rel_frobenius_err_vs_fp64": err})
                del opt, yt
        fp64 = {r["D"]: r["ms"] for r in table if r["dtype"] == "fp64"}
        for r in table:
            r["speedup_vs_fp64"] = fp64[r["D"]] / r["ms"]

    dmrg = None
    if rank == 0 and not args.no_dmrg:
        dmrg = dmrg_section(h, fm)
    u1 = None
    if rank == 0 and not args.no_u1:
        u1 = u1_section(h, fm)
    tdvp = tgrad = None
    if rank == 0 and not args.no_grad:
        tdvp = tdvp_section(h, fm)
        tgrad = tdvp_grad_section(h, fm)

    nxt = None
    if rank == 0 and not args.no_next:
        nxt = next_rows_section(h, fm)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(D)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec in ("fp64", "fp64_tc") else prec, "data": "synthetic",
            "config": config_dict(args, prec), "clocks": clocks, "e2e": e2e,
            "gpu_launches": n_launch, "roofline": roof, "cpu_baseline": cpu,
            "per_dtype": table, "dmrg": dmrg, "u1": u1, "tdvp1": tdvp, "tdvp_gradient": tgrad,
            "next_rows": nxt,
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
