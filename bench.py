"""Benchmark of the perturbation + line-of-sight path on the full ΛCDM + massive-ν workload.

Workload ("LCDM+nu_m, lγ=30, 1000 k, 2000 τ, TT/TE/EE to l=2500"): one massive neutrino
(m = 0.06 eV, 5 momentum bins, l_max 10) plus N_eff = 2.0328 massless; photon l_max 30;
1000 modes log-spaced over 1e-5..5 h/Mpc; sources on a 2000-point τ grid; C_l TT, TE, EE to
l = 2500 through the line-of-sight quadrature with tabulated spherical Bessel functions
(l sampled at 200 log-spaced values and splined to every l, as the reference's spectrum_cmb does).
Inputs are synthetic (a fixed parameter set); there is no dataset.

A step is one complete cosmology: background solve, 1000 perturbation modes, source
k-interpolation, line-of-sight integrals and C_l.  value = k-mode solves/s from CUDA-event device
time of the pipeline (inputs resident on the device); e2e = the same through the public
spectrum_cmb call with host buffers (background solve and host<->device copies included).

--impl reference: the CPU restatement of the reference's algorithm (the oracle: Rodas5P with a
sparse LU, the same k-interpolation, line of sight and C_l; the Julia reference cannot run on these
machines) on all host cores, the whole workload once per step.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "symboltz.jl_gb300"), os.path.join(ROOT, "oracle")]

H_PLANCK = 0.67
PARAMS = dict(h=H_PLANCK, Omega_c=0.12 / H_PLANCK**2, Omega_b=0.022 / H_PLANCK**2, T0=2.7255, Neff=2.0328, YHe=0.245,
              ln_As1e10=3.04, ns=0.965, m_nu_eV=0.06, N_nu=1.0)
MODEL = dict(lmax_gamma=30, lmax_nu=10, lmax_h=10, nx=5)
NK, NTAU, LMAX = 1000, 2000, 2500
METRIC = "k-mode solves/s (cosmologies/s) at <=1e-4 rel C_l err"
# Lazy-refinement threshold of the timed configuration: the later stages of a step skip their FP64
# refinement when stage 1's first correction is below 1e-2 of the error weights.  Measured on this
# workload at the tolerances below: C_l 7.4e-6 from the all-FP64 solver, 1.5e-5 from a converged
# solution, 2.01 s per spectrum (2.90 s at 1e-4, 2.26 s at 1e-3).  The library default (1e-5) keeps
# pointwise sources at the fully refined accuracy; the accuracy field of every run checks the C_l.
REFINE_SKIP_CL = 1e-2
# Integrator tolerances of the timed configuration.  The reference's defaults (rtol = atol = 1e-5,
# src/solve.jl:383) leave the low-l C_l about 1e-2 from a converged solution, and two integrations
# at those settings (mixed against FP64, GPU against the oracle) can end up 1e-3 apart.  The low-l
# error is set by atol (the shear of superhorizon modes is small in absolute terms but enters Ψ
# divided by k²): at rtol 1e-6 every l is within 1.1e-4 of a converged solution for atol 1e-7 and
# within 1.3e-5 for atol 3e-8 (oracle, Rodas5P, against rtol = atol = 1e-9).
PT_RTOL, PT_ATOL = 1e-6, 3e-8
# DRAM bytes (read + write) of the spectrum's perturbation launch: one ncu pass of
# dram__bytes_read.sum + dram__bytes_write.sum on `bench.py --profile-case los` (4.15 MB + 2.53 MB)
PT_LAUNCH_DRAM_BYTES = 6.68e6


def workload_grids(S, prob):
    bg = prob.solvebg()
    ks = S.k_from_hMpc(S.loggrid(1e-5, 5.0, length=NK))
    t = bg.t(0)
    t = t[t >= 1e-2]
    taus = t[0] + (bg.tau0[0] - t[0]) * S.cosgrid(0.0, 1.0, length=NTAU)
    ls = np.unique(np.round(np.exp(np.linspace(np.log(2), np.log(LMAX), 200))).astype(np.int32))
    return ks, taus, ls


def fp64_flops_per_step(n, refined_stages):
    """FP64 flops of one Rodas5P step as implemented (2 flops per FMA), counting only the work done
    in FP64: 8 operator products (the stage inputs of stages 2-8 and f at the step end; 11 flops per
    row + 60 for the metric functionals), ∂f/∂τ (15 per row + 100), one refinement residual per
    refined stage (operator product + 2 per row), the stage combinations and error norm (121 per
    row: Σ A U for stages 2-6, Σ C U / h and the ∂f/∂τ terms for stages 2-8, y1, the weighted norm),
    the factorisation inputs (4 per row), the coefficients at the five later stage times (~4.0k) and
    the step-size controller (~100).  In mixed precision the factorisation and stage solves are FP32
    and not counted; with lazy refinement one stage per step is refined at least."""
    F_mv = 11 * n + 60
    return 8 * F_mv + (15 * n + 100) + 121 * n + 4 * n + 4000 + 100 + refined_stages * (F_mv + 2 * n)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200", "-i", "0"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            sm = [float(r[1]) for r in rows]
            mx = float(rows[0][2])
            reasons = set()
            for r in rows:
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(name)
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(rows)}
        except Exception as e:  # noqa: BLE001
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def fp64_peak_tflops(torch):
    """FP64 throughput measured here with a cuBLAS DGEMM (MEASURED_PEAKS.json holds no FP64 figure)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e9
    for _ in range(5):
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2 * n**3 / best / 1e12


def run_ours(args):
    import torch
    import symboltz as S

    assert torch.cuda.is_available(), "bench needs a GPU"
    from symboltz import replicas as R
    rank, world = R.init("nccl")  # replicas: each rank runs the whole workload, no data-path collective
    M = S.ΛCDM(lmax_gamma=MODEL["lmax_gamma"], lmax_nu=MODEL["lmax_nu"], lmax_h=MODEL["lmax_h"], nx=MODEL["nx"])
    prob = S.CosmologyProblem(M, PARAMS, precision=args.precision, refine_skip=REFINE_SKIP_CL, pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
    ks, taus, ls = workload_grids(S, prob)
    jl = S.SphericalBesselCache(ls)
    kinterp = S.CubicSplineInterpolator(ks, f=np.log)
    stream = torch.cuda.current_stream()
    S._lib.lib().sbz_problem_set_stream(prob._h, S._lib.C.c_void_p(stream.cuda_stream))
    lall = np.arange(2, LMAX + 1)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def step():
        prob.bg = None  # full cosmology each step: background + tables + modes + LOS + C_l
        return S.spectrum_cmb(["TT", "TE", "EE"], prob, jl, lall, kinterp=kinterp, taus=taus, return_status=True,
                              normalization="Dl")

    for _ in range(args.warmup):
        Dl, st = step()
    assert np.all(st == 0), f"failed modes: {np.count_nonzero(st)}"
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dev_ms, e2e_ms, pt_ms, phases = [], [], [], []
    steps_total = 0
    with Clocks(args.clocks_log) as ck:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            R.barrier()
            e0.record(stream)
            Dl, st = step()
            e1.record(stream)
            torch.cuda.synchronize()
            e2e_ms.append(e0.elapsed_time(e1))
            t = S.timings(prob)
            phases.append(t)
            dev_ms.append(t["perturbations"] + t["kinterp"] + t["los"] + t["cl"])
            pt_ms.append(t["perturbations"])
    # accuracy of the timed configuration (outside the timed region), per l range, TE relative to
    # sqrt(TT EE): against an all-FP64 GPU solve at the same tolerances, against a converged all-FP64
    # GPU solve (rtol = atol = 1e-9), and against the oracle on the host (the CPU baseline's run,
    # same tolerances and grids)
    def rel_by_range(D, R):
        den = [np.abs(R[:, 0]), np.sqrt(np.abs(R[:, 0] * R[:, 2])), np.abs(R[:, 2])]
        out = {}
        for lo, hi in ((2, LMAX), (2, 29), (30, LMAX)):
            sel = (lall >= lo) & (lall <= hi)
            rel = {}
            for i, m in enumerate(("TT", "TE", "EE")):
                r = np.abs(D[sel, i] - R[sel, i]) / den[i][sel]
                rel[m] = {"max": float(r.max()), "at_l": int(lall[sel][np.argmax(r)]), "median": float(np.median(r))}
            out[f"l{lo}_{hi}"] = rel
        return out

    accuracy = {"tolerances": {"pt_rtol": PT_RTOL, "pt_atol": PT_ATOL}}
    if args.precision == "mixed":
        p64 = S.CosmologyProblem(M, PARAMS, precision="fp64", pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
        Dl64, st64 = S.spectrum_cmb(["TT", "TE", "EE"], p64, jl, lall, kinterp=kinterp, taus=taus, return_status=True,
                                    normalization="Dl")
        accuracy["vs_fp64_gpu"] = rel_by_range(Dl, Dl64)
        accuracy["fp64_failed_modes"] = int(np.count_nonzero(st64))
        # the all-FP64 kernel on the same modes (one untimed-loop call: CUDA-event phase time)
        accuracy["fp64_perturbations_ms"] = round(float(S.timings(p64)["perturbations"]), 1)
    pconv = S.CosmologyProblem(M, PARAMS, precision="fp64", pt_rtol=1e-9, pt_atol=1e-9, maxiters=10**7)
    Dlc, stc = S.spectrum_cmb(["TT", "TE", "EE"], pconv, jl, lall, kinterp=kinterp, taus=taus, return_status=True,
                              normalization="Dl")
    accuracy["vs_converged_fp64_gpu_1e-9"] = rel_by_range(Dl, Dlc)
    accuracy["converged_failed_modes"] = int(np.count_nonzero(stc))
    # per-mode step counts for the roofline (one extra solve of the same modes)
    out, stt, stp = S.solvept(prob, ks, prob.opts.tau_ini, saveat=taus, output="sources")
    steps_total = int(stp.sum())
    dev = float(np.sum(dev_ms))
    e2e = float(np.sum(e2e_ms))
    dev, e2e = R.reduce_over_ranks([dev, e2e], op="max")
    K = args.steps
    tau0 = float(prob.solvebg().tau0[0])
    nk_fine = int(len(S.lingrid(float(ks.min()), float(ks.max()), step=np.pi / tau0)))
    value = world * NK * K / (dev / 1e3)
    e2e_v = world * NK * K / (e2e / 1e3)
    peaks = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch)
    fl = fp64_flops_per_step(prob.nstate, 1 if args.precision == "mixed" else 0)
    pt_avg = float(np.mean(pt_ms)) / 1e3
    achieved = steps_total * fl / pt_avg / 1e12
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "k-modes/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(dev / K, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+f32",
        "data": "synthetic (fixed cosmological parameters)",
        "config": {"workload": "LCDM+massive-nu, l_gamma=30, 1000 k log 1e-5..5 h/Mpc, 2000 tau, TT/TE/EE to l=2500",
                   "n_state": prob.nstate, "nk": NK, "ntau": NTAU, "nl_sampled": int(len(ls)), "nk_fine": nk_fine,
                   "precision": args.precision, "pt_rtol": prob.opts.pt_rtol, "pt_atol": prob.opts.pt_atol,
                   "refine_skip": REFINE_SKIP_CL,
                   "l2": "flushed (256 MB write) between steps"},
        "cosmologies_per_s": round(world * K / (dev / 1e3), 4),
        "e2e": {"value": round(e2e_v, 2), "unit": "k-modes/s", "cosmologies_per_s": round(world * K / (e2e / 1e3), 4),
                "h2d_bytes_per_step": int(8 * (3 * NK + 2 * NTAU + 2 * len(ls))), "d2h_bytes_per_step": int(8 * 3 * len(ls) + 4 * NK)},
        "phases_ms": {k: round(float(np.mean([p[k] for p in phases])), 3) for k in phases[0]},
        "roofline": {"bound": "fp64", "achieved": round(achieved, 5), "peak": round(fp64_peak, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / fp64_peak, 5),
                     # dram__bytes_read.sum + dram__bytes_write.sum of one full pt_kernel launch of this
                     # workload (ncu, profiles/launches_bench_lcdm_massive_nu.md): 1.98 MB + 2.66 MB; the
                     # coefficient tables stay in L1/L2, the kernel is FP64-latency bound
                     "traffic": PT_LAUNCH_DRAM_BYTES,
                     "kernel": "pt_kernel (perturbation modes)", "flops_per_step": fl, "steps_per_launch": steps_total,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)",
                     # the same launch against the HBM roofline: measured traffic over its CUDA-event time
                     "hbm": {"achieved_gbs": round(PT_LAUNCH_DRAM_BYTES / pt_avg / 1e9, 6), "peak_gbs": peaks.get("hbm_gbs"),
                             "frac": round(PT_LAUNCH_DRAM_BYTES / pt_avg / 1e9 / peaks["hbm_gbs"], 8) if peaks.get("hbm_gbs") else None}},
        "accuracy": accuracy,
        "gpu_launches": int(K * 6),
        "clocks": ck.summary(),
        "hbm_peak_gbs": peaks.get("hbm_gbs"),
    }
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"], Dl_cpu = cpu_baseline(taus=taus, return_dl=True)
        line["accuracy"]["vs_oracle_cpu"] = rel_by_range(Dl, Dl_cpu)
    if rank == 0:
        print(json.dumps(line), flush=True)
    R.finalize()


def cpu_baseline(taus=None, return_dl=False):
    """The reference's algorithm restated on the host (the oracle library): background, all NK
    perturbation modes with Rodas5P and a sparse LU of W (minimum-degree order, threshold pivoting:
    the reference's KLU path, src/solve.jl:314-341) over every host core (OpenMP over modes, as the
    reference threads over k), then the same k-interpolation, line-of-sight integrals, C_l
    k-integral and l-spline as the GPU pipeline.  The whole workload is timed once.  taus: the
    line-of-sight grid (default: the oracle background's own, by the workload's rule)."""
    import oracle as O
    ncores = os.cpu_count() or 1
    O.set_threads(ncores)
    m = dict(lmax_g=MODEL["lmax_gamma"], lmax_nu=MODEL["lmax_nu"], lmax_h=MODEL["lmax_h"], nx=MODEL["nx"], Hswitch=1, Heswitch=6,
             reionization=1)
    ks = np.exp(np.linspace(np.log(1e-5), np.log(5.0), NK)) * (299792458.0 / 1e5)
    ks[0], ks[-1] = 1e-5 * (299792458.0 / 1e5), 5.0 * (299792458.0 / 1e5)
    ls = np.unique(np.round(np.exp(np.linspace(np.log(2), np.log(LMAX), 200))).astype(np.int32))
    t0 = time.perf_counter()
    bg = O.Background(PARAMS, m, pt_rtol=PT_RTOL, pt_atol=PT_ATOL, alg="rodas5p", linsolve="sparse")
    if taus is None:
        t = bg.t[bg.t >= 1e-2]
        taus = t[0] + (bg.tau0 - t[0]) * (1 - np.cos(np.pi * np.linspace(0, 0.5, NTAU)))
    Dl, parts = O.spectrum_cmb_kspline(bg, ks, taus, O.BesselCache(ls), np.arange(2, LMAX + 1), return_parts=True)
    total = time.perf_counter() - t0
    info = {"value": round(NK / total, 3), "unit": "k-modes/s", "cores": ncores, "kind": "port",
            "sample": f"the whole workload once: background, all {NK} modes (Rodas5P, sparse LU with minimum-degree order "
                      f"and threshold pivoting, rtol {PT_RTOL:g} atol {PT_ATOL:g}), k-interpolation to {parts['nk_fine']} k, "
                      f"line of sight, C_l TT/TE/EE and l-spline; {int(np.count_nonzero(parts['status']))} failed modes",
            "seconds": round(total, 3)}
    return (info, Dl) if return_dl else info


def run_reference(args):
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    vals = []
    for _ in range(args.warmup):
        pass  # the CPU port has no warm-up effects beyond the first call
    for _ in range(max(1, args.steps)):
        vals.append(cpu_baseline())
    v = float(np.median([x["value"] for x in vals]))
    cb = dict(vals[0]); cb["value"] = round(v, 3)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "k-modes/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (fixed cosmological parameters)",
            "config": {"workload": "LCDM+massive-nu, l_gamma=30, 1000 k log 1e-5..5 h/Mpc, 2000 tau, TT/TE/EE to l=2500"},
            "cpu_baseline": cb, "e2e": {"value": round(v, 3), "unit": "k-modes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_workload(ncosmo=256, seed=0):
    """256 cosmologies drawn uniformly from the parameter box (numpy PCG64, fixed seed): h in
    [0.6, 0.8], ω_c in [0.10, 0.14], ω_b in [0.020, 0.024], n_s in [0.92, 1.0], ln(1e10 A_s) in
    [2.9, 3.2], Σm_ν in [0.06, 0.3] eV (one massive species of that mass); each with its own
    log-spaced k grid of U{200..800} modes over 1e-5..5 h/Mpc."""
    rng = np.random.default_rng(seed)
    pars = []
    for _ in range(ncosmo):
        h = rng.uniform(0.6, 0.8)
        oc, ob = rng.uniform(0.10, 0.14), rng.uniform(0.020, 0.024)
        ns, las, mnu = rng.uniform(0.92, 1.0), rng.uniform(2.9, 3.2), rng.uniform(0.06, 0.3)
        pars.append(dict(h=h, Omega_c=oc / h**2, Omega_b=ob / h**2, T0=2.7255, Neff=2.0328, YHe=0.245, ln_As1e10=las, ns=ns,
                         m_nu_eV=mnu, N_nu=1.0))
    nks = rng.integers(200, 801, size=ncosmo)
    return pars, nks


def run_batched(args):
    """Batched P(k): every mode of every cosmology in one perturbation launch (Δm output), the
    launch shape picked by the autotuner for each precision, mixed precision against all-FP64."""
    import torch
    import symboltz as S
    assert torch.cuda.is_available(), "bench needs a GPU"
    pars, nks = batched_workload()
    M = S.ΛCDM(lmax_gamma=MODEL["lmax_gamma"], lmax_nu=MODEL["lmax_nu"], lmax_h=MODEL["lmax_h"], nx=MODEL["nx"])
    ks = np.concatenate([S.k_from_hMpc(S.loggrid(1e-5, 5.0, length=int(n))) for n in nks])
    cos = np.concatenate([np.full(int(n), i) for i, n in enumerate(nks)])
    ti = lambda k: np.minimum(1e-2 / k, 1e-4)  # noqa: E731  (spectrum_matter's rule, fourier.jl:76-81)
    res = {}
    for prec in ("mixed", "fp64"):  # each precision runs the launch shape the autotuner picks for it
        skip = REFINE_SKIP_CL if prec == "mixed" else None
        prob = S.CosmologyProblem(M, pars, precision=prec, pt_rtol=PT_RTOL, pt_atol=PT_ATOL, refine_skip=skip)
        t0 = time.perf_counter()
        bg = prob.solvebg()
        t_bg = time.perf_counter() - t0
        assert np.all(bg.status == 0)
        tune = S.autotune(prob, ks, ti, output="delta_m", cosmo=cos)
        times = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            dm, st, stp = S.solvept(prob, ks, ti, output="delta_m", cosmo=cos)
            times.append(time.perf_counter() - t0)
        res[prec] = dict(s=min(times), dm=dm, failed=int(np.count_nonzero(st)), steps=int(stp.sum()), bg_s=t_bg, tune=tune)
    rel = np.abs(res["mixed"]["dm"] ** 2 - res["fp64"]["dm"] ** 2) / res["fp64"]["dm"] ** 2
    hi = ks >= S.k_from_hMpc(1e-4)
    n = len(ks)
    line = {"metric": "k-mode solves/s (batched P(k))", "value": round(n / res["mixed"]["s"], 2), "unit": "k-modes/s",
            "workload": f"batched: {len(pars)} cosmologies from the parameter box, U{{200..800}} k each ({n} modes), P(k) at z=0",
            "config": {"model": "LCDM+massive-nu, l_gamma=30, n_state=133", "seed": 0, "launches": 1},
            "mixed": {"s": round(res["mixed"]["s"], 3), "kmodes_per_s": round(n / res["mixed"]["s"], 1), "failed": res["mixed"]["failed"],
                      "steps": res["mixed"]["steps"], "autotune": {"chosen": [res["mixed"]["tune"]["warps_per_mode"], res["mixed"]["tune"]["blocks_per_sm"]],
                                                                   "candidates_ms": {str(k): round(v, 1) for k, v in res["mixed"]["tune"]["candidates_ms"].items()}}},
            "fp64": {"s": round(res["fp64"]["s"], 3), "kmodes_per_s": round(n / res["fp64"]["s"], 1), "failed": res["fp64"]["failed"],
                     "steps": res["fp64"]["steps"], "autotune": {"chosen": [res["fp64"]["tune"]["warps_per_mode"], res["fp64"]["tune"]["blocks_per_sm"]],
                                                                 "candidates_ms": {str(k): round(v, 1) for k, v in res["fp64"]["tune"]["candidates_ms"].items()}}},
            "speedup_mixed_over_fp64": round(res["fp64"]["s"] / res["mixed"]["s"], 3),
            "pk_rel_mixed_vs_fp64": {"max": float(rel.max()), "median": float(np.median(rel)), "max_k_ge_1e-4_hMpc": float(rel[hi].max())},
            "tolerances": {"pt_rtol": PT_RTOL, "pt_atol": PT_ATOL, "refine_skip_mixed": REFINE_SKIP_CL},
            "background_s": round(res["mixed"]["bg_s"], 3)}
    print(json.dumps(line), flush=True)


def mlp_step_bytes(batch=65536, nin_pad=64, width=512, nhidden=4, nout_pad=64, nparams=794631):
    """Algorithmic HBM bytes of one training step of the surrogate (each array read or written once
    per kernel that touches it): forward layers read X_{l-1} and write X_l, Z_l and X_lᵀ (BF16), the
    output layer writes FP32 Y; the loss reads Y and writes dY, dYᵀ; each backward dX GEMM reads its
    output gradient and Z and writes dZ, dZᵀ; each weight-gradient GEMM reads dZᵀ and Xᵀ; Adam reads
    and writes p, m, v and reads the gradient (FP32) and writes two BF16 copies of the weights."""
    a, w = 2 * batch, width
    fwd = a * nin_pad + 3 * a * w + (nhidden - 1) * (a * w + 3 * a * w) + a * w + 4 * batch * nout_pad
    loss = 4 * batch * nout_pad + 2 * a * nout_pad
    dx = (a * nout_pad + a * w + 2 * a * w) + (nhidden - 1) * (a * w + a * w + 2 * a * w)
    dw = (a * w + a * nout_pad) + (nhidden - 1) * (2 * a * w) + (a * w + a * nin_pad)
    adam = nparams * (7 * 4 + 2 * 2)
    gather = batch * (8 * 4 + 7 * 4) + 2 * a * nin_pad
    return fwd + loss + dx + dw + adam + gather


def run_surrogate(args):
    """Learned part end to end (cfg4 training, cfg5 mixed workload).

    Training: scrambled-Sobol cosmologies of the box, solved in shards of 64 by the batched GPU
    solver at the workload's tolerances (perturbation factors on 400 k over 1e-4..0.5 h/Mpc × 500 τ),
    a random subset of each cosmology's points streamed into a flat SBZTRN01 training-set file, two
    MLP members (10 → 4×512 SiLU → 7, BF16 tcgen05 GEMMs, FP32 accumulation, Adam, batch 65536)
    trained from it; a P(k) surrogate (θ, log k → ln Δ_m², 1e-4..10 h/Mpc) trained on the solver's
    Δ_m.  Held-out accuracy: D_l TT/TE/EE to l = 2500 of held-out cosmologies against the all-FP64
    solver on the same grids, the surrogate alone and with fallback.  Mixed workload: cosmologies
    drawn uniformly from the box, D_l to l = 3000 and P(k) from the surrogates, the cosmologies whose
    ensemble error estimate exceeds the tolerance recomputed by the mixed-precision solver (all of
    them in one launch), cosmologies/s against the plain solver path, fallback rate, and the error
    of a sample against the all-FP64 solver."""
    import torch
    import symboltz as S
    from symboltz import surrogate as SG
    assert torch.cuda.is_available(), "bench needs a GPU"
    M = S.ΛCDM(lmax_gamma=MODEL["lmax_gamma"], lmax_nu=MODEL["lmax_nu"], lmax_h=MODEL["lmax_h"], nx=MODEL["nx"])
    ks = S.k_from_hMpc(S.loggrid(1e-4, 0.5, length=400))
    sur = SG.SourceSurrogate(M, ks, ntau=500, width=512, nhidden=4, batch=65536, seed=0, members=2, pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
    rng = np.random.default_rng(0)
    # ---- training data, streamed shard by shard into a flat training-set file
    os.makedirs(args.workdir, exist_ok=True)
    path = os.path.join(args.workdir, "sbz_train.sbztrn")
    if os.path.exists(path):
        os.remove(path)
    train = SG.sample_box(args.train_cosmologies, seed=0, sobol=True)
    t0 = time.perf_counter()
    keep = args.points_per_cosmology
    for s0 in range(0, len(train), 64):
        th = train[s0:s0 + 64]
        F, taus, vis, _ = sur.solve_factors(th)
        for c, t in enumerate(th):
            X = sur.features(t, taus[c], vis[c])
            Y = sur.to_targets(F[c], ks, vis[c]).reshape(-1, 7)
            idx = rng.choice(len(X), size=min(keep, len(X)), replace=False)
            SG.write_training_set(path, X[idx], Y[idx])
    t_data = time.perf_counter() - t0
    nin, nout, nrows = SG.training_set_info(path)
    X, Y = SG.read_training_set(path)
    # ---- training both members (fit sets the envelope and standardisation from the same data)
    step_s = 1.2e-3
    steps = max(200, int(args.train_seconds / len(sur.nets) / step_s))
    t0 = time.perf_counter()
    losses = sur.fit(X, Y, steps=steps, lr=1e-3, lr_final=1e-5)
    t_train = time.perf_counter() - t0
    mse_train = sur.mse(X[:: max(1, len(X) // 2_000_000)], Y[:: max(1, len(X) // 2_000_000)])
    del X, Y
    flops_step = 3 * 2 * 65536 * (64 * 512 + 3 * 512 * 512 + 512 * 64)
    # P(k) surrogate, trained on the solver's Δ_m at the reference's default tolerances
    kpk = S.k_from_hMpc(S.loggrid(1e-4, 10.0, length=128))
    msur = SG.MatterSurrogate(M, kpk, seed=1)
    t0 = time.perf_counter()
    Xp, Yp = [], []
    for s0 in range(0, args.pk_train_cosmologies, 128):
        xp, yp = msur.dataset(train[s0:min(s0 + 128, args.pk_train_cosmologies)])
        Xp.append(xp); Yp.append(yp)
    msur.fit(np.concatenate(Xp), np.concatenate(Yp).astype(np.float32), steps=4000, lr=1e-3, lr_final=1e-5)
    t_pk = time.perf_counter() - t0
    # ---- held-out accuracy against the all-FP64 solver (same grids and tolerances)
    ls = np.unique(np.round(np.exp(np.linspace(np.log(2), np.log(LMAX), 200))).astype(np.int32))
    lall = np.arange(2, LMAX + 1)
    jl = S.SphericalBesselCache(ls)
    kin = S.CubicSplineInterpolator(ks, f=np.log)
    test = SG.sample_box(args.test_cosmologies, seed=1)

    def solver_spectra(thetas, precision):
        prob = S.CosmologyProblem(M, [SG.box_params(t) for t in thetas], precision=precision, pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
        bg = prob.solvebg()
        taus = np.stack([SG.cmb_taus(bg.t(c), bg.tau0[c], sur.ntau) for c in range(len(thetas))])
        src, st, _ = S.solvept(prob, np.tile(ks, len(thetas)), prob.opts.tau_ini, saveat=taus, output="sources",
                               cosmo=np.repeat(np.arange(len(thetas)), len(ks)))
        src = src.reshape(len(thetas), len(ks), sur.ntau, 3)
        return np.stack([S.spectrum_cmb(["TT", "TE", "EE"], prob, jl, lall, kinterp=kin, taus=taus[c], cosmo=c, normalization="Dl",
                                        sources=src[c]) for c in range(len(thetas))])

    def rel_max(D, R):
        den = [np.abs(R[..., 0]), np.sqrt(np.abs(R[..., 0] * R[..., 2])), np.abs(R[..., 2])]
        return np.stack([np.max(np.abs(D[..., i] - R[..., i]) / den[i], axis=-1) for i in range(3)], axis=-1).max(axis=-1)

    ref64 = solver_spectra(test, "fp64")
    t0 = time.perf_counter()
    solver_spectra(test, "mixed")
    t_solver = time.perf_counter() - t0
    t0 = time.perf_counter()
    Dl, errs, fb = sur.spectra(test, jl, lall, kin, tol=args.surrogate_tol)
    t_sur = time.perf_counter() - t0
    t0 = time.perf_counter()
    Dl_raw, _, _ = sur.spectra(test, jl, lall, kin, fallback=False)
    t_raw = time.perf_counter() - t0
    rel, rel_raw = rel_max(Dl, ref64), rel_max(Dl_raw, ref64)
    n = len(test)
    line = {"metric": "cosmologies/s (surrogate + fallback vs solver)", "value": round(n / t_sur, 3), "unit": "cosmologies/s",
            "workload": f"{n} held-out cosmologies from the box, D_l TT/TE/EE to l={LMAX}, 400 k x 500 tau, rtol {PT_RTOL:g} atol {PT_ATOL:g}",
            "solver_cosmologies_per_s": round(n / t_solver, 3), "speedup": round(t_solver / t_sur, 3),
            "fallback_rate": float(fb.mean()), "tol": args.surrogate_tol,
            "cl_max_rel_vs_fp64": {"with_fallback": {"median": float(np.median(rel)), "max": float(rel.max())},
                                   "surrogate_only": {"median": float(np.median(rel_raw)), "max": float(rel_raw.max()),
                                                      "p90": float(np.quantile(rel_raw, 0.9))}},
            "surrogate_only": {"cosmologies_per_s": round(n / t_raw, 3), "speedup_vs_solver": round(t_solver / t_raw, 2)},
            "estimate_vs_true": {"median_ratio": float(np.median(errs / rel_raw)),
                                 "pairs": [[round(float(e), 6), round(float(t), 6)] for e, t in zip(errs[:16], rel_raw[:16])]},
            "training": {"cosmologies": len(train), "rows": int(nrows), "points_per_cosmology": keep, "file": "SBZTRN01",
                         "data_s": round(t_data, 2), "steps_per_member": steps, "members": len(sur.nets), "train_s": round(t_train, 2),
                         "tflops": round(len(sur.nets) * steps * flops_step / t_train / 1e12, 1), "batch": 65536,
                         "loss_first_last": [losses[0][0], losses[0][-1]], "mse_train_standardised": mse_train,
                         "pk_surrogate": {"cosmologies": args.pk_train_cosmologies, "k": len(kpk), "s": round(t_pk, 2)}},
            "model": f"MLP {SG.SourceSurrogate.NIN} -> 4x512 SiLU -> 7 (perturbation factors) x 2 members, BF16 tcgen05 GEMMs, FP32 accumulate, Adam"}
    peaks = measured_peaks()
    nbytes = mlp_step_bytes()
    sps = t_train / (len(sur.nets) * steps)
    line["training"]["roofline"] = {
        "bound": "hbm", "unit": "GB/s", "achieved": round(nbytes / sps / 1e9, 1), "peak": peaks.get("hbm_gbs"),
        "frac": round(nbytes / sps / 1e9 / peaks["hbm_gbs"], 4) if peaks.get("hbm_gbs") else None, "traffic": None,
        "bytes_per_step": nbytes, "ms_per_step": round(sps * 1e3, 4),
        "tensor_tflops": round(flops_step / sps / 1e12, 1), "tensor_peak_sustained": peaks.get("bf16_tflops_sustained"),
        "tensor_frac": round(flops_step / sps / 1e12 / peaks["bf16_tflops_sustained"], 4) if peaks.get("bf16_tflops_sustained") else None}
    # ---- mixed workload: D_l to l = 3000 and P(k) from the surrogates, flagged cosmologies to the solver
    if args.mixed_cosmologies > 0:
        lmix = np.arange(2, 3001)
        lsm = np.unique(np.round(np.exp(np.linspace(np.log(2), np.log(3000), 200))).astype(np.int32))
        jlm = S.SphericalBesselCache(lsm)
        mix = SG.sample_box(args.mixed_cosmologies, seed=2)
        t0 = time.perf_counter()
        Dm, em, fm, tm = sur.spectra(mix, jlm, lmix, kin, tol=args.surrogate_tol, return_timings=True)
        Pm, epm, fpm = msur.spectra(mix, tol=args.surrogate_tol)
        t_mix = time.perf_counter() - t0
        nchk = min(args.mixed_check, len(mix))
        prob = S.CosmologyProblem(M, [SG.box_params(t) for t in mix[:nchk]], precision="fp64", pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
        bg = prob.solvebg()
        taus = np.stack([SG.cmb_taus(bg.t(c), bg.tau0[c], sur.ntau) for c in range(nchk)])
        src, _, _ = S.solvept(prob, np.tile(ks, nchk), prob.opts.tau_ini, saveat=taus, output="sources",
                              cosmo=np.repeat(np.arange(nchk), len(ks)))
        src = src.reshape(nchk, len(ks), sur.ntau, 3)
        Dref = np.stack([S.spectrum_cmb(["TT", "TE", "EE"], prob, jlm, lmix, kinterp=kin, taus=taus[c], cosmo=c, normalization="Dl",
                                        sources=src[c]) for c in range(nchk)])
        mref = SG.MatterSurrogate(M, kpk, members=1, pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
        Pref = np.stack([S.spectrum_primordial(kpk, prob, c) for c in range(nchk)]) * mref.solve(mix[:nchk], prob=prob) ** 2
        rc = rel_max(Dm[:nchk], Dref)
        rp = np.max(np.abs(Pm[:nchk] / Pref - 1), axis=1)
        line["mixed_workload"] = {
            "cosmologies": len(mix), "cosmologies_per_s": round(len(mix) / t_mix, 3), "seconds": round(t_mix, 2),
            "fallback_rate_cl": float(fm.mean()), "fallback_rate_pk": float(fpm.mean()), "phases_s": {k: round(v, 2) for k, v in tm.items()},
            "checked_vs_fp64": nchk, "cl_max_rel_l2_3000": {"median": float(np.median(rc)), "max": float(rc.max())},
            "pk_max_rel_1e-4_10hMpc": {"median": float(np.median(rp)), "max": float(rp.max())},
            "plain_solver_cosmologies_per_s": round(n / t_solver, 3)}
    print(json.dumps(line), flush=True)


def profile_case(args):
    """Small cases for ncu section captures, at the workload's tolerances and refinement threshold.  pt: 64 of the 1000 modes
    (even in log k, the slowest included), sources on 200 times.  los: one spectrum_cmb of the full workload (the line-of-sight
    kernel runs once on the full fine k grid; ~1.5 GB on the device).  mlp: the surrogate's training
    step (8 -> 4x512 -> 7, batch 65536; the same GEMM shapes as the 10-input surrogate, inputs padded to 64) on 2 M synthetic samples, one eager step, the graph capture
    and 4 graph replays, plus a timed run of 200 steps printed first."""
    import symboltz as S
    if args.profile_case == "mlp":
        from symboltz.surrogate import MLP
        rng = np.random.default_rng(0)
        net = MLP(8, 512, 4, 7, 65536, 0)
        net.set_data(rng.uniform(-1, 1, (2_000_000, 8)).astype(np.float32), rng.normal(size=(2_000_000, 7)).astype(np.float32))
        net.train(5, 1e-3)
        if args.steps > 5:
            t0 = time.perf_counter()
            net.train(args.steps, 1e-3)
            dt = time.perf_counter() - t0
            print(json.dumps({"profile_case": "mlp training step", "steps": args.steps, "ms_per_step": round(dt / args.steps * 1e3, 4),
                              "tflops": round(3 * 2 * 65536 * (64 * 512 + 3 * 512 * 512 + 512 * 64) * args.steps / dt / 1e12, 1)}))
        return
    M = S.ΛCDM(lmax_gamma=MODEL["lmax_gamma"], lmax_nu=MODEL["lmax_nu"], lmax_h=MODEL["lmax_h"], nx=MODEL["nx"])
    prob = S.CosmologyProblem(M, PARAMS, precision=args.precision, refine_skip=REFINE_SKIP_CL, pt_rtol=PT_RTOL, pt_atol=PT_ATOL)
    ks, taus, ls = workload_grids(S, prob)
    if args.profile_case == "pt":
        sel = ks[np.linspace(0, len(ks) - 1, 64).round().astype(int)]
        out, st, stp = S.solvept(prob, sel, prob.opts.tau_ini, saveat=taus[::10], output="sources")
        print(json.dumps({"profile_case": "pt: 64 modes, 200 saved times", "failed": int(np.count_nonzero(st)), "steps": int(stp.sum())}))
    else:
        jl = S.SphericalBesselCache(ls)
        Dl, st = S.spectrum_cmb(["TT", "TE", "EE"], prob, jl, np.arange(2, LMAX + 1), kinterp=S.CubicSplineInterpolator(ks, f=np.log),
                                taus=taus, return_status=True)
        print(json.dumps({"profile_case": "los: one spectrum_cmb", "failed": int(np.count_nonzero(st)), "timings_ms": S.timings(prob)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--train-cosmologies", type=int, default=1024)
    ap.add_argument("--points-per-cosmology", type=int, default=40000)
    ap.add_argument("--pk-train-cosmologies", type=int, default=512)
    ap.add_argument("--train-seconds", type=float, default=300.0)
    ap.add_argument("--test-cosmologies", type=int, default=32)
    ap.add_argument("--mixed-cosmologies", type=int, default=4096)
    ap.add_argument("--mixed-check", type=int, default=16)
    ap.add_argument("--surrogate-tol", type=float, default=1e-3)
    ap.add_argument("--workdir", default=tempfile.gettempdir(), help="where the training-set file is written")
    ap.add_argument("--clocks-log", default=os.path.join(tempfile.gettempdir(), "sbz_bench_clocks.csv"),
                    help="CSV of the nvidia-smi clock samples taken during the timed region")
    ap.add_argument("--workload", choices=("spectrum", "batched", "surrogate"), default="spectrum",
                    help="spectrum: the headline single-cosmology C_l workload; batched: 256 cosmologies, ragged k grids")
    ap.add_argument("--profile-case", choices=("pt", "los", "mlp"), default=None,
                    help="small cases for ncu section captures (see profile_case)")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
    elif args.workload == "batched" and args.impl == "ours":
        run_batched(args)
    elif args.workload == "surrogate" and args.impl == "ours":
        run_surrogate(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
