"""The benchmarked workloads against the oracle, through the C-ABI.

* The C_l workload of bench.py (ΛCDM with one massive ν of 0.06 eV in 5 momentum bins with
  l_max 10, N_eff 2.0328 massless, photon l_max 30; 1000 k log-spaced over 1e-5..5 h/Mpc; sources
  on the bench's 2000-point τ grid; natural-spline k-interpolation in log k; C_l TT/TE/EE to
  l = 2500) at the bench's integrator tolerances, in both precisions: every l from 2 to 2500 within
  1e-4 of the oracle (TE relative to sqrt(TT EE)), and P(k) at z = 0 on the same k.
* The batched P(k) workload: four cosmologies at the corners of the Σm_ν × h box solved in one
  launch, each against the oracle.

The oracle runs its sparse-LU path here (the same integrator and equations as its dense checker,
tested equal to it in tests/test_oracle_golden.py) so the 1000 modes take seconds on the host.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def S():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import symboltz
    return symboltz


@pytest.fixture(scope="module")
def B():
    import bench
    return bench


def _oracle_model(B):
    return dict(lmax_g=B.MODEL["lmax_gamma"], lmax_nu=B.MODEL["lmax_nu"], lmax_h=B.MODEL["lmax_h"], nx=B.MODEL["nx"], Hswitch=1,
                Heswitch=6, reionization=1)


def _rel(D, R):
    den = [np.abs(R[:, 0]), np.sqrt(np.abs(R[:, 0] * R[:, 2])), np.abs(R[:, 2])]
    return np.stack([np.abs(D[:, i] - R[:, i]) / den[i] for i in range(3)], axis=1)


@pytest.fixture(scope="module")
def oracle_spectrum(S, B):
    M = S.ΛCDM(lmax_gamma=B.MODEL["lmax_gamma"], lmax_nu=B.MODEL["lmax_nu"], lmax_h=B.MODEL["lmax_h"], nx=B.MODEL["nx"])
    prob = S.CosmologyProblem(M, B.PARAMS, pt_rtol=B.PT_RTOL, pt_atol=B.PT_ATOL)
    ks, taus, ls = B.workload_grids(S, prob)
    bg = O.Background(B.PARAMS, _oracle_model(B), pt_rtol=B.PT_RTOL, pt_atol=B.PT_ATOL, linsolve="sparse")
    lall = np.arange(2, B.LMAX + 1)
    Dl, parts = O.spectrum_cmb_kspline(bg, ks, taus, O.BesselCache(ls), lall, return_parts=True)
    assert np.count_nonzero(parts["status"]) == 0
    return dict(M=M, ks=ks, taus=taus, ls=ls, lall=lall, Dl=Dl, bg=bg)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_bench_spectrum_matches_oracle(S, B, oracle_spectrum, precision):
    """Every l of TT, TE, EE within 1e-4 of the oracle at the bench's settings (the timed
    configuration itself: mixed precision with the bench's lazy-refinement threshold)."""
    o = oracle_spectrum
    skip = B.REFINE_SKIP_CL if precision == "mixed" else None
    prob = S.CosmologyProblem(o["M"], B.PARAMS, precision=precision, refine_skip=skip, pt_rtol=B.PT_RTOL, pt_atol=B.PT_ATOL)
    jl = S.SphericalBesselCache(o["ls"])
    kin = S.CubicSplineInterpolator(o["ks"], f=np.log)
    Dl, st = S.spectrum_cmb(["TT", "TE", "EE"], prob, jl, o["lall"], kinterp=kin, taus=o["taus"], return_status=True,
                            normalization="Dl")
    assert np.all(st == 0)
    r = _rel(Dl, o["Dl"])
    worst = {m: (float(r[:, i].max()), int(o["lall"][np.argmax(r[:, i])])) for i, m in enumerate(("TT", "TE", "EE"))}
    assert r.max() <= 1e-4, worst


def test_bench_pk_matches_oracle(S, B, oracle_spectrum):
    """P(k) at z = 0 on the workload's 1000 k (spectrum_matter's initial times, fourier.jl:76-81):
    within 1e-4 of the oracle for k >= 1e-4 h/Mpc.  Below, Δ_m of a mode far outside the horizon
    carries 3ℋθ/k² with θ ∝ k² small against atol, so two integrations at atol 3e-8 agree only to
    a few 1e-4 there (measured 1.2e-4 at 1.1e-5 h/Mpc); that range is held to 3e-4."""
    o = oracle_spectrum
    prob = S.CosmologyProblem(o["M"], B.PARAMS, pt_rtol=B.PT_RTOL, pt_atol=B.PT_ATOL)
    P, st = S.spectrum_matter(prob, o["ks"], return_status=True)
    Po, sto, _ = O.spectrum_matter(o["bg"], o["ks"])
    assert np.all(st == 0) and np.all(sto == 0)
    rel = np.abs(P / Po - 1)
    hi = o["ks"] >= S.k_from_hMpc(1e-4)
    assert rel[hi].max() <= 1e-4, (float(rel[hi].max()), float(o["ks"][hi][np.argmax(rel[hi])]))
    assert rel.max() <= 3e-4, (float(rel.max()), float(o["ks"][np.argmax(rel)]))


def test_batched_box_corners_match_oracle(S, B):
    """Four cosmologies at the corners of Σm_ν ∈ [0.06, 0.3] eV × h ∈ [0.6, 0.8] (other parameters
    at the box centre), ragged k grids, all modes in one perturbation launch (the batched workload's
    path), P(k) of each against the oracle at matched tolerances."""
    M = S.ΛCDM(lmax_gamma=B.MODEL["lmax_gamma"], lmax_nu=B.MODEL["lmax_nu"], lmax_h=B.MODEL["lmax_h"], nx=B.MODEL["nx"])
    pars = []
    for mnu in (0.06, 0.3):
        for h in (0.6, 0.8):
            pars.append(dict(h=h, Omega_c=0.12 / h**2, Omega_b=0.022 / h**2, T0=2.7255, Neff=2.0328, YHe=0.245, ln_As1e10=3.05,
                             ns=0.96, m_nu_eV=mnu, N_nu=1.0))
    nks = [60, 45, 52, 38]
    ks = [S.k_from_hMpc(S.loggrid(1e-5, 5.0, length=n)) for n in nks]
    cos = np.concatenate([np.full(n, i) for i, n in enumerate(nks)])
    tol = 1e-7
    prob = S.CosmologyProblem(M, pars, pt_rtol=tol, pt_atol=tol)
    P, st = S.spectrum_matter(prob, np.concatenate(ks), cosmo=cos, return_status=True)
    assert np.all(st == 0)
    off = 0
    for c, p in enumerate(pars):
        bg = O.Background(p, _oracle_model(B), pt_rtol=tol, pt_atol=tol, linsolve="sparse")
        Po, sto, _ = O.spectrum_matter(bg, ks[c])
        assert np.all(sto == 0)
        rel = np.abs(P[off:off + nks[c]] / Po - 1)
        assert rel.max() <= 1e-4, (c, float(rel.max()), float(ks[c][np.argmax(rel)]))
        off += nks[c]
