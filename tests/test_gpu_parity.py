"""GPU parity: the CUDA path (through the C-ABI) against the CPU oracle and the reference's fixtures.

Tolerances: the GPU and the oracle integrate the same equations with the same Rodas4 tableau and
tolerances; they differ in the linear algebra (structured elimination vs dense LU), in FP32
factorisation with FP64 refinement (mixed precision) and in how background coefficients are
interpolated, so step sequences differ at the tolerance level.  Parity bar: 1e-4 relative on P(k)
and on C_l (pt rtol 1e-5), as the reference's matched-tolerance target; bit-level agreement is
expected for the purely algebraic kernels (Bessel cache, line-of-sight sums, C_l spline integral).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402

MODEL5 = dict(lmax_g=5, lmax_nu=5, lmax_h=5, nx=4, Hswitch=1, Heswitch=6, reionization=1)


@pytest.fixture(scope="module")
def S():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import symboltz
    return symboltz


@pytest.fixture(scope="module")
def bg5():
    return O.Background(O.PLANCK18, MODEL5)


@pytest.fixture(scope="module", params=["mixed", "fp64"])
def prob5(S, request):
    M = S.ΛCDM(lmax=5)
    p = S.CosmologyProblem(M, S.parameters_Planck18(M), precision=request.param)
    p.solvebg()
    return p


def test_background_matches_oracle(S, prob5, bg5):
    bg = prob5.solvebg()
    assert bg.status[0] == 0
    assert abs(bg.tau0[0] / bg5.tau0 - 1) < 1e-8
    assert abs(bg.kappa0[0] / bg5.kappa0 - 1) < 1e-8
    assert abs(bg.taurec[0] / bg5.taurec - 1) < 1e-5


def test_pk_matches_oracle(S, prob5, golden):
    """P(k) against the oracle at matched integrator tolerances, and against the reference's CLASS
    fixture at the reference's own settings.

    Parity is measured at rtol = atol = 1e-7, where the integration error of P(k) (the oracle's own
    distance to a converged solution, at most 1.0e-4 over these k) is below the bar.  At the
    reference's default 1e-5 that error is up to 2e-3 (at the lowest k) and two integrations whose
    coefficient evaluations differ in the last bits (the device table against the oracle's spline)
    can take a different accept/reject decision and end up that far apart."""
    d = np.loadtxt(os.path.join(golden, "class_Pk.txt"))
    ks = d[:, 0]
    M = S.ΛCDM(lmax=5)
    prec = "fp64" if prob5.opts.precision == 0 else "mixed"
    tight = S.CosmologyProblem(M, S.parameters_Planck18(M), precision=prec, pt_rtol=1e-7, pt_atol=1e-7)
    P, st = S.spectrum_matter(tight, ks, return_status=True)
    bgo = O.Background(O.PLANCK18, MODEL5, pt_rtol=1e-7, pt_atol=1e-7)
    Po, sto, _ = O.spectrum_matter(bgo, ks)
    assert np.all(st == 0) and np.all(sto == 0)
    rel = np.abs(P / Po - 1)
    assert np.max(rel[ks > 0.15]) < 1e-4, np.max(rel)
    assert np.linalg.norm(P - Po) <= 1e-5 * np.linalg.norm(Po)
    # the reference's settings (rtol = atol = 1e-5) against its CLASS fixture (test/runtests.jl:871-876)
    P5, st5 = S.spectrum_matter(prob5, ks, return_status=True)
    assert np.all(st5 == 0)
    assert np.linalg.norm(P5 - d[:, 1]) <= 1e-3 * np.linalg.norm(d[:, 1])
    assert np.linalg.norm(P5 - P) <= 1e-4 * np.linalg.norm(P)


@pytest.mark.parametrize("tol,bar", [(1e-5, 1e-3), (1e-7, 2e-5)])
def test_sources_match_oracle(S, prob5, tol, bar):
    """Line-of-sight sources against the oracle at the same integrator tolerance, in both precisions.

    The error norm and the step-size controller are FP64 in both precisions, like the oracle's, and
    the stage solutions are FP64 after refinement, so the step sequences stay together and the
    sources agree to well inside the tolerance (bar, relative to each mode's largest source value).
    Also, measured against a converged oracle solution (tolerance / 100), the GPU solution is no
    further off than three times the oracle's own distance plus a tenth of the bar."""
    M = S.ΛCDM(lmax=5)
    fp64 = prob5.opts.precision == 0
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M), pt_rtol=tol, pt_atol=tol,
                              precision="fp64" if fp64 else "mixed")
    bgo = O.Background(O.PLANCK18, MODEL5, pt_rtol=tol, pt_atol=tol)
    ks = np.array([2.0, 50.0, 300.0, 2000.0])
    # S_E and S_ψ carry 1/χ² and 1/χ (χ = τ0 - τ): near τ0 they magnify the 1e-8 relative difference
    # of the two background integrations' τ0 by τ0/χ, so the grid stops at χ = 0.01 τ0
    taus = np.linspace(bgo.tau0 * 0.01, bgo.tau0 * 0.99, 64)
    out, st, _ = S.solvept(prob, ks, 1e-6, saveat=taus, output="sources")
    ref, sto, _ = bgo.solve_pt(ks, 1e-6, taus, mode=0)
    conv, stc, _ = O.Background(O.PLANCK18, MODEL5, pt_rtol=tol / 100, pt_atol=tol / 100).solve_pt(ks, 1e-6, taus, mode=0)
    assert np.all(st == 0) and np.all(sto == 0) and np.all(stc == 0)
    for s in range(3):
        scale = np.max(np.abs(conv[:, :, s]), axis=1, keepdims=True) + 1e-300
        assert np.max(np.abs(out[:, :, s] - ref[:, :, s]) / scale) < bar, s
        ours = np.max(np.abs(out[:, :, s] - conv[:, :, s]) / scale)
        theirs = np.max(np.abs(ref[:, :, s] - conv[:, :, s]) / scale)
        assert ours <= 3 * theirs + 0.1 * bar, (s, ours, theirs)


def test_state_matches_oracle(S, prob5):
    tol = 1e-7
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M), pt_rtol=tol, pt_atol=tol,
                              precision="fp64" if prob5.opts.precision == 0 else "mixed")
    bgo = O.Background(O.PLANCK18, MODEL5, pt_rtol=tol, pt_atol=tol)
    ks = np.array([0.5, 30.0, 800.0])
    taus = np.array([1e-6, 1e-3, 0.02, 0.06, 0.5, bgo.tau0 * (1 - 1e-6)])
    out, st, _ = S.solvept(prob, ks, 1e-6, saveat=taus, output="state")
    ref, sto, _ = bgo.solve_pt(ks, 1e-6, taus, mode=2)
    assert np.all(st == 0) and np.all(sto == 0)
    g = out[:, :, S.state_index(M)]
    np.testing.assert_allclose(g[:, 0], ref[:, 0], rtol=1e-12, atol=1e-300)  # initial conditions
    # per component, in units of the integrator's error weights (atol + rtol |y|)
    w = tol + tol * np.max(np.abs(ref), axis=1, keepdims=True)
    assert np.max(np.abs(g - ref) / w) < 50


def test_failed_modes_report_status(S, prob5):
    P, st = S.spectrum_matter(prob5, np.array([0.0, np.nan, 1.0]), return_status=True)
    assert st[0] != 0 and st[1] != 0 and st[2] == 0


def test_maxiters_status(S):
    M = S.ΛCDM(lmax=5)
    p = S.CosmologyProblem(M, S.parameters_Planck18(M), maxiters=20)
    P, st = S.spectrum_matter(p, np.array([1.0, 100.0]), return_status=True)
    assert np.all(st == 1)


def test_bessel_cache_matches_oracle(S):
    from scipy.special import spherical_jn
    ls = np.array([2, 3, 10, 57, 200, 999, 1500])
    jl = S.SphericalBesselCache(ls)
    jo = O.BesselCache(ls)
    xs = np.concatenate([[0.0], np.geomspace(1e-3, jl.xmax * 0.999, 4000)])
    for il in range(len(ls)):
        a, b = jl(il, xs), jo(il, xs)
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(a, spherical_jn(ls[il], xs), atol=1e-5)


def test_los_and_cl_match_oracle(S):
    rng = np.random.default_rng(0)
    ls = np.array([2, 5, 10, 30, 100, 400])
    jl, jo = S.SphericalBesselCache(ls), O.BesselCache(ls)
    taus = np.sort(rng.uniform(0.05, 3.0, 200))
    ks = np.linspace(1.0, 150.0, 97)
    Sg = rng.standard_normal((len(taus), len(ks), 3))
    for l_limber in (2**31 - 1, 10):
        a = S.los_integrate(Sg, ls, taus, ks, jl, l_limber=l_limber)
        b = O.los_integrate(Sg, taus, ks, jo, l_limber)
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12 * np.max(np.abs(b)))
    P0 = rng.uniform(0.5, 1.5, len(ks))
    ThA, ThB = rng.standard_normal((len(ks), len(ls))), rng.standard_normal((len(ks), len(ls)))
    np.testing.assert_allclose(S.spectrum_cmb(ThA, ThB, P0, ls, ks), O.cl_integrate(ks, P0, ThA, ThB), rtol=1e-11)


def test_cmb_matches_oracle_and_class(S, golden, bg5):
    """D_l TT/EE/ψψ against the oracle at matched tolerances (rtol 1e-6, atol 3e-8, where the
    integration error of the low-l D_l is far below the bar; see test_pk_matches_oracle), and the
    reference's default settings against its CLASS fixture at the reference's tolerance."""
    d = np.loadtxt(os.path.join(golden, "class_Cl.txt"))
    lc = d[:, 0]
    ls = np.unique(np.round(np.exp(np.linspace(np.log(lc[0]), np.log(lc[-1]), 200))).astype(int))
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M))
    jl = S.SphericalBesselCache(ls)
    Dl = S.spectrum_cmb(["TT", "EE", "ψψ"], prob, jl, lc, normalization="Dl")
    # the reference's default τ-grid starts at the first background knot >= τcut; the two background
    # integrations place knots slightly differently, so parity is measured on one shared grid
    t = bg5.t[bg5.t >= 1e-2]
    taus = t[0] + (bg5.tau0 * (1 - 1e-12) - t[0]) * S.cosgrid(0.0, 1.0, length=300)
    tight = S.CosmologyProblem(M, S.parameters_Planck18(M), pt_rtol=1e-6, pt_atol=3e-8)
    Dg = S.spectrum_cmb(["TT", "EE", "ψψ"], tight, jl, lc, normalization="Dl", taus=taus)
    bgt = O.Background(O.PLANCK18, MODEL5, pt_rtol=1e-6, pt_atol=3e-8)
    Do = O.spectrum_cmb(bgt, ["TT", "EE", "ψψ"], O.BesselCache(ls), lc, taus=taus)
    for j in range(3):
        assert np.linalg.norm(Dg[:, j] - Do[:, j]) <= 1e-4 * np.linalg.norm(Do[:, j]), j
        assert np.linalg.norm(Dl[:, j] - d[:, j + 1]) <= 2e-3 * np.linalg.norm(d[:, j + 1]), j


def test_rhs_matches_oracle(S, prob5, bg5):
    """The GPU operator (f = J y, ∂f/∂τ) against the oracle's dense right-hand side."""
    rng = np.random.default_rng(1)
    M = S.ΛCDM(lmax=5)
    idx = S.state_index(M)
    ks = np.array([0.3, 3.0, 30.0, 300.0, 3000.0])
    taus = np.array([1e-6 * 1.7, 3e-5, 2e-3, 0.06, 1.5])
    for tau in taus:
        Yo = rng.standard_normal((len(ks), bg5.nstate))
        Yg = np.zeros_like(Yo)
        Yg[:, idx] = Yo
        f, ft = S.pt_rhs(prob5, ks, np.full(len(ks), tau), Yg)
        for i, k in enumerate(ks):
            fo, Jo, fto = bg5.rhs(k, tau, Yo[i], jac=True)
            scale = np.abs(Jo) @ np.abs(Yo[i]) + 1e-300
            np.testing.assert_array_less(np.abs(f[i, idx] - fo) / scale, 1e-6, err_msg=f"f tau={tau} k={k}")
            # ∂f/∂τ from the derivatives of the tabulated coefficients (the table's Hermite slopes)
            # against the oracle's exact derivatives through the background spline: measured at most
            # 3.1e-7 of the largest entry (at recombination, where κ̇ changes fastest)
            tscale = np.abs(fto).max() + 1e-300
            assert np.max(np.abs(ft[i, idx] - fto)) / tscale < 1e-6, (tau, k)


def test_batched_cosmologies_match_single_solves(S):
    """Several cosmologies with ragged k grids in one launch give, mode for mode, the same Δm as
    each cosmology solved alone (modes are independent; same launch shape → same arithmetic)."""
    M = S.ΛCDM(lmax=5)
    base = S.parameters_Planck18(M)
    pars = [dict(base, h=0.62 + 0.04 * i, Omega_c=base["Omega_c"] * (0.9 + 0.1 * i)) for i in range(3)]
    rng = np.random.default_rng(0)
    nks = rng.integers(8, 24, size=3)
    ks = [S.k_from_hMpc(S.loggrid(1e-4, 2.0, length=int(n))) for n in nks]
    cos = np.concatenate([np.full(int(n), i) for i, n in enumerate(nks)])
    ti = lambda k: np.minimum(1e-2 / k, 1e-4)  # noqa: E731
    batch = S.CosmologyProblem(M, pars, warps_per_mode=4)
    dm, st, _ = S.solvept(batch, np.concatenate(ks), ti, output="delta_m", cosmo=cos)
    assert np.all(st == 0)
    for i, p in enumerate(pars):
        one = S.CosmologyProblem(M, p, warps_per_mode=4)
        d1, s1, _ = S.solvept(one, ks[i], ti, output="delta_m")
        assert np.all(s1 == 0)
        np.testing.assert_array_equal(dm[cos == i], d1)


def test_autotune_picks_a_candidate_and_keeps_results(S):
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M))
    ks = S.k_from_hMpc(S.loggrid(1e-4, 1.0, length=40))
    ti = lambda k: np.minimum(1e-2 / k, 1e-4)  # noqa: E731
    ref, _, _ = S.solvept(prob, ks, ti, output="delta_m")
    tune = S.autotune(prob, ks, ti, output="delta_m")
    assert (tune["warps_per_mode"], tune["blocks_per_sm"]) in tune["candidates_ms"]
    assert all(v > 0 for v in tune["candidates_ms"].values())
    got, st, _ = S.solvept(prob, ks, ti, output="delta_m")
    assert np.all(st == 0)
    np.testing.assert_allclose(got, ref, rtol=1e-4)  # another launch shape: same solution to tolerance


def test_source_grid_adaptive_on_the_device(S):
    """source_grid_adaptive (src/observables/fourier.jl:312-410): the refined grid contains the initial
    one, its values are the solver's at those k, and every split was warranted (each inserted
    midpoint failed or passed the test against its parents' interpolation as the rule says)."""
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M))
    ks0 = S.k_from_hMpc(np.geomspace(1e-3, 0.3, 4))
    bg = prob.solvebg()
    taus = np.linspace(0.05, bg.tau0[0], 6)
    s0, _, _ = S.solvept(prob, ks0, 1e-6, saveat=taus, output="sources")
    atol = 1e-2 * np.max(np.abs(s0))  # sources cross zero: a purely relative test never passes there
    ks, vals = S.source_grid_adaptive(prob, taus, ks0, atol=atol, rtol=1e-2, ktransform=(np.log, np.exp), ptivini=1e-6)
    assert len(ks) > len(ks0) and np.all(np.diff(ks) > 0)
    assert np.all(np.isin(np.round(ks0, 9), np.round(ks, 9)))
    direct, st, _ = S.solvept(prob, ks, 1e-6, saveat=taus, output="sources")
    assert np.all(st == 0)
    np.testing.assert_allclose(vals, direct, rtol=1e-12, atol=1e-300)
    kd, dm = S.source_grid_adaptive(prob, None, ks0, output="delta_m", rtol=1e-3, ktransform=(np.log, np.exp), ptivini=1e-6)
    assert dm.shape == kd.shape and np.all(np.isfinite(dm))


def test_adaptive_spectrum_matter(S, bg5):
    """spectrum_matter(prob, (kmin, kmax)) (src/observables/fourier.jl:103-125): 9-point log grid
    refined on Δ_m (atol 4, rtol 4e-3).  The refined grid is the oracle's (same rule driven by the
    oracle's Δ_m), the values are the solver's at those k, and P(k) matches the oracle there."""
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M))
    kmin, kmax = S.k_from_hMpc(1e-4), S.k_from_hMpc(1.0)
    ks, P = S.spectrum_matter(prob, (kmin, kmax))
    assert ks[0] == kmin and ks[-1] == kmax and len(ks) > 9 and np.all(np.diff(ks) > 0)
    dm, st, _ = S.solvept(prob, ks, -np.inf, output="delta_m")
    assert np.all(st == 0)
    np.testing.assert_allclose(P, S.spectrum_primordial(ks, prob) * dm**2, rtol=1e-12)

    def oracle_dm(kk):
        out, sto, _ = bg5.solve_pt(kk, bg5.t[0], None, mode=1)
        assert np.all(sto == 0)
        return out
    ko, dmo = S.refine_grid(oracle_dm, S.loggrid(kmin, kmax, length=9), atol=4.0, rtol=4e-3, ktransform=(np.log, np.exp))
    assert len(ko) == len(ks)
    np.testing.assert_allclose(ks, ko, rtol=1e-14)
    assert np.linalg.norm(dm - dmo) <= 1e-4 * np.linalg.norm(dmo)  # the P(k) parity bar, normwise


def test_set_params_reuses_the_problem(S):
    """sbz_problem_set_params: the same handle, re-uploaded with 1 then 3 parameter sets, gives
    bit-identical modes to fresh problems (stale device tables would show here)."""
    M = S.ΛCDM(lmax=5)
    base = S.parameters_Planck18(M)
    ks = S.k_from_hMpc(S.loggrid(1e-4, 1.0, length=24))
    ti = lambda k: np.minimum(1e-2 / k, 1e-4)  # noqa: E731
    p = S.CosmologyProblem(M, base, warps_per_mode=2)
    S.solvept(p, ks, ti, output="delta_m")
    sets = [dict(base, h=0.7), dict(base, h=0.64, Omega_b=0.05), dict(base, ns=0.95), dict(base, h=0.71, Omega_c=0.3)]
    p.set_params(sets[0])
    got, st, _ = S.solvept(p, ks, ti, output="delta_m")
    ref, _, _ = S.solvept(S.CosmologyProblem(M, sets[0], warps_per_mode=2), ks, ti, output="delta_m")
    assert np.all(st == 0)
    np.testing.assert_array_equal(got, ref)
    p.set_params(sets[1:])
    cos = np.repeat(np.arange(3), len(ks))
    got, st, _ = S.solvept(p, np.tile(ks, 3), ti, output="delta_m", cosmo=cos)
    assert np.all(st == 0)
    for i in range(3):
        one, _, _ = S.solvept(S.CosmologyProblem(M, sets[1 + i], warps_per_mode=2), ks, ti, output="delta_m")
        np.testing.assert_array_equal(got[cos == i], one)


# plain ΛCDM: h = 0.67, ω_c = 0.12, ω_b = 0.022, T_CMB = 2.7255 K, N_eff = 3.046 massless ν,
# Y_He = 0.245, ln(1e10 A_s) = 3.04, n_s = 0.965; photon and massless-ν hierarchies to l = 10
PLAIN_PARAMS = dict(h=0.67, Omega_c=0.12 / 0.67**2, Omega_b=0.022 / 0.67**2, T0=2.7255, Neff=3.046, YHe=0.245, ln_As1e10=3.04,
                    ns=0.965, m_nu_eV=0.0, N_nu=0.0)
MODEL10_MASSLESS = dict(lmax_g=10, lmax_nu=10, lmax_h=10, nx=0, Hswitch=1, Heswitch=6, reionization=1)


def test_plain_lcdm_fp64_rtol1e6(S):
    """Plain ΛCDM in FP64 at rtol = atol = 1e-6: 100 modes log-spaced over 1e-4..1 h/Mpc, P(k) at
    z = 0 and the line-of-sight sources on 500 times, against the oracle at the same tolerance; the
    mixed-precision solver's P(k) on the same modes at the same bar."""
    M = S.ΛCDM(lmax=10, massive_nu=False)
    prob = S.CosmologyProblem(M, PLAIN_PARAMS, pt_rtol=1e-6, pt_atol=1e-6, precision="fp64")
    bgo = O.Background(PLAIN_PARAMS, MODEL10_MASSLESS, pt_rtol=1e-6, pt_atol=1e-6)
    assert prob.nstate == bgo.nstate == 38
    khm = S.loggrid(1e-4, 1.0, length=100)
    ks = S.k_from_hMpc(khm)
    P, st = S.spectrum_matter(prob, ks, return_status=True)
    Po, sto, _ = O.spectrum_matter(bgo, ks)
    assert np.all(st == 0) and np.all(sto == 0)
    rel = np.abs(P / Po - 1)
    assert np.max(rel[khm > 0.15]) < 1e-4, np.max(rel)
    assert np.linalg.norm(P - Po) <= 1e-4 * np.linalg.norm(Po)
    mixed = S.CosmologyProblem(M, PLAIN_PARAMS, pt_rtol=1e-6, pt_atol=1e-6)
    Pm, stm = S.spectrum_matter(mixed, ks, return_status=True)
    assert np.all(stm == 0) and np.linalg.norm(Pm - Po) <= 1e-4 * np.linalg.norm(Po)
    taus = np.linspace(bgo.tau0 * 0.01, bgo.tau0 * 0.999, 500)
    out, st, _ = S.solvept(prob, ks, 1e-6, saveat=taus, output="sources")
    ref, sto, _ = bgo.solve_pt(ks, 1e-6, taus, mode=0)
    assert np.all(st == 0) and np.all(sto == 0)
    for s in range(3):
        scale = np.max(np.abs(ref[:, :, s]), axis=1, keepdims=True) + 1e-300
        assert np.max(np.abs(out[:, :, s] - ref[:, :, s]) / scale) < 1e-3, s


def test_device_table_matches_oracle(S, bg5):
    """The coefficient table built on the device (what the kernels read; bg.coefficients serves it)
    against the oracle's background, at the tolerances the host build is held to on CPU."""
    M = S.ΛCDM(lmax=5)
    p = S.CosmologyProblem(M, S.parameters_Planck18(M))
    bg = p.solvebg()
    ts = np.geomspace(1e-6 * 1.01, bg5.tau0 * (1 - 1e-9), 400)
    c, b = bg.coefficients(ts), bg5.eval(ts)
    for q, j, tol in ((0, 0, 1e-7), (1, 1, 1e-7), (2, 2, 2e-6)):  # a, ℋ, κ̇
        np.testing.assert_allclose(c[:, q], b[:, j], rtol=tol)
    # c_s² follows the slopes of the stiff ΔT spline: where it is ~4e-9 the background solved on an
    # aarch64 host differs from the x86 oracle fixture's by ~1.5e-5 (4.5e-6 on x86)
    np.testing.assert_allclose(c[:, 3], b[:, 6], rtol=5e-5)
    ek = np.exp(-b[:, 3])  # e^{-κ} from the oracle's κ, where the sources see it (early on κ is huge)
    seen = ek > 1e-3
    np.testing.assert_allclose(c[seen, 4], ek[seen], rtol=1e-5)


def test_spline_kinterp_pipeline_matches_oracle(S):
    """The device pipeline with natural-spline k-interpolation (the bench's interpolator: splines in
    log k through the coarse modes, sbz_spectrum_cmb_sources) against the oracle's restatement on the
    same smooth synthetic sources: both are linear in the sources, so they agree to rounding."""
    rng = np.random.default_rng(3)
    M = S.ΛCDM(lmax=5)
    prob = S.CosmologyProblem(M, S.parameters_Planck18(M), los_precision="fp64")
    bg = prob.solvebg()
    ks = S.k_from_hMpc(S.loggrid(1e-4, 0.5, length=57))
    t = bg.t(0)
    t = t[t >= 1e-2]
    taus = t[0] + (bg.tau0[0] - t[0]) * S.cosgrid(0.0, 1.0, length=180)
    lk, lt = np.log(ks)[:, None], (taus / taus[-1])[None, :]
    src = np.zeros((len(ks), len(taus), 3))
    for s in range(3):
        a = rng.uniform(0.5, 2.0, 3)
        src[:, :, s] = np.sin(a[0] * lk + 3 * a[1] * lt) * np.exp(-((lt - 0.02 * a[2]) ** 2) / 0.01) + 0.1 * np.cos(a[2] * lk)
    ls = np.unique(np.round(np.exp(np.linspace(np.log(2), np.log(400), 40))).astype(int))
    lall = np.arange(2, 401)
    Dg = S.spectrum_cmb(["TT", "TE", "EE"], prob, S.SphericalBesselCache(ls), lall, kinterp=S.CubicSplineInterpolator(ks, f=np.log),
                        taus=taus, normalization="Dl", sources=src)
    bgo = O.Background(O.PLANCK18, MODEL5)
    bgo.tau0 = float(bg.tau0[0])  # the device pipeline's fine k grid uses the device background's τ0
    Do = O.spectrum_cmb_kspline(bgo, ks, taus, O.BesselCache(ls), lall, sources=src)
    np.testing.assert_allclose(Dg, Do, rtol=1e-9, atol=1e-12 * np.max(np.abs(Do)))
    # the mixed-precision line of sight (FP32 Bessel table and chunk sums, FP64 accumulation) on the
    # same sources: these oscillatory synthetic integrands cancel to ~1e-6 of their terms
    pm = S.CosmologyProblem(M, S.parameters_Planck18(M))
    Dm = S.spectrum_cmb(["TT", "TE", "EE"], pm, S.SphericalBesselCache(ls), lall, kinterp=S.CubicSplineInterpolator(ks, f=np.log),
                        taus=taus, normalization="Dl", sources=src)
    np.testing.assert_allclose(Dm, Do, rtol=1e-5, atol=1e-9 * np.max(np.abs(Do)))
