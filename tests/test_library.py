"""CPU-side checks of the C-ABI library: it loads and exports every entry point that
include/symboltz_gb300.h declares (no compute calls: there is no GPU here), plus host logic."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "symboltz_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(sbz_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    from symboltz import _lib
    assert sorted(_lib.EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol():
    from symboltz import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    L = _lib.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_default_options():
    import ctypes as C
    from symboltz import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    o = _lib.Opts()
    _lib.lib().sbz_default_opts(C.byref(o))
    assert o.bg_rtol == 1e-7 and o.pt_rtol == 1e-5 and o.tau_ini == 1e-6 and o.maxiters == 100000 and o.refine_iters == 3 and o.refine_skip == -1.0
    assert o.precision == _lib.SBZ_MIXED


def test_momentum_quadrature_host(golden):
    """The product's quadrature is host code; it matches the published table without a GPU."""
    from symboltz import _lib
    import symboltz as S
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    tab = np.loadtxt(os.path.join(golden, "quadrature.txt"))
    for row in tab:
        N = int(row[0])
        x, W = S.momentum_quadrature(N)
        np.testing.assert_allclose(x, row[1:1 + N], atol=6e-6)
        np.testing.assert_allclose(W, row[9:9 + N], atol=6e-6)


def test_host_stages_run_and_gpu_calls_fail_loudly_without_gpu():
    """Problem set-up and the background stage are host code; perturbation solves need the GPU
    and raise (no CPU fallback)."""
    import torch
    from symboltz import _lib
    import symboltz as S
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    p = S.CosmologyProblem(S.ΛCDM(lmax=5), S.parameters_Planck18())
    assert p.solvebg().status[0] == 0
    with pytest.raises(S.SbzError):
        S.spectrum_matter(p, [1.0])


def test_parameter_updates_equal_fresh_problems():
    """parameter_updater (src/solve.jl:271-306): a new problem by default, the same handle with
    inplace=True, several parameter sets from a 2-D array; backgrounds equal fresh problems'."""
    from symboltz import _lib
    import symboltz as S
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    M = S.ΛCDM(lmax=5)
    base = S.parameters_Planck18()
    p = S.CosmologyProblem(M, base)
    tau0 = p.solvebg().tau0[0]
    upd = S.parameter_updater(p, ["h", "Omega_c"])
    q = upd([0.7, 0.25])
    assert q is not p and p.pars[0]["h"] == base["h"] and p.solvebg().tau0[0] == tau0
    fresh = S.CosmologyProblem(M, dict(base, h=0.7, Omega_c=0.25))
    assert q.solvebg().tau0[0] == fresh.solvebg().tau0[0] != tau0
    assert q.opts.pt_rtol == p.opts.pt_rtol and q.opts.precision == p.opts.precision
    same = S.parameter_updater(p, ["h", "Omega_c"], inplace=True)({"h": 0.7, "Omega_c": 0.25})
    assert same is p and p.bg is None and p.solvebg().tau0[0] == fresh.solvebg().tau0[0]
    rows = np.array([[0.65, 0.3], [0.72, 0.22], [0.68, 0.27]])
    S.parameter_updater(p, ["h", "Omega_c"], inplace=True)(rows)
    bg = p.solvebg()
    assert p.ncosmo == 3 and len(bg.tau0) == 3
    for i, (h, oc) in enumerate(rows):
        assert bg.tau0[i] == S.CosmologyProblem(M, dict(base, h=h, Omega_c=oc)).solvebg().tau0[0]
    with pytest.raises(S.SbzError):  # the C-ABI refuses an empty parameter set
        S._lib.check(S._lib.lib().sbz_problem_set_params(p._h, None, 0), "set_params")
    assert p.solvebg().tau0.shape == (3,)  # and leaves the problem as it was
    with pytest.raises(KeyError):
        S.parameter_updater(p, ["H0"])
    with pytest.raises(ValueError):
        S.parameter_updater(p, ["h"])([0.7, 0.2])


def test_background_and_table_match_oracle():
    """The product's host background (solve, spline, coefficient table) against the oracle."""
    from symboltz import _lib
    import symboltz as S
    import oracle as O
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    p = S.CosmologyProblem(S.ΛCDM(lmax=5), S.parameters_Planck18())
    bg = p.solvebg()
    o = O.Background(O.PLANCK18, dict(lmax_g=5, lmax_nu=5, lmax_h=5, nx=4, Hswitch=1, Heswitch=6, reionization=1))
    assert abs(bg.tau0[0] / o.tau0 - 1) < 1e-8
    assert abs(bg.kappa0[0] / o.kappa0 - 1) < 1e-8
    assert abs(bg.taurec[0] / o.taurec - 1) < 1e-5  # flat maximum of the visibility
    # from the second table node on: the table smooths the ~1e-14-wide ΔT transient at the initial
    # time over its first interval
    ts = np.geomspace(1e-6 * 1.01, o.tau0 * (1 - 1e-9), 400)
    a, b, c = bg.eval(ts), o.eval(ts), bg.coefficients(ts)
    # the two background integrations take slightly different steps (rounding), so spline values
    # agree to ~1e-7 (a, ℋ) and ~1e-6 where Xe changes fast (κ̇, Xe in reionization)
    for j, tol in ((0, 1e-7), (1, 1e-7), (2, 2e-6), (7, 2e-6)):  # a, ℋ, κ̇, Xe
        np.testing.assert_allclose(a[:, j], b[:, j], rtol=tol)
    np.testing.assert_allclose(a[:, 6], b[:, 6], rtol=1e-5)  # c_s² (slope-sensitive ΔT spline)
    for q, j, tol in ((0, 0, 1e-7), (1, 1, 1e-7), (2, 2, 2e-6)):  # table interpolation as the kernels read it
        np.testing.assert_allclose(c[:, q], b[:, j], rtol=tol)
    np.testing.assert_allclose(c[:, 3], b[:, 6], rtol=1e-5)


def test_grids_match_reference_definitions():
    import symboltz as S
    g = S.cosgrid(0.0, 1.0, length=300)
    assert g[0] == 0.0 and abs(g[-1] - 1.0) < 1e-15 and np.all(np.diff(g) > 0)
    lg = S.loggrid(1e-4, 1.0, length=100)
    assert lg[0] == 1e-4 and lg[-1] == 1.0
    ci = S.ChebyshevInterpolator(1e-2, 2e3, 60)
    assert ci.xs[0] == 2e3 and ci.xs[-1] == 1e-2 and len(ci.xs) == 61
    # barycentric interpolation reproduces low-order polynomials exactly
    kf = np.linspace(1e-2, 2e3, 1001)
    Mx = ci.matrix(kf)
    np.testing.assert_allclose(Mx @ (ci.xs**2), kf**2, rtol=1e-9)


def _reference_refinement(fun, ks, atol, rtol, f, finv):
    """Direct recursive restatement of the reference's rule (src/observables/fourier.jl:385-394)."""
    out = {float(k): fun(np.array([k]))[0] for k in ks}

    def split(k1, k3):
        k2 = float(finv((f(k1) + f(k3)) / 2))
        s2 = fun(np.array([k2]))[0]
        out[k2] = s2
        si = (out[k1] + out[k3]) / 2
        if any(np.linalg.norm(s2[r] - si[r]) > max(atol, rtol * max(np.linalg.norm(s2[r]), np.linalg.norm(si[r])))
               for r in range(s2.shape[0])):
            split(k2, k3)
            split(k1, k2)

    for a, b in zip(ks[:-1], ks[1:]):
        split(float(a), float(b))
    return np.array(sorted(out))


def test_adaptive_refinement_matches_the_reference_rule():
    """Level-synchronous refinement yields the grid of the reference's recursive rule, and every
    accepted leaf interval passes the midpoint test."""
    import symboltz as S
    calls = []

    def fun(kk):
        calls.append(len(kk))
        x = np.log(kk)[:, None]
        return np.concatenate([np.sin(6 * x) * np.exp(-0.1 * x * x), np.cos(3 * x)], axis=1)[:, None, :]  # [k][1 row][2]

    ks0 = np.geomspace(1e-3, 1.0, 5)
    f, finv = np.log, np.exp
    got, vals = S.refine_grid(fun, ks0, atol=1e-3, ktransform=(f, finv))
    ref = _reference_refinement(fun, ks0, 1e-3, 0.0, f, finv)
    np.testing.assert_allclose(got, ref, rtol=1e-15)
    assert np.all(np.diff(got) > 0) and set(np.round(ks0, 15)) <= set(np.round(got, 15))
    assert len(calls) > 2 and max(calls[1:]) > 1  # midpoints are evaluated a level at a time
    np.testing.assert_allclose(vals[:, 0, :], fun(got)[:, 0, :])
    with pytest.raises(ValueError):
        S.refine_grid(fun, ks0, atol=1e-12, ktransform=(f, finv), maxks=64)


def test_surrogate_routing_sends_non_finite_estimates_to_the_solver():
    """A cosmology keeps the surrogate's C_l only when its error estimate is a number within the
    tolerance: NaN and infinite estimates fall back to the solver like estimates above it."""
    from symboltz.surrogate import needs_solver
    errs = np.array([1e-4, 1e-3, 2e-3, np.nan, np.inf, 0.0])
    np.testing.assert_array_equal(needs_solver(errs, 1e-3), [False, False, True, True, True, False])


def test_training_set_file_round_trip(tmp_path):
    """Flat SBZTRN01 training-set files: shards appended one after another read back exactly, in
    any row range; mismatched shapes, ranges past the end and foreign files are refused."""
    from symboltz import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    from symboltz import surrogate as SG
    rng = np.random.default_rng(0)
    path = tmp_path / "train.sbz"
    shards = [(rng.standard_normal((n, 8)).astype(np.float32), rng.standard_normal((n, 7)).astype(np.float32)) for n in (5, 70000, 3)]
    for X, Y in shards:
        SG.write_training_set(path, X, Y)
    assert SG.training_set_info(path) == (8, 7, 70008)
    X, Y = SG.read_training_set(path)
    np.testing.assert_array_equal(X, np.concatenate([s[0] for s in shards]))
    np.testing.assert_array_equal(Y, np.concatenate([s[1] for s in shards]))
    Xp, Yp = SG.read_training_set(path, first=69990, n=18)
    np.testing.assert_array_equal(Xp, X[69990:])
    np.testing.assert_array_equal(Yp, Y[69990:])
    with pytest.raises(_lib.SbzError):
        SG.write_training_set(path, np.zeros((2, 6), np.float32), np.zeros((2, 7), np.float32))
    with pytest.raises(_lib.SbzError):
        SG.read_training_set(path, first=70000, n=9)
    bad = tmp_path / "other.bin"
    bad.write_bytes(b"SBZMLP01" + bytes(16))
    with pytest.raises(_lib.SbzError):
        SG.training_set_info(bad)


def test_bessel_cache_rejects_non_integer_multipoles():
    """The cache tabulates integer l (one recurrence in l per x); non-integer l, which the
    reference's SphericalBesselCache also accepts (test/runtests.jl:903-913), fails loudly instead of
    being truncated."""
    import symboltz as S
    for bad in (S.loggrid(2, 2500, length=100), [2, 3.5], [-1, 2], []):
        with pytest.raises(ValueError, match="non-negative integers"):
            S.SphericalBesselCache(bad)
