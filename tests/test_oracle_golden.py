"""Pins the CPU oracle to the reference's own known answers (no GPU needed).

Mirrors test/runtests.jl of the reference: momentum quadrature (:549-559), callbacks (:68-74),
initial conditions (:232-278), Bessel functions and cache (:98-145), the CLASS comparison
(:871-886; normwise isapprox with rtol 1e-3 for P(k) and 2e-3 for D_l), and P(k) self-convergence
(:624-630).
"""
import math
import os

import numpy as np
import pytest

import oracle as O

MODEL5 = dict(lmax_g=5, lmax_nu=5, lmax_h=5, nx=4, Hswitch=1, Heswitch=6, reionization=1)


@pytest.fixture(scope="module")
def bg5():
    return O.Background(O.PLANCK18, MODEL5)


def test_quadrature_matches_published_table(golden):
    tab = np.loadtxt(os.path.join(golden, "quadrature.txt"))
    for row in tab:
        N = int(row[0])
        x, W = O.momentum_quadrature(N)
        np.testing.assert_allclose(x, row[1:1 + N], atol=6e-6)
        np.testing.assert_allclose(W, row[9:9 + N], atol=6e-6)


def test_quadrature_fermi_dirac_moments():
    from scipy.special import zeta
    for N in range(1, 6):
        x, W = O.momentum_quadrature(4)  # the reference test always uses 4 points
        for n in range(2, 9):
            num = np.sum(W * x ** (n - 2))
            anal = math.factorial(n) * (1 - 2.0**-n) * zeta(n + 1)
            assert abs(num / anal - 1) <= 10.0 ** (-6 + n - N)


def test_background_callbacks(bg5):
    assert bg5.status == 0
    e = bg5.eval([bg5.tau0])[0]
    assert abs(e[0] - 1.0) < 1e-12 and e[0] >= 1.0  # a(τ0) = 1
    assert e[3] == 0.0  # κ(τ0) = 0
    v = bg5.eval(bg5.t)[:, 4]
    assert abs(bg5.taurec - bg5.t[np.argmax(v)]) < 2 * np.max(np.diff(bg5.t[np.argmax(v) - 1:np.argmax(v) + 2]))
    # flat: closure on Lambda
    assert abs(bg5.Og0 + bg5.On0 + bg5.Oh0 + bg5.OL0 + O.PLANCK18["Omega_c"] + O.PLANCK18["Omega_b"] - 1) < 1e-14


def test_recombination_fractions_bounded():
    for sw in (dict(Hswitch=0), dict(Heswitch=0), dict(reionization=0)):
        m = dict(MODEL5, **sw)
        bg = O.Background(O.PLANCK18, m)
        assert bg.status == 0
        assert np.all(bg.y[:, 3] <= 1 + 1e-5) and np.all(bg.y[:, 4] <= 1 + 1e-5)


def test_initial_conditions(bg5):
    tau = bg5.t[0]
    a = bg5.eval([tau])[0][0]
    # a ≈ sqrt(Ω_r) τ with the relativistic massive-ν density
    x, W = O.momentum_quadrature(4)
    Or = bg5.Og0 + bg5.On0 + bg5.Oh0 / bg5.Irho0 * 7 * np.pi**4 / 120
    assert abs(a - np.sqrt(Or) * tau) < 1e-10
    assert abs(bg5.eval([tau])[0][1] * tau - 1) < 1e-10  # τ ≈ 1/ℋ
    ks = np.array([1e-1, 1e0]) * 2997.92458 / O.PLANCK18["h"]
    ys = []
    for k in ks:
        y, (Phi, Psi, fnu) = bg5.initial(k, tau)
        assert abs(Phi / Psi - (1 + 0.4 * fnu)) < 1e-4
        ys.append(y)
    # F_l ∝ k^l for the first photon multipoles
    F = np.array([y[5:11] for y in ys])
    ratio = F[0, :4] / F[1, :4]
    np.testing.assert_allclose(ratio[:4], (ks[0] / ks[1]) ** np.arange(4), rtol=1e-6)
    # adiabatic: δ/(1+w) and u/k agree across species (c, b, γ, ν, h)
    n = bg5.nstate
    for k, y in zip(ks, ys):
        Lg, Ln, Lh = 5, 5, 5
        iF, iN, iH = 5, 5 + 2 * (Lg + 1), 5 + 2 * (Lg + 1) + (Ln + 1)
        e = bg5.eval([tau])[0]
        ah = e[0]
        E = np.sqrt(x**2 + bg5.y0**2 * ah**2)
        Irho, IP = np.sum(W * E), np.sum(W * x**2 / E)
        wh = IP / (3 * Irho)
        dh = np.sum(W * E * y[iH + np.arange(4) * (Lh + 1)]) / Irho
        uh = np.sum(W * x * y[iH + 1 + np.arange(4) * (Lh + 1)]) / (Irho + IP / 3)
        d = [y[1], y[3], y[iF] / (4 / 3), y[iN] / (4 / 3), dh / (1 + wh)]
        u = [y[2] / k / k, y[4] / k / k, 0.75 * y[iF + 1] / k, 0.75 * y[iN + 1] / k, uh / k]
        assert (max(d) - min(d)) <= 1e-3 * abs(np.mean(d))
        assert (max(u) - min(u)) <= 1e-3 * abs(np.mean(u))


def test_bessel_against_scipy():
    from scipy.special import spherical_jn
    ls = np.array([0, 1, 2, 5, 10, 50, 200, 1000, 2500])
    xs = np.concatenate([[0.0, 1e-3, 0.5], np.linspace(1, 60, 40), np.linspace(100, 3000, 60), [5e4]])
    j = O.sph_bessel(ls, xs)
    ref = spherical_jn(ls[None, :], xs[:, None])
    np.testing.assert_allclose(j, ref, rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("hermite,dx", [(False, 2 * np.pi / 150), (True, 2 * np.pi / 15)])
def test_bessel_cache_accuracy(hermite, dx):
    from scipy.special import spherical_jn
    ls = np.arange(10, 101, 10)
    jl = O.BesselCache(ls, dx=dx, hermite=hermite)
    assert abs(jl(0, 0.0)[0] - spherical_jn(10, 0.0)) < 1e-16
    assert abs(jl(0, jl.xmax)[0] - spherical_jn(10, jl.xmax)) < 1e-16
    xs = np.arange(0.0, jl.xmax, 0.01)
    for il, l in enumerate(ls):
        np.testing.assert_allclose(jl(il, xs), spherical_jn(l, xs), atol=1e-5)


def test_pk_matches_class(golden, bg5):
    d = np.loadtxt(os.path.join(golden, "class_Pk.txt"))
    P, status, _ = O.spectrum_matter(bg5, d[:, 0])
    assert np.all(status == 0)
    assert np.linalg.norm(P - d[:, 1]) <= 1e-3 * np.linalg.norm(d[:, 1])


def test_cl_matches_class(golden, bg5):
    d = np.loadtxt(os.path.join(golden, "class_Cl.txt"))
    lc = d[:, 0]
    ls = np.unique(np.round(np.exp(np.linspace(np.log(lc[0]), np.log(lc[-1]), 200))).astype(int))
    jl = O.BesselCache(ls)
    Dl = O.spectrum_cmb(bg5, ["TT", "EE", "ψψ"], jl, lc)
    for j in range(3):
        assert np.linalg.norm(Dl[:, j] - d[:, j + 1]) <= 2e-3 * np.linalg.norm(d[:, j + 1])


def test_pk_self_convergence():
    ks = 10 ** np.linspace(-1, 4, 24)
    bg = O.Background(O.PLANCK18, MODEL5)
    P, st, _ = O.spectrum_matter(bg, ks)
    bgt = O.Background(O.PLANCK18, MODEL5, bg_rtol=1e-10, bg_atol=1e-10, pt_rtol=1e-9, pt_atol=1e-9,
                       maxiters=10**6)
    P0, st0, _ = O.spectrum_matter(bgt, ks, kτini=0.0, τinimax=0.0)
    assert np.all(st == 0) and np.all(st0 == 0)
    assert np.all(np.abs(P / P0 - 1) < 1e-3)


def test_failed_modes_report_status(bg5):
    _, st, _ = bg5.solve_pt(np.array([0.0, np.nan, 1.0]), 1e-4, mode=1)
    assert st[0] != 0 and st[1] != 0 and st[2] == 0


def test_mlp_oracle_gradient_matches_finite_differences():
    """The MLP oracle's backpropagation against central finite differences (FP64)."""
    import mlp as MO
    rng = np.random.default_rng(3)
    sizes = MO.layer_sizes(3, 8, 2, 2)
    n = sum(a * b + b for a, b in zip(sizes[:-1], sizes[1:]))
    p = rng.normal(0, 0.5, n)
    X, Y = rng.normal(size=(5, 3)), rng.normal(size=(5, 2))
    loss, g = MO.loss_and_grad(p, X, Y, sizes)
    h = 1e-6
    fd = np.array([(MO.loss_and_grad(p + h * e, X, Y, sizes)[0] - MO.loss_and_grad(p - h * e, X, Y, sizes)[0]) / (2 * h)
                   for e in np.eye(n)])
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-9)
    assert MO.bf16_round(np.array([1.0, 1.00390625, 3.14159]))[2] == 3.140625


def test_sparse_lu_path_equals_dense_checker():
    """The oracle's sparse-LU path (the timed CPU baseline and the fast checker of the large
    workloads) integrates the same equations with the same Rodas5P steps as the dense-LU checker:
    same step counts, sources equal to rounding (the two eliminations order their operations
    differently), on the massive-ν, l_γ = 30 model at low and intermediate k."""
    m = dict(lmax_g=30, lmax_nu=10, lmax_h=10, nx=5, Hswitch=1, Heswitch=6, reionization=1)
    p = dict(O.PLANCK18, m_nu_eV=0.06, N_nu=1.0, Neff=2.0328)
    ks = np.array([0.05, 3.0, 60.0, 300.0])
    out = {}
    for ls in ("dense", "sparse"):
        bg = O.Background(p, m, linsolve=ls)
        taus = np.linspace(bg.tau0 * 0.01, bg.tau0 * 0.99, 40)
        S, st, stats = bg.solve_pt(ks, bg.t[0], taus, mode=0)
        assert np.all(st == 0)
        out[ls] = (S, stats)
    np.testing.assert_array_equal(out["dense"][1], out["sparse"][1])
    scale = np.max(np.abs(out["dense"][0]), axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(out["dense"][0] - out["sparse"][0]) / scale) < 1e-8  # measured 1.5e-9
