"""GB300 drop-in for the perturbation + line-of-sight path of SymBoltz.jl.

Same surface as the reference module (src/SymBoltz.jl:50-59): build a model with ``ΛCDM``/``LCDM``
(src/models/cosmologies.jl:27-48), parameters with ``parameters_Planck18`` (src/parameters.jl),
then ``CosmologyProblem`` -> ``solve``/``solvebg``/``solvept`` (src/solve.jl) and the observables
``spectrum_matter`` (src/observables/fourier.jl:74-101), ``source_grid`` (fourier.jl:267-291),
``SphericalBesselCache``, ``los_integrate`` and ``spectrum_cmb`` (src/observables/angular.jl).
All numerical work runs in libsymboltz_gb300.so on the GPU; this module only marshals arrays.
Units: τ in 1/H0, k in H0/c.  ``k_from_hMpc`` converts h/Mpc.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import SbzError

__all__ = [
    "ΛCDM", "LCDM", "parameters_Planck18", "CosmologyProblem", "CosmologySolution", "solve", "solvebg", "solvept",
    "issuccess", "spectrum_primordial", "spectrum_matter", "source_grid", "SphericalBesselCache", "los_integrate",
    "spectrum_cmb", "lingrid", "loggrid", "cosgrid", "ChebyshevInterpolator", "CubicSplineInterpolator",
    "momentum_quadrature", "k_from_hMpc", "SbzError", "parameter_updater", "source_grid_adaptive",
]

C_LIGHT = 299792458.0


def k_from_hMpc(k):
    """k in h/Mpc -> H0/c units (src/constants.jl:19 k0)."""
    return np.asarray(k, dtype=np.float64) * (C_LIGHT / 1e5)


# ----------------------------------------------------------------------------------------------
@dataclass
class Model:
    """Options of the ΛCDM model (src/models/cosmologies.jl:27-48)."""
    lmax_gamma: int = 10
    lmax_nu: int = 10
    lmax_h: int = 10
    nx_h: int = 4
    Hswitch: int = 1
    Heswitch: int = 6
    reionization: bool = True

    @property
    def massive_nu(self):
        return self.nx_h > 0

    def c(self):
        return L.Model(self.lmax_gamma, self.lmax_nu, self.lmax_h if self.nx_h else 3, self.nx_h, self.Hswitch,
                       self.Heswitch, int(bool(self.reionization)))


def ΛCDM(*, lmax=10, lmax_gamma=None, lmax_nu=None, lmax_h=None, nx=4, massive_nu=True, Hswitch=1, Heswitch=6,
         reionization=True):
    """ΛCDM(lmax, Hswitch, Heswitch, reionization); separate hierarchy truncations may be given."""
    return Model(lmax_gamma or lmax, lmax_nu or lmax, lmax_h or lmax, nx if massive_nu else 0, Hswitch, Heswitch,
                 reionization)


LCDM = ΛCDM


def parameters_Planck18(M: Model | None = None):
    """Planck 2018 parameters as used by the reference (src/parameters.jl:1-21)."""
    h = 0.6736
    p = dict(h=h, Omega_c=0.1200 / h**2, Omega_b=0.0224 / h**2, T0=2.7255, Neff=2.99, YHe=0.2454,
             ln_As1e10=math.log(2.099e-9 * 1e10), ns=0.965, m_nu_eV=0.02, N_nu=3.0)
    if M is not None and not M.massive_nu:
        p["m_nu_eV"], p["N_nu"] = 0.0, 0.0
    return p


def momentum_quadrature(N=4):
    """Momentum bins x_i and weights W_i (src/models/neutrinos.jl:55-60)."""
    x, W = np.zeros(N), np.zeros(N)
    L.check(L.lib().sbz_momentum_quadrature(N, L.dptr(x), L.dptr(W)), "momentum_quadrature")
    return x, W


_PKEYS = ("h", "Omega_c", "Omega_b", "T0", "Neff", "YHe", "ln_As1e10", "ns", "m_nu_eV", "N_nu")


def _params_c(pars):
    if isinstance(pars, dict):
        pars = [pars]
    arr = (L.Params * len(pars))()
    for i, p in enumerate(pars):
        arr[i] = L.Params(*[float(p.get(k, 0.0)) for k in _PKEYS])
    return arr, len(pars)


class CosmologyProblem:
    """CosmologyProblem(M, pars) (src/solve.jl:129-236).  ``pars`` may be a list of parameter dicts:
    all of them share the model and are solved together (one kernel launch for all their modes)."""

    def __init__(self, M: Model, pars, *, bg_rtol=1e-7, bg_atol=1e-7, pt_rtol=1e-5, pt_atol=1e-5, ivspan=(1e-6, 100.0),
                 maxiters=100000, precision="mixed", refine_iters=3, table_points=8192, warps_per_block=0,
                 warps_per_mode=0, blocks_per_sm=0, los_precision=None, refine_skip=None):
        self.M = M
        self.pars = [dict(p) for p in ([pars] if isinstance(pars, dict) else pars)]
        o = L.Opts()
        L.lib().sbz_default_opts(C.byref(o))
        o.bg_rtol, o.bg_atol, o.pt_rtol, o.pt_atol = bg_rtol, bg_atol, pt_rtol, pt_atol
        o.tau_ini, o.tau_max = ivspan
        o.maxiters = maxiters
        o.precision = {"mixed": L.SBZ_MIXED, "fp64": L.SBZ_FP64}[precision]
        o.refine_iters, o.table_points, o.warps_per_block = refine_iters, table_points, warps_per_block
        o.warps_per_mode, o.blocks_per_sm = warps_per_mode, blocks_per_sm
        o.los_precision = -1 if los_precision is None else {"fp64": L.SBZ_FP64, "mixed": L.SBZ_MIXED}[los_precision]
        if refine_skip is not None:
            o.refine_skip = refine_skip
        self.opts = o
        self._m = M.c()
        pc, n = _params_c(self.pars)
        h = C.c_void_p()
        L.check(L.lib().sbz_problem_create(C.byref(self._m), pc, n, C.byref(o), C.byref(h)), "CosmologyProblem")
        self._h = h
        self.ncosmo = n
        self.nstate = L.lib().sbz_problem_nstate(h)
        self.bg = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib().sbz_problem_destroy(h)
            self._h = None

    def set_params(self, pars):
        """Replace the parameter sets in place (one dict or a list; the count may change), keeping the
        model, options, stream and device buffers; the background is solved again on next use."""
        self.pars = [dict(p) for p in ([pars] if isinstance(pars, dict) else pars)]
        pc, n = _params_c(self.pars)
        L.check(L.lib().sbz_problem_set_params(self._h, pc, n), "set_params")
        self.ncosmo = n
        self.bg = None
        return self

    def solvebg(self):
        if self.bg is None:
            n = self.ncosmo
            t0, k0, tr = np.zeros(n), np.zeros(n), np.zeros(n)
            st = np.zeros(n, dtype=np.int32)
            L.check(L.lib().sbz_solve_bg(self._h, L.dptr(t0), L.dptr(k0), L.dptr(tr), L.iptr(st)), "solvebg")
            self.bg = BackgroundSolution(self, t0, k0, tr, st)
        return self.bg


@dataclass
class BackgroundSolution:
    prob: CosmologyProblem
    tau0: np.ndarray
    kappa0: np.ndarray
    taurec: np.ndarray
    status: np.ndarray

    def t(self, c=0):
        """Background solution times (bgsol.t) of cosmology c."""
        n = L.lib().sbz_bg_knots(self.prob._h, c, 0, None, None)
        L.check(n, "bg_knots")
        t = np.zeros(n)
        L.lib().sbz_bg_knots(self.prob._h, c, n, L.dptr(t), None)
        return t

    def eval(self, taus, c=0):
        """a, ℋ, κ̇, κ, v, v̇, c_s², Xe, Tb at taus."""
        taus = L.f64(np.atleast_1d(taus))
        out = np.zeros((len(taus), 9))
        L.check(L.lib().sbz_bg_eval(self.prob._h, c, len(taus), L.dptr(taus), L.dptr(out)), "bg_eval")
        return out


    def coefficients(self, taus, c=0):
        """a, ℋ, κ̇, c_s², e^{-κ}, κ̈, κ⃛ as the GPU kernels interpolate them."""
        taus = L.f64(np.atleast_1d(taus))
        out = np.zeros((len(taus), 7))
        L.check(L.lib().sbz_bg_coefficients(self.prob._h, c, len(taus), L.dptr(taus), L.dptr(out)), "bg_coefficients")
        return out


def parameter_updater(prob: CosmologyProblem, idxs, *, inplace=False):
    """parameter_updater(prob, idxs) (src/solve.jl:271-306): a function that takes values for the
    parameter names `idxs` (a sequence in that order, or a dict by name) and returns a problem with
    them updated.  Like the reference it returns a new problem and leaves `prob` as it was; with
    inplace=True it re-uploads into `prob` itself (sbz_problem_set_params: no new device
    allocations).  A 2-D array of values (one row per cosmology) updates that many parameter sets,
    the unnamed parameters taken from the first of `prob`'s."""
    idxs = list(idxs)
    for k in idxs:
        if k not in _PKEYS:
            raise KeyError(f"unknown parameter {k!r}; known: {', '.join(_PKEYS)}")

    def updater(p):
        rows = [[p[k] for k in idxs]] if isinstance(p, dict) else np.atleast_2d(np.asarray(p, dtype=np.float64))
        if np.shape(rows)[1] != len(idxs):
            raise ValueError(f"expected {len(idxs)} values per parameter set")
        new = [dict(prob.pars[0], **{k: float(v) for k, v in zip(idxs, row)}) for row in rows]
        if inplace:
            return prob.set_params(new)
        o = prob.opts
        return CosmologyProblem(prob.M, new, bg_rtol=o.bg_rtol, bg_atol=o.bg_atol, pt_rtol=o.pt_rtol, pt_atol=o.pt_atol,
                                ivspan=(o.tau_ini, o.tau_max), maxiters=o.maxiters,
                                precision={L.SBZ_MIXED: "mixed", L.SBZ_FP64: "fp64"}[o.precision], refine_iters=o.refine_iters,
                                table_points=o.table_points, warps_per_block=o.warps_per_block, warps_per_mode=o.warps_per_mode,
                                blocks_per_sm=o.blocks_per_sm,
                                los_precision=None if o.los_precision < 0 else {L.SBZ_FP64: "fp64", L.SBZ_MIXED: "mixed"}[o.los_precision],
                                refine_skip=o.refine_skip)

    return updater


def solvebg(prob: CosmologyProblem):
    """solvebg (src/solve.jl:427-435)."""
    return prob.solvebg()


_OUT = {"sources": L.SBZ_OUT_SOURCES, "delta_m": L.SBZ_OUT_DELTA_M, "state": L.SBZ_OUT_STATE, "sources4": L.SBZ_OUT_SOURCES4, "factors": L.SBZ_OUT_FACTORS}


def autotune(prob: CosmologyProblem, ks, ptivini=-np.inf, *, saveat=None, output="sources", cosmo=None):
    """Pick the perturbation kernel's launch shape (warps per mode, blocks per SM) for this workload
    by timing the candidates on a k-stratified sample of it (``sbz_autotune_pt``); the choice is
    stored in the problem and used by later solves.  Returns {"warps_per_mode", "blocks_per_sm",
    "candidates_ms": {(nw, bps): ms}}."""
    prob.solvebg()
    ks = L.f64(np.atleast_1d(ks))
    nk = len(ks)
    ti = np.asarray(ptivini(ks) if callable(ptivini) else np.full(nk, ptivini), dtype=np.float64)
    ti = L.f64(np.broadcast_to(ti, (nk,)))
    cos = L.i32(np.zeros(nk) if cosmo is None else cosmo)
    kind = _OUT[output]
    if kind == L.SBZ_OUT_DELTA_M:
        taus = np.zeros((prob.ncosmo, 0))
    else:
        taus = np.asarray(saveat, dtype=np.float64)
        taus = np.broadcast_to(taus, (prob.ncosmo, taus.shape[-1])) if taus.ndim == 1 else taus
    taus = L.f64(taus)
    best = L.i32(np.zeros(2))
    ms = L.f64(np.zeros(7))
    L.check(L.lib().sbz_autotune_pt(prob._h, nk, L.iptr(cos), L.dptr(ks), L.dptr(ti), taus.shape[1], L.dptr(taus), kind,
                                    L.iptr(best), L.dptr(ms)), "autotune")
    cands = [(1, 0), (2, 0), (2, 2), (4, 1), (4, 2), (4, 3), (8, 1)]
    prob.opts.warps_per_mode, prob.opts.blocks_per_sm = int(best[0]), int(best[1])
    return {"warps_per_mode": int(best[0]), "blocks_per_sm": int(best[1]), "candidates_ms": {c: float(m) for c, m in zip(cands, ms)}}


def solvept(prob: CosmologyProblem, ks, ptivini=-np.inf, *, saveat=None, output="state", cosmo=None):
    """solvept (src/solve.jl:543-569) for modes ks (cosmology index per mode in ``cosmo``).

    ``ptivini`` is a number or a function of k, clamped to the background span.  ``saveat`` is a 1-d
    array of times (one cosmology) or a (ncosmo, ntau) array.  Returns (out, status, steps); out is
    [nk, ntau, nstate] for output="state", [nk, ntau, 3] (k S_T, k² S_E, S_ψ) for "sources" and [nk]
    Δ_m(τ0) for "delta_m"."""
    prob.solvebg()
    ks = L.f64(np.atleast_1d(ks))
    nk = len(ks)
    ti = np.asarray(ptivini(ks) if callable(ptivini) else np.full(nk, ptivini), dtype=np.float64)
    ti = L.f64(np.broadcast_to(ti, (nk,)))
    cos = L.i32(np.zeros(nk) if cosmo is None else cosmo)
    kind = _OUT[output]
    if kind == L.SBZ_OUT_DELTA_M:
        taus = np.zeros((prob.ncosmo, 0))
    else:
        taus = np.asarray(saveat, dtype=np.float64)
        taus = np.broadcast_to(taus, (prob.ncosmo, taus.shape[-1])) if taus.ndim == 1 else taus
    taus = L.f64(taus)
    ntau = taus.shape[1]
    shape = {L.SBZ_OUT_DELTA_M: (nk,), L.SBZ_OUT_SOURCES: (nk, ntau, 3), L.SBZ_OUT_SOURCES4: (nk, ntau, 4), L.SBZ_OUT_FACTORS: (nk, ntau, 7),
             L.SBZ_OUT_STATE: (nk, ntau, prob.nstate)}[kind]
    out = np.zeros(shape)
    st = np.zeros(nk, dtype=np.int32)
    steps = np.zeros((nk, 2), dtype=np.int64)
    L.check(L.lib().sbz_solve_pt(prob._h, nk, L.iptr(cos), L.dptr(ks), L.dptr(ti), ntau, L.dptr(taus), kind,
                                 L.dptr(out), L.iptr(st), L.i64ptr(steps)), "solvept")
    return out, st, steps


def _isapprox(x, y, atol, rtol, norm):
    """Julia's isapprox for arrays: norm(x - y) <= max(atol, rtol * max(norm(x), norm(y)))."""
    return norm(x - y) <= max(atol, rtol * max(norm(x), norm(y)))


def refine_grid(fun, ks, *, atol=0.0, rtol=None, norm=np.linalg.norm, ktransform=(lambda k: k, lambda k: k), maxks=1024,
                compare=slice(None), sort=True):
    """Adaptive k refinement of source_grid_adaptive (src/observables/fourier.jl:312-410), level by
    level: every interval (k1, k3) whose midpoint value (midpoint in ktransform space) is not
    isapprox the linear interpolation (S1 + S3)/2 at the compared rows is split, and all midpoints of
    a level are evaluated in one call fun(k_array) -> values[len(k_array), rows, ...].  An interval's
    decision depends only on its end and midpoint values, so the refined grid is the reference's
    whatever the evaluation order.  rtol defaults to √eps when atol == 0 (Julia's default)."""
    f, finv = ktransform
    rtol = (np.sqrt(np.finfo(float).eps) if atol == 0 else 0.0) if rtol is None else rtol
    ks = [float(k) for k in ks]
    if len(ks) < 2:
        raise ValueError("Initial k-grid must have at least 2 values")
    for k in (min(ks), max(ks)):
        if not np.isclose(finv(f(k)), k):
            raise ValueError("ktransform is not a tuple of inverse functions")
    vals = list(np.asarray(fun(np.array(ks))))
    todo = [(i - 1, i) for i in range(1, len(ks))]
    while todo:
        if len(ks) + len(todo) > maxks:
            raise ValueError(f"Source function refinement needs more than {maxks} k-refinements. Reduce refinement criteria.")
        mids = np.array([finv((f(ks[a]) + f(ks[b])) / 2) for a, b in todo])
        new = np.asarray(fun(mids))
        nxt = []
        for (a, b), km, sm in zip(todo, mids, new):
            m = len(ks)
            ks.append(float(km))
            vals.append(sm)
            si = (vals[a] + vals[b]) / 2
            rows = range(sm.shape[0])[compare] if sm.ndim >= 1 else [None]
            bad = any(not _isapprox(sm[r], si[r], atol, rtol, norm) for r in rows) if sm.ndim >= 1 else \
                not _isapprox(np.atleast_1d(sm), np.atleast_1d(si), atol, rtol, norm)
            if bad:
                nxt += [(m, b), (a, m)]
        todo = nxt
    ks = np.array(ks)
    vals = np.array(vals)
    if sort:
        o = np.argsort(ks, kind="stable")
        ks, vals = ks[o], vals[o]
    return ks, vals


def source_grid_adaptive(prob: CosmologyProblem, taus, ks, *, output="sources", ptivini=-np.inf, cosmo=0, atol=0.0, rtol=None,
                         norm=np.linalg.norm, ktransform=(lambda k: k, lambda k: k), maxks=1024, sort=True):
    """source_grid_adaptive (src/observables/fourier.jl:312-410) on the GPU: each refinement level's
    midpoints are solved in one perturbation launch.  taus = None: final time only.  Returns (ks,
    values[len(ks), ntau, 3]) for output "sources", (ks, Δm[len(ks)]) for "delta_m"."""
    prob.solvebg()
    if taus is None:
        taus = np.array([prob.bg.tau0[cosmo] * (1 - 1e-12)])
    taus = np.atleast_1d(np.asarray(taus, dtype=np.float64))
    nt = len(taus)
    compare = slice(0, max(nt - 1, 1))  # χ = 0 excluded (sources ∝ 1/χ), unless it is the only time

    def fun(kk):
        tt = np.broadcast_to(taus, (prob.ncosmo, nt)) if prob.ncosmo > 1 else taus
        out, st, _ = solvept(prob, kk, ptivini, saveat=None if output == "delta_m" else tt, output=output,
                             cosmo=np.full(len(kk), cosmo))
        if np.any(st != 0):
            raise L.SbzError(f"{int(np.count_nonzero(st))} modes failed during k refinement")
        return out

    return refine_grid(fun, ks, atol=atol, rtol=rtol, norm=norm, ktransform=ktransform, maxks=maxks, compare=compare, sort=sort)


def state_index(M: Model):
    """Map from the oracle/reference ordering [Φ, δc, θc, δb, θb, F0..FLγ, G0..GLγ, N0..NLν, ψ_{j,0..Lh}]
    to this library's state ordering (chains after the photon-baryon head)."""
    Lg, Ln, Lh, nx = M.lmax_gamma, M.lmax_nu, M.lmax_h, M.nx_h
    idx = list(range(5))
    oFt, oGt = 11, 11 + Lg - 2
    idx += [5 + l if l <= 2 else oFt + l - 3 for l in range(Lg + 1)]
    idx += [8 + l if l <= 2 else oGt + l - 3 for l in range(Lg + 1)]
    oN = oGt + Lg - 2
    idx += [oN + l for l in range(Ln + 1)]
    oH = oN + Ln + 1
    idx += [oH + j * (Lh + 1) + l for j in range(nx) for l in range(Lh + 1)]
    return np.array(idx)


def pt_rhs(prob: CosmologyProblem, ks, taus, Y, cosmo=None):
    """f = J(τ) y and ∂f/∂τ for states Y [nk, nstate] (library ordering) — the ODE function."""
    prob.solvebg()
    ks, taus, Y = L.f64(np.atleast_1d(ks)), L.f64(np.atleast_1d(taus)), L.f64(np.atleast_2d(Y))
    nk = len(ks)
    cos = L.i32(np.zeros(nk) if cosmo is None else cosmo)
    f, ft = np.zeros_like(Y), np.zeros_like(Y)
    L.check(L.lib().sbz_pt_rhs(prob._h, nk, L.iptr(cos), L.dptr(ks), L.dptr(taus), L.dptr(Y), L.dptr(f), L.dptr(ft)), "pt_rhs")
    return f, ft


@dataclass
class CosmologySolution:
    prob: CosmologyProblem
    bg: BackgroundSolution
    ks: np.ndarray | None = None
    states: np.ndarray | None = None  # [nk, nstate] at τ0
    status: np.ndarray | None = None
    steps: np.ndarray | None = None


def solve(prob: CosmologyProblem, ks=None, *, ptivini=-np.inf):
    """solve(prob, ks) (src/solve.jl:380-402): background, then the perturbation modes (final states)."""
    bg = prob.solvebg()
    if ks is None:
        return CosmologySolution(prob, bg)
    ks = L.f64(np.atleast_1d(ks))
    out, st, steps = solvept(prob, ks, ptivini, saveat=np.array([bg.tau0[0]]), output="state")
    return CosmologySolution(prob, bg, ks, out[:, 0, :], st, steps)


def issuccess(sol: CosmologySolution):
    """issuccess (src/solve.jl:604-606)."""
    ok = bool(np.all(sol.bg.status == 0))
    return ok and (sol.status is None or bool(np.all(sol.status == 0)))


def spectrum_primordial(k, prob: CosmologyProblem, c=0):
    """P0(k) = 2π² As/k³ (k/k_pivot)^(ns-1) (src/observables/fourier.jl:14-30)."""
    k = L.f64(np.atleast_1d(k))
    P0 = np.zeros(len(k))
    L.check(L.lib().sbz_spectrum_primordial(prob._h, c, len(k), L.dptr(k), L.dptr(P0)), "spectrum_primordial")
    return P0


def spectrum_matter(prob: CosmologyProblem, ks, *, kτini=1e-2, τinimax=1e-4, cosmo=None, return_status=False,
                    sourceopts=None, coarse_length=9):
    """Linear P(k, τ0) = P0 Δ_m² (src/observables/fourier.jl:79-101).

    ks = (kmin, kmax): the adaptive form (fourier.jl:103-125) — a coarse_length-point log grid
    refined in log k until Δ_m at each midpoint is within sourceopts (default atol 4, rtol 4e-3) of
    the linear interpolation, modes started at the first background time; returns (ks, P)."""
    if isinstance(ks, tuple) and len(ks) == 2:
        c = 0 if cosmo is None else int(cosmo)
        kmin, kmax = (float(k) for k in ks)
        k0 = loggrid(kmin, kmax, length=coarse_length)
        opts = dict(atol=4.0, rtol=4e-3) if sourceopts is None else dict(sourceopts)
        kk, dm = source_grid_adaptive(prob, None, k0, output="delta_m", cosmo=c, ktransform=(np.log, np.exp), **opts)
        return kk, spectrum_primordial(kk, prob, c) * dm**2
    prob.solvebg()
    ks = L.f64(np.atleast_1d(ks))
    nk = len(ks)
    cos = L.i32(np.zeros(nk) if cosmo is None else cosmo)
    P = np.zeros(nk)
    st = np.zeros(nk, dtype=np.int32)
    L.check(L.lib().sbz_spectrum_matter(prob._h, nk, L.iptr(cos), L.dptr(ks), kτini, τinimax, L.dptr(P), L.iptr(st)),
            "spectrum_matter")
    return (P, st) if return_status else P


# ----------------------------------------------------------------------------------------------
# grids and k-interpolators (src/utils.jl:269-292, src/observables/fourier.jl:195-571)
def lingrid(a, b, *, step=None, length=None):
    if step is not None:
        length = int(math.ceil((b - a) / step)) + 1
    return np.linspace(a, b, length)


def loggrid(a, b, *, length):
    x = np.exp(lingrid(math.log(a), math.log(b), length=length))
    x[0], x[-1] = a, b
    return x


def cosgrid(a, b, *, length):
    return a + (b - a) * (1 - np.cos(np.pi * lingrid(0.0, 0.5, length=length)))


class ChebyshevInterpolator:
    """Chebyshev k-grid + barycentric interpolation in y = f(k) (fourier.jl:419-459,524-535)."""

    def __init__(self, xmin, xmax, order, f=None, finv=None):
        self.f = f or (lambda x: x)
        finv = finv or (lambda y: y)
        ymin, ymax = self.f(xmin), self.f(xmax)
        j = np.arange(order + 1)
        self.ys = 0.5 * (ymin + ymax) + 0.5 * (ymax - ymin) * np.cos(np.pi * j / order)
        self.xs = np.asarray(finv(self.ys), dtype=np.float64)
        self.xs[-1], self.xs[0] = xmin, xmax
        self.ws = np.where(j % 2 == 0, 1.0, -1.0)
        self.ws[0] /= 2
        self.ws[-1] /= 2

    def matrix(self, kfine):
        y = self.f(np.asarray(kfine, dtype=np.float64))
        dy = y[:, None] - self.ys[None, :]
        exact = dy == 0
        with np.errstate(divide="ignore", invalid="ignore"):
            t = self.ws[None, :] / dy
            M = t / t.sum(axis=1, keepdims=True)
        rows = exact.any(axis=1)
        M[rows] = exact[rows].astype(np.float64)
        return M


class CubicSplineInterpolator:
    """Natural cubic spline in f(k) through the solved modes (fourier.jl:199-231)."""

    def __init__(self, xs, f=None):
        self.xs = np.asarray(xs, dtype=np.float64)
        self.f = f or (lambda x: x)
        self.ys = self.f(self.xs)

    def matrix(self, kfine):
        n = len(self.xs)
        M = np.zeros((len(kfine), n))
        for j in range(n):
            e = np.zeros(n)
            e[j] = 1.0
            M[:, j] = _natural_spline(self.ys, e, self.f(np.asarray(kfine, dtype=np.float64)))
        return M


def _natural_spline(x, y, xq):
    n = len(x)
    h = np.diff(x)
    A = np.zeros((n, n))
    r = np.zeros(n)
    A[0, 0] = A[-1, -1] = 1
    for i in range(1, n - 1):
        A[i, i - 1], A[i, i], A[i, i + 1] = h[i - 1], 2 * (h[i - 1] + h[i]), h[i]
        r[i] = 6 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    z = np.linalg.solve(A, r)
    i = np.clip(np.searchsorted(x, xq) - 1, 0, n - 2)
    a, b = x[i + 1] - xq, xq - x[i]
    hh = h[i]
    return z[i] * a**3 / (6 * hh) + z[i + 1] * b**3 / (6 * hh) + (y[i + 1] / hh - z[i + 1] * hh / 6) * b + (y[i] / hh - z[i] * hh / 6) * a


def fk_tanh(k, k0=2000.0):
    return np.tanh(np.asarray(k) / k0)


def fkinv_tanh(y, k0=2000.0):
    return k0 * np.arctanh(np.asarray(y))


def source_grid(prob: CosmologyProblem, taus, ks, kinterp=None, *, cosmo=0):
    """Sources (k S_T, k² S_E, S_ψ) on (τ, k) (src/observables/fourier.jl:267-291): solved at ks, or at
    kinterp.xs and interpolated to ks.  Returns [ntau, nk, 3]."""
    prob.solvebg()
    taus = L.f64(taus)
    ti = prob.opts.tau_ini
    if kinterp is None:
        out, st, _ = solvept(prob, ks, ti, saveat=taus, output="sources", cosmo=np.full(len(ks), cosmo))
        return np.ascontiguousarray(out.transpose(1, 0, 2)), st
    out, st, _ = solvept(prob, kinterp.xs, ti, saveat=taus, output="sources", cosmo=np.full(len(kinterp.xs), cosmo))
    M = kinterp.matrix(ks)
    return np.einsum("fc,cts->tfs", M, out), st


# ----------------------------------------------------------------------------------------------
class SphericalBesselCache:
    """SphericalBesselCache(ls; xmax = 20 ls[end], dx = 2π/15, hermite) (angular.jl:18-26), on the GPU."""

    def __init__(self, ls, *, xmax=None, dx=2 * np.pi / 15, hermite=True):
        la = np.asarray(ls, dtype=np.float64)
        if la.size == 0 or np.any(la != np.round(la)) or np.any(la < 0):
            raise ValueError("SphericalBesselCache: the multipoles must be non-negative integers "
                             "(non-integer l, which the reference's cache also accepts, is not supported)")
        self.l = L.i32(la)
        self.xmax = float(20 * self.l[-1] if xmax is None else xmax)
        self.dx = dx
        h = C.c_void_p()
        L.check(L.lib().sbz_bessel_create(len(self.l), L.iptr(self.l), self.xmax, dx, int(hermite), C.byref(h)),
                "SphericalBesselCache")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib().sbz_bessel_destroy(h)
            self._h = None

    def __call__(self, il, x):
        x = L.f64(np.atleast_1d(x))
        out = np.zeros(len(x))
        L.check(L.lib().sbz_bessel_eval(self._h, int(il), len(x), L.dptr(x), L.dptr(out)), "jl")
        return out


def los_integrate(Ss, ls, taus, ks, jl: SphericalBesselCache, *, l_limber=2**31 - 1):
    """Iₗ(k) = ∫dτ S(τ,k) jₗ(k(τ0-τ)) (angular.jl:109-185).  Ss [ntau, nk] or [ntau, nk, nsrc];
    returns [nk, nl] or [nk, nl, nsrc]."""
    if not np.array_equal(np.asarray(ls), jl.l):
        raise ValueError("ls must match the l-values stored in the Bessel cache")
    S = L.f64(Ss)
    squeeze = S.ndim == 2
    if squeeze:
        S = S[:, :, None]
    nt, nk, ns = S.shape
    out = np.zeros((nk, len(jl.l), ns))
    L.check(L.lib().sbz_los_integrate(jl._h, ns, L.dptr(S), nt, L.dptr(L.f64(taus)), nk, L.dptr(L.f64(ks)),
                                      int(min(l_limber, 2**31 - 1)), L.dptr(out)), "los_integrate")
    return out[:, :, 0] if squeeze else out


def _cl_kint(ThA, ThB, P0s, ls, ks, normalization="Cl"):
    ThA, ThB = L.f64(ThA), L.f64(ThB)
    nk, nl = ThA.shape
    Cl = np.zeros(nl)
    L.check(L.lib().sbz_cl_integrate(nk, L.dptr(L.f64(ks)), L.dptr(L.f64(P0s)), nl, L.dptr(ThA), L.dptr(ThB),
                                     L.dptr(Cl)), "spectrum_cmb")
    ls = np.asarray(ls, dtype=np.float64)
    return Cl * ls * (ls + 1) / (2 * np.pi) if normalization == "Dl" else Cl


def spectrum_cmb(*args, **kw):
    """spectrum_cmb(ΘA, ΘB, P0s, ls, ks; normalization) — the k-integral (angular.jl:198-223), or
    spectrum_cmb(modes, prob, jl[, ls]; normalization, kinterp, Δkτ0, xs, τcut, l_limber) — the full driver
    (angular.jl:260-359), returning [nl, nmodes]."""
    if isinstance(args[0], np.ndarray):
        return _cl_kint(*args, **kw)
    return _spectrum_cmb_driver(*args, **kw)


def _spectrum_cmb_driver(modes, prob: CosmologyProblem, jl: SphericalBesselCache, ls_out=None, *, normalization="Cl",
                         kinterp=None, Δkτ0=np.pi, xs=None, τcut=1e-2, l_limber=10, cosmo=0, taus=None, return_status=False,
                         sources=None):
    """Grids as in the reference driver; everything after them runs in one device pipeline
    (sbz_spectrum_cmb): coarse solve -> k-interpolation -> line of sight -> Θ scaling -> C_l."""
    modes = [modes] if isinstance(modes, str) else list(modes)
    joined = "".join(modes)
    iT = "T" in joined
    iP = "ψ" in joined
    if kinterp is None:
        kinterp = (ChebyshevInterpolator(1e-2, 1e4, 130, fk_tanh, fkinv_tanh) if iP else ChebyshevInterpolator(1e-2, 2e3, 60))
    bg = prob.solvebg()
    if bg.status[cosmo] != 0:
        raise SbzError(f"background of cosmology {cosmo} failed (status {bg.status[cosmo]})")
    ls = jl.l.astype(np.float64)
    tau0 = bg.tau0[cosmo]
    kmin, kmax = float(np.min(kinterp.xs)), float(np.max(kinterp.xs))
    ks_fine = lingrid(kmin, kmax, step=Δkτ0 / tau0)
    if taus is None:  # background times >= τcut, resampled on the fractional grid xs (angular.jl:280-290)
        t = bg.t(cosmo)
        t = t[t >= τcut]
        xs = cosgrid(0.0, 1.0, length=300) if xs is None else np.asarray(xs)
        taus = t[0] + (t[-1] - t[0]) * xs
    taus = L.f64(taus)
    code = {"T": 0, "E": 1, "ψ": 2}
    pa = L.i32([code[m[0]] for m in modes])
    pb = L.i32([code[m[-1]] for m in modes])
    if isinstance(kinterp, ChebyshevInterpolator):
        kind, yc, wc = L.SBZ_KINTERP_BARYCENTRIC, L.f64(kinterp.ys), L.f64(kinterp.ws)
    else:
        kind, yc, wc = L.SBZ_KINTERP_SPLINE, L.f64(kinterp.ys), L.f64(np.zeros(len(kinterp.xs)))
    xs_c = L.f64(kinterp.xs)
    yf = L.f64(kinterp.f(ks_fine))
    nl = len(ls)
    Cl = np.zeros((len(modes), nl))
    st = np.zeros(len(xs_c), dtype=np.int32)
    if sources is None:
        L.check(L.lib().sbz_spectrum_cmb(prob._h, cosmo, jl._h, len(xs_c), L.dptr(xs_c), L.dptr(yc), L.dptr(wc), kind,
                                         len(taus), L.dptr(taus), len(ks_fine), L.dptr(L.f64(ks_fine)), L.dptr(yf), len(modes),
                                         L.iptr(pa), L.iptr(pb), int(l_limber), L.dptr(Cl), L.iptr(st)), "spectrum_cmb")
    else:  # coarse sources supplied by the caller (k S_T, k² S_E, S_ψ) on (kinterp.xs, taus)
        src = L.f64(np.asarray(sources, dtype=np.float64).reshape(len(xs_c), len(taus), 3))
        L.check(L.lib().sbz_spectrum_cmb_sources(prob._h, cosmo, jl._h, len(xs_c), L.dptr(xs_c), L.dptr(yc), L.dptr(wc), kind,
                                                 len(taus), L.dptr(taus), L.dptr(src), len(ks_fine), L.dptr(L.f64(ks_fine)),
                                                 L.dptr(yf), len(modes), L.iptr(pa), L.iptr(pb), int(l_limber), L.dptr(Cl)),
                "spectrum_cmb_sources")
    out = Cl.T.copy()
    if normalization == "Dl":
        out *= (ls * (ls + 1) / (2 * np.pi))[:, None]
    if ls_out is not None:
        ls_out = np.asarray(ls_out, dtype=np.float64)
        out = np.stack([_natural_spline(ls, out[:, i], ls_out) for i in range(len(modes))], axis=1)
    return (out, st) if return_status else out


def timings(prob: CosmologyProblem):
    """CUDA-event phase durations (ms) of the last spectrum_cmb pipeline:
    h2d, perturbations, kinterp, los, cl, d2h, total."""
    t = np.zeros(8)
    L.check(L.lib().sbz_problem_timings(prob._h, L.dptr(t)), "timings")
    return dict(zip(("h2d", "perturbations", "kinterp", "los", "cl", "d2h", "total"), t[:7]))
