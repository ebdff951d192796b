"""ctypes wrapper and spectrum drivers for the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline may import this module, and only as the checker; the product package never does.

The drivers restate the reference's orchestration in numpy:
  * ``spectrum_matter``  src/observables/fourier.jl:74-101 (ptivini = min(kτini/k, τinimax))
  * ``spectrum_cmb``     src/observables/angular.jl:260-359 (grids, k-interpolation, LOS, C_l,
                         ℓ-spline), ``source_grid`` src/observables/fourier.jl:267-291
  * grids               src/utils.jl:269-292
  * Chebyshev k-interp  src/observables/fourier.jl:419-459,524-535
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

PLANCK18 = dict(h=0.6736, Omega_c=0.1200 / 0.6736**2, Omega_b=0.0224 / 0.6736**2, T0=2.7255,
                Neff=2.99, YHe=0.2454, ln_As1e10=float(np.log(2.099e-9 * 1e10)), ns=0.965,
                m_nu_eV=0.02, N_nu=3.0)
"""parameters_Planck18 (src/parameters.jl:1-21) for the reference's ΛCDM with massive ν."""


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "Omega_c", "Omega_b", "T0", "Neff", "YHe", "ln_As1e10", "ns", "m_nu_eV", "N_nu")]


class Model(C.Structure):
    _fields_ = [(n, C.c_int) for n in
                ("lmax_g", "lmax_nu", "lmax_h", "nx", "Hswitch", "Heswitch", "reionization")]


class Opts(C.Structure):
    _fields_ = [("bg_rtol", C.c_double), ("bg_atol", C.c_double), ("pt_rtol", C.c_double),
                ("pt_atol", C.c_double), ("tau_ini", C.c_double), ("tau_max", C.c_double),
                ("maxiters", C.c_long), ("nthreads", C.c_int), ("alg_bg", C.c_int), ("alg_pt", C.c_int),
                ("pt_linsolve", C.c_int)]


RODAS4, RODAS5P = 0, 1
_ALGS = {"rodas4": RODAS4, "rodas5p": RODAS5P}


_lib = None


def build():
    """Compile the oracle with its Makefile (portable flags, no reference sources)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp, ip, lp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_long)
        L.orc_momentum_quadrature.argtypes = [C.c_int, dp, dp]
        L.orc_bg_solve.restype = C.c_void_p
        L.orc_bg_solve.argtypes = [C.POINTER(Params), C.POINTER(Model), C.POINTER(Opts), ip]
        L.orc_bg_free.argtypes = [C.c_void_p]
        L.orc_bg_info.argtypes = [C.c_void_p, dp]
        L.orc_bg_nknots.argtypes = [C.c_void_p]
        L.orc_bg_knots.argtypes = [C.c_void_p, dp, dp]
        L.orc_bg_eval.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.orc_pt_nstate.argtypes = [C.POINTER(Model)]
        L.orc_pt_solve.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_int, dp, C.c_int, dp, ip, lp]
        L.orc_pt_rhs.argtypes = [C.c_void_p, C.c_double, C.c_double, dp, dp, dp, dp]
        L.orc_pt_initial.argtypes = [C.c_void_p, C.c_double, C.c_double, dp, dp]
        L.orc_sph_bessel.argtypes = [C.c_int, ip, C.c_int, dp, dp]
        L.orc_jl_create.restype = C.c_void_p
        L.orc_jl_create.argtypes = [C.c_int, ip, C.c_double, C.c_double, C.c_int]
        L.orc_jl_free.argtypes = [C.c_void_p]
        L.orc_jl_nx.argtypes = [C.c_void_p]
        L.orc_jl_xmax.restype = C.c_double
        L.orc_jl_xmax.argtypes = [C.c_void_p]
        L.orc_jl_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp]
        L.orc_los_integrate.argtypes = [C.c_void_p, C.c_int, dp, C.c_int, dp, C.c_int, dp, C.c_int, dp]
        L.orc_cl_integrate.argtypes = [C.c_int, dp, dp, C.c_int, dp, dp, dp]
        L.orc_cubic_spline.argtypes = [C.c_int, dp, dp, C.c_int, dp, dp]
        L.orc_cubic_spline_columns.argtypes = [C.c_int, dp, C.c_int, dp, C.c_int, dp, dp]
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def set_threads(n):
    os.environ["OMP_NUM_THREADS"] = str(n)


def momentum_quadrature(N):
    x = np.zeros(N); W = np.zeros(N)
    _, xp = _d(x); _, Wp = _d(W)
    lib().orc_momentum_quadrature(N, xp, Wp)
    return x, W


# -------------------------------------------------------------------------------------------
# grids (src/utils.jl:269-292)
def lingrid(a, b, *, step=None, length=None):
    if step is not None:
        length = int(np.ceil((b - a) / step)) + 1
    return np.linspace(a, b, length)


def cosgrid(a, b, *, length):
    return a + (b - a) * (1 - np.cos(np.pi * lingrid(0.0, 0.5, length=length)))


def loggrid(a, b, *, length):
    x = np.exp(lingrid(np.log(a), np.log(b), length=length))
    x[0], x[-1] = a, b
    return x


class ChebyshevInterpolator:
    """Chebyshev-point k-grid with barycentric interpolation in y = f(k)
    (src/observables/fourier.jl:419-459,524-535)."""

    def __init__(self, xmin, xmax, order, f=None, finv=None):
        f = f or (lambda x: x)
        finv = finv or (lambda y: y)
        ymin, ymax = f(xmin), f(xmax)
        j = np.arange(order + 1)
        ys = 0.5 * (ymin + ymax) + 0.5 * (ymax - ymin) * np.cos(np.pi * j / order)  # descending
        xs = finv(ys)
        xs[-1], xs[0] = xmin, xmax
        ws = np.where(j % 2 == 0, 1.0, -1.0)
        ws[0] /= 2
        ws[-1] /= 2
        self.xs, self.ys, self.ws, self.f = xs, ys, ws, f

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


def fk_tanh(k, k0=2000.0):
    return np.tanh(k / k0)


def fkinv_tanh(y, k0=2000.0):
    return k0 * np.arctanh(y)


# -------------------------------------------------------------------------------------------
class Background:
    """Background + thermodynamics solution of one cosmology (src/solve.jl:427-435)."""

    def __init__(self, params: dict, model: dict, *, bg_rtol=1e-7, bg_atol=1e-7, pt_rtol=1e-5,
                 pt_atol=1e-5, tau_ini=1e-6, tau_max=100.0, maxiters=100000, alg="rodas5p", bg_alg="rodas4",
                 linsolve="dense"):
        """linsolve: "dense" (LU with partial pivoting, the checker) or "sparse" (the reference's
        sparse-LU path restated, used as the timed CPU baseline)."""
        self.params, self.model = dict(params), dict(model)
        self.p = Params(**params)
        self.m = Model(**model)
        self.o = Opts(bg_rtol, bg_atol, pt_rtol, pt_atol, tau_ini, tau_max, maxiters, 0, _ALGS[bg_alg], _ALGS[alg],
                      {"dense": 0, "sparse": 1}[linsolve])
        st = C.c_int(0)
        self.h = lib().orc_bg_solve(C.byref(self.p), C.byref(self.m), C.byref(self.o), C.byref(st))
        self.status = st.value
        info = np.zeros(13)
        lib().orc_bg_info(self.h, _d(info)[1])
        (self.tau0, self.kappa0, self.taurec, self.Og0, self.On0, self.Oh0, self.OL0, nk, self.fHe,
         self.As, self.kpivot, self.y0, self.Irho0) = info
        n = lib().orc_bg_nknots(self.h)
        self.t = np.zeros(n); self.y = np.zeros((n, 5))
        lib().orc_bg_knots(self.h, _d(self.t)[1], self.y.ctypes.data_as(C.POINTER(C.c_double)))
        self.nstate = lib().orc_pt_nstate(C.byref(self.m))

    def __del__(self):
        try:
            lib().orc_bg_free(self.h)
        except Exception:
            pass

    def eval(self, taus):
        """a, ℋ, κ̇, κ, v, v̇, cs², Xe, Tb, XHe⁺⁺ at taus."""
        taus, tp = _d(np.atleast_1d(taus))
        out = np.zeros((len(taus), 10))
        lib().orc_bg_eval(self.h, len(taus), tp, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def primordial(self, k):
        k = np.asarray(k, dtype=np.float64)
        return 2 * np.pi**2 * self.As / k**3 * (k / self.kpivot) ** (self.params["ns"] - 1)

    def solve_pt(self, ks, tau_ini, taus=None, mode=0):
        ks, kp = _d(ks)
        ti, tp = _d(np.broadcast_to(np.asarray(tau_ini, dtype=np.float64), ks.shape))
        taus = np.zeros(0) if taus is None else np.asarray(taus, dtype=np.float64)
        taus, tsp = _d(taus)
        nk, nt = len(ks), len(taus)
        if mode == 0:
            out = np.zeros((nk, nt, 3))
        elif mode == 1:
            out = np.zeros(nk)
        else:
            out = np.zeros((nk, nt, self.nstate))
        status = np.zeros(nk, dtype=np.int32)
        stats = np.zeros((nk, 2), dtype=np.int64)
        lib().orc_pt_solve(self.h, nk, kp, tp, nt, tsp, mode, out.ctypes.data_as(C.POINTER(C.c_double)),
                           status.ctypes.data_as(C.POINTER(C.c_int)), stats.ctypes.data_as(C.POINTER(C.c_long)))
        return out, status, stats

    def rhs(self, k, tau, y, jac=False):
        y, yp = _d(y)
        n = self.nstate
        f = np.zeros(n)
        if not jac:
            lib().orc_pt_rhs(self.h, float(k), float(tau), yp, _d(f)[1], None, None)
            return f
        J = np.zeros((n, n)); ft = np.zeros(n)
        lib().orc_pt_rhs(self.h, float(k), float(tau), yp, _d(f)[1], J.ctypes.data_as(C.POINTER(C.c_double)), _d(ft)[1])
        return f, J, ft

    def initial(self, k, tau):
        y = np.zeros(self.nstate); extra = np.zeros(3)
        lib().orc_pt_initial(self.h, float(k), float(tau), _d(y)[1], _d(extra)[1])
        return y, extra


class BesselCache:
    """SphericalBesselCache (src/observables/angular.jl:18-26)."""

    def __init__(self, ls, xmax=None, dx=2 * np.pi / 15, hermite=True):
        ls = np.asarray(ls, dtype=np.int32)
        self.l = ls
        xmax = 20.0 * ls[-1] if xmax is None else xmax
        self.h = lib().orc_jl_create(len(ls), _i(ls)[1], float(xmax), float(dx), int(hermite))
        self.xmax = lib().orc_jl_xmax(self.h)

    def __del__(self):
        try:
            lib().orc_jl_free(self.h)
        except Exception:
            pass

    def __call__(self, il, x):
        x, xp = _d(np.atleast_1d(x))
        out = np.zeros(len(x))
        lib().orc_jl_eval(self.h, int(il), len(x), xp, _d(out)[1])
        return out


def sph_bessel(ls, x):
    ls, lp = _i(np.atleast_1d(ls))
    x, xp = _d(np.atleast_1d(x))
    out = np.zeros((len(x), len(ls)))
    lib().orc_sph_bessel(len(ls), lp, len(x), xp, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def los_integrate(S, taus, ks, jl: BesselCache, l_limber=2**31 - 1):
    """S[it, ik, s] -> I[ik, il, s]."""
    S = np.ascontiguousarray(S, dtype=np.float64)
    nt, nk, ns = S.shape
    out = np.zeros((nk, len(jl.l), ns))
    lib().orc_los_integrate(jl.h, ns, S.ctypes.data_as(C.POINTER(C.c_double)), nt, _d(taus)[1], nk,
                            _d(ks)[1], int(min(l_limber, 2**31 - 1)), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def cl_integrate(ks, P0, ThA, ThB):
    ks, kp = _d(ks); P0, pp = _d(P0)
    ThA, ap = _d(ThA); ThB, bp = _d(ThB)
    nk, nl = ThA.shape
    Cl = np.zeros(nl)
    lib().orc_cl_integrate(nk, kp, pp, nl, ap, bp, _d(Cl)[1])
    return Cl


def cubic_spline_columns(x, Y, xq):
    """Natural cubic splines through (x, Y[:, c]) for every column c, evaluated at xq -> [len(xq), m]."""
    x, xp = _d(x); xq, qp = _d(xq)
    Y = np.ascontiguousarray(Y, dtype=np.float64).reshape(len(x), -1)
    out = np.zeros((len(xq), Y.shape[1]))
    lib().orc_cubic_spline_columns(len(x), xp, Y.shape[1], Y.ctypes.data_as(C.POINTER(C.c_double)), len(xq), qp,
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def cubic_spline(x, y, xq):
    x, xp = _d(x); y, yp = _d(y); xq, qp = _d(xq)
    out = np.zeros(len(xq))
    lib().orc_cubic_spline(len(x), xp, yp, len(xq), qp, _d(out)[1])
    return out


# -------------------------------------------------------------------------------------------
def spectrum_matter(bg: Background, ks, kτini=1e-2, τinimax=1e-4):
    """Linear P(k) at τ0 (src/observables/fourier.jl:79-101)."""
    ks = np.asarray(ks, dtype=np.float64)
    ti = np.minimum(kτini / ks, τinimax)
    dm, status, stats = bg.solve_pt(ks, ti, mode=1)
    return bg.primordial(ks) * dm**2, status, stats


def spectrum_cmb(bg: Background, modes, jl: BesselCache, ls_out=None, *, kinterp=None, dkt0=np.pi,
                 xs=None, taucut=1e-2, l_limber=10, normalization="Dl", return_parts=False, taus=None):
    """Angular spectra C_l/D_l for modes like ['TT','EE','ψψ'] (src/observables/angular.jl:260-359)."""
    modes = list(modes)
    joined = "".join(modes)
    iT = 1 if "T" in joined else 0
    iE = iT + 1 if "E" in joined else 0
    iP = max(iE, iT) + 1 if "ψ" in joined else 0
    if kinterp is None:
        kinterp = (ChebyshevInterpolator(1e-2, 1e4, 130, fk_tanh, fkinv_tanh) if iP
                   else ChebyshevInterpolator(1e-2, 2e3, 60))
    ls = jl.l.astype(np.float64)
    tau0 = bg.tau0
    kmin, kmax = kinterp.xs[-1], kinterp.xs[0]
    ks_fine = lingrid(kmin, kmax, step=dkt0 / tau0)
    if taus is None:
        taus = bg.t[bg.t >= taucut]
        xs = cosgrid(0.0, 1.0, length=300) if xs is None else np.asarray(xs)
        taus = taus[0] + (taus[-1] - taus[0]) * xs
    taus = np.asarray(taus, dtype=np.float64)
    # coarse solve (ptivini = -Inf -> background start) and k-interpolation
    Sc, status, stats = bg.solve_pt(kinterp.xs, bg.t[0], taus, mode=0)  # [ik, it, 3]
    M = kinterp.matrix(ks_fine)  # [nfine, ncoarse]
    sel = [s for s, i in ((0, iT), (1, iE), (2, iP)) if i > 0]
    Sf = np.einsum("fc,cts->tfs", M, Sc[:, :, sel])
    Sf[-1] = 0.0
    Th = los_integrate(Sf, taus, ks_fine, jl)  # [ik, il, s]
    pos = {}
    col = 0
    for name, i in (("T", iT), ("E", iE), ("ψ", iP)):
        if i > 0:
            pos[name] = col
            col += 1
    if iT:
        Th[:, :, pos["T"]] /= ks_fine[:, None]
    if iE:
        Th[:, :, pos["E"]] *= (np.sqrt((ls + 2) * (ls + 1) * ls * (ls - 1)))[None, :] / ks_fine[:, None] ** 2
    if iP and l_limber <= ls[-1]:
        Th[:, :, pos["ψ"]] = los_integrate(Sf[:, :, pos["ψ"]:pos["ψ"] + 1], taus, ks_fine, jl, l_limber)[:, :, 0]
    P0 = bg.primordial(ks_fine)
    out = np.zeros((len(ls), len(modes)))
    for im, mode in enumerate(modes):
        A, B = pos[mode[0]], pos[mode[-1]]
        Cl = cl_integrate(ks_fine, P0, Th[:, :, A], Th[:, :, B])
        out[:, im] = Cl * ls * (ls + 1) / (2 * np.pi) if normalization == "Dl" else Cl
    if ls_out is not None:
        ls_out = np.asarray(ls_out, dtype=np.float64)
        out = np.stack([cubic_spline(ls, out[:, i], ls_out) for i in range(len(modes))], axis=1)
    if return_parts:
        return out, dict(status=status, stats=stats, taus=taus, ks_fine=ks_fine, Sc=Sc, Th=Th)
    return out


def spectrum_cmb_kspline(bg: Background, ks, taus, jl: BesselCache, ls_out, modes=("TT", "TE", "EE"), dkt0=np.pi,
                         return_parts=False, sources=None):
    """spectrum_cmb (src/observables/angular.jl:260-341) with the sources solved at ks and interpolated
    to the fine grid lingrid(ks[0], ks[-1], step=Δkτ0/τ0) by natural cubic splines in log k, on the
    given τ grid (the last time's sources set to zero), T and E only; D_l at ls_out (l-spline).
    sources: coarse sources [k][tau][3] to use instead of solving."""
    ks = np.asarray(ks, dtype=np.float64)
    taus = np.asarray(taus, dtype=np.float64)
    if sources is None:
        Sc, status, stats = bg.solve_pt(ks, bg.t[0], taus, mode=0)  # [k][tau][3]
    else:
        Sc, status, stats = np.asarray(sources, dtype=np.float64), np.zeros(len(ks), dtype=np.int32), None
    kf = lingrid(ks[0], ks[-1], step=dkt0 / bg.tau0)
    Sf = cubic_spline_columns(np.log(ks), Sc[:, :, :2].reshape(len(ks), -1), np.log(kf)).reshape(len(kf), len(taus), 2)
    Sf = np.ascontiguousarray(Sf.transpose(1, 0, 2))
    Sf[-1] = 0.0
    Th = los_integrate(Sf, taus, kf, jl)
    ls = jl.l.astype(np.float64)
    Th[:, :, 0] /= kf[:, None]
    Th[:, :, 1] *= np.sqrt((ls + 2) * (ls + 1) * ls * (ls - 1))[None, :] / kf[:, None] ** 2
    P0 = bg.primordial(kf)
    pos = {"T": 0, "E": 1}
    out = []
    for mode in modes:
        Cl = cl_integrate(kf, P0, Th[:, :, pos[mode[0]]], Th[:, :, pos[mode[-1]]]) * ls * (ls + 1) / (2 * np.pi)
        out.append(cubic_spline(ls, Cl, np.asarray(ls_out, dtype=np.float64)))
    Dl = np.stack(out, axis=1)
    if return_parts:
        return Dl, dict(status=status, stats=stats, nk_fine=len(kf))
    return Dl
