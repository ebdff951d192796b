"""Learned source surrogate with solver fallback.

An MLP maps (six cosmological parameters, log k, log τ) to the smooth perturbation factors of the
line-of-sight sources (src/models/cosmologies.jl:99-104); the sources follow exactly from them and
each cosmology's visibility function.  It is trained on factors computed by the GPU perturbation
solver (output "factors") with the library's own BF16 tensor-core forward/backward kernels
(``sbz_surrogate_*``), and evaluated the same way.
Its sources go through the regular k-interpolation → line-of-sight → C_ℓ pipeline
(``sbz_spectrum_cmb_sources``).  Each cosmology gets an error estimate in the C_ℓ metric, from the
disagreement of two networks trained from different initialisations (no mode solved), or from 48
probe modes solved with the real solver; a cosmology whose estimate exceeds the tolerance is
recomputed by the solver (all flagged cosmologies' modes in one launch), which therefore remains
the reference for every result.
"""
import ctypes as C

import numpy as np

from . import _lib as L

# parameter box: h, ω_c, ω_b, n_s, ln(1e10 A_s), Σm_ν [eV] (one massive species of that mass)
BOX = np.array([[0.6, 0.8], [0.10, 0.14], [0.020, 0.024], [0.92, 1.0], [2.9, 3.2], [0.06, 0.3]])
NAMES = ("h", "omega_c", "omega_b", "ns", "ln_As1e10", "m_nu")
LOGTAU = (np.log(1e-2), np.log(4.0))  # τ in 1/H0


def box_params(theta):
    """Parameter dict of the library for θ = (h, ω_c, ω_b, n_s, ln 1e10 A_s, Σm_ν)."""
    h, oc, ob, ns, las, mnu = (float(v) for v in theta)
    return dict(h=h, Omega_c=oc / h**2, Omega_b=ob / h**2, T0=2.7255, Neff=2.0328, YHe=0.245, ln_As1e10=las, ns=ns, m_nu_eV=mnu,
                N_nu=1.0)


def sample_box(n, seed=0, sobol=False):
    """n points of the box: uniform (PCG64) or scrambled Sobol."""
    if sobol:
        from scipy.stats import qmc
        u = qmc.Sobol(6, scramble=True, seed=seed).random(n)
    else:
        u = np.random.default_rng(seed).random((n, 6))
    return BOX[:, 0] + u * (BOX[:, 1] - BOX[:, 0])


def needs_solver(errs, tol):
    """Fallback mask: a cosmology keeps the surrogate's result only if its error estimate is a
    number at or below tol; NaN or infinite estimates (a network that produced non-finite sources)
    go to the solver like any estimate above tol."""
    return ~(np.asarray(errs, dtype=np.float64) <= tol)


def write_training_set(path, X, Y):
    """Append rows (X [n, nin], Y [n, nout], float32) to the flat SBZTRN01 training-set file at path,
    creating it if needed (sbz_trainset_append)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.ascontiguousarray(Y, dtype=np.float32)
    if X.ndim != 2 or Y.ndim != 2 or len(X) != len(Y):
        raise ValueError("X and Y must be 2-d with one row per sample")
    fp = C.POINTER(C.c_float)
    L.check(L.lib().sbz_trainset_append(str(path).encode(), X.shape[1], Y.shape[1], len(X), X.ctypes.data_as(fp),
                                        Y.ctypes.data_as(fp)), "write_training_set")


def training_set_info(path):
    """(nin, nout, nrows) of a training-set file."""
    a, b, n = C.c_int(), C.c_int(), C.c_longlong()
    L.check(L.lib().sbz_trainset_info(str(path).encode(), C.byref(a), C.byref(b), C.byref(n)), "training_set_info")
    return a.value, b.value, n.value


def read_training_set(path, first=0, n=None):
    """Rows [first, first + n) of a training-set file as (X, Y) float32 arrays (all rows by default)."""
    nin, nout, rows = training_set_info(path)
    n = rows - first if n is None else n
    X = np.empty((n, nin), dtype=np.float32)
    Y = np.empty((n, nout), dtype=np.float32)
    fp = C.POINTER(C.c_float)
    L.check(L.lib().sbz_trainset_read(str(path).encode(), first, n, X.ctypes.data_as(fp), Y.ctypes.data_as(fp)),
            "read_training_set")
    return X, Y


class MLP:
    """The device MLP (nin → nhidden × width SiLU → nout) of ``sbz_surrogate_*``."""

    def __init__(self, nin=8, width=512, nhidden=4, nout=4, batch=65536, seed=0, _handle=None):
        self.nin, self.width, self.nhidden, self.nout, self.batch = nin, width, nhidden, nout, batch
        if _handle is None:
            h = C.c_void_p()
            L.check(L.lib().sbz_surrogate_create(nin, width, nhidden, nout, batch, seed, C.byref(h)), "sbz_surrogate_create")
            _handle = h
        self._h = _handle

    @classmethod
    def load(cls, path, batch=65536):
        h = C.c_void_p()
        L.check(L.lib().sbz_surrogate_load(str(path).encode(), batch, C.byref(h)), "sbz_surrogate_load")
        hdr = np.fromfile(path, dtype=np.int32, count=6)[2:]
        return cls(int(hdr[0]), int(hdr[1]), int(hdr[2]), int(hdr[3]), batch, _handle=h)

    def __del__(self):
        if getattr(self, "_h", None):
            L.lib().sbz_surrogate_destroy(self._h)
            self._h = None

    @property
    def nparams(self):
        return int(L.lib().sbz_surrogate_nparams(self._h))

    def get_params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        L.check(L.lib().sbz_surrogate_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        L.check(L.lib().sbz_surrogate_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))), "set_params")

    def set_data(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        fp = C.POINTER(C.c_float)
        L.check(L.lib().sbz_surrogate_set_data(self._h, len(X), X.ctypes.data_as(fp), Y.ctypes.data_as(fp)), "set_data")

    def train(self, nsteps, lr):
        loss = C.c_double()
        L.check(L.lib().sbz_surrogate_train(self._h, int(nsteps), float(lr), C.byref(loss)), "train")
        return loss.value

    def gradients(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double()
        fp = C.POINTER(C.c_float)
        L.check(L.lib().sbz_surrogate_gradients(self._h, len(X), X.ctypes.data_as(fp), Y.ctypes.data_as(fp), C.byref(loss),
                                                g.ctypes.data_as(fp)), "gradients")
        return loss.value, g

    def infer(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((len(X), self.nout), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        L.check(L.lib().sbz_surrogate_infer(self._h, len(X), X.ctypes.data_as(fp), Y.ctypes.data_as(fp)), "infer")
        return Y

    def save(self, path):
        L.check(L.lib().sbz_surrogate_save(self._h, str(path).encode()), "save")


def cmb_taus(bg_t, tau0, ntau):
    """Line-of-sight time grid of a cosmology: first background knot ≥ 1e-2 to τ0 on the reference's
    cosine grid (src/observables/angular.jl:280-290)."""
    from . import cosgrid
    t = bg_t[bg_t >= 1e-2]
    return t[0] + (tau0 - t[0]) * cosgrid(0.0, 1.0, length=ntau)


class SourceSurrogate:
    """Line-of-sight sources on a fixed coarse k grid and per-cosmology τ grids, from an MLP of the
    seven perturbation factors the sources are built from (f0 = δγ/4 + Ψ + Π/16, f1 = Ψ' + Φ',
    f2 = θb, f3 = θb', f4 = Π, f5 = Π', f6 = Π''; solver output "factors").  The sharp recombination
    structure lives in the visibility v and its derivatives, which come exactly from each cosmology's
    background; the network learns the smooth factors, scaled by powers of k and, except the ISW
    factor, tapered by the normalised visibility envelope (so the loss ignores times the sources never
    see).  Sources: k S_T = k [v f0 + e^{-κ} f1 + (v̇ f2 + v f3)/k² + 3 (v̈ f4 + 2 v̇ f5 + v f6)/(16 k²)],
    k² S_E = 3 v f4 / (16 χ²)  (src/models/cosmologies.jl:99-104)."""

    KPOW = np.array([0, 0, 1, 2, 0, 1, 2])  # factors are learned as f_j / k^KPOW[j]
    NIN = 10  # inputs: θ (6), log k, log τ, sin and cos of the acoustic phase k r_s(τ)

    @property
    def net(self):
        return self.nets[0]

    def __init__(self, M, ks, ntau=500, width=512, nhidden=4, batch=65536, seed=0, members=2, pt_rtol=1e-5, pt_atol=1e-5):
        """members: networks trained from different initialisations on the same data; the sources are
        their mean and their disagreement is the per-cosmology error estimate.  pt_rtol, pt_atol: the
        solver tolerances of the training data and of the fallback."""
        self.M, self.ks, self.ntau = M, np.asarray(ks, dtype=np.float64), ntau
        self.logk = (np.log(self.ks.min()), np.log(self.ks.max()))
        self.nets = [MLP(self.NIN, width, nhidden, 7, batch, seed + 7919 * i) for i in range(max(1, members))]
        self.pt_rtol, self.pt_atol = pt_rtol, pt_atol
        self.mean = np.zeros(7)
        self.scale = np.ones(7)
        self.env_lk = np.array([-1.0, 1.0])  # k envelope: log k feature nodes and log RMS per factor
        self.env_la = np.zeros((2, 7))

    # ---- features, background, targets ------------------------------------------------------
    def features(self, theta, taus, vis, ks=None):
        """[nk * ntau, NIN] inputs for one cosmology: θ mapped to [-1, 1] by the box, log k and log τ to
        [-1, 1], and the sine and cosine of the acoustic phase k r_s(τ) (r_s, the photon-baryon sound
        horizon, is row 4 of vis), so the network does not have to build the acoustic oscillations
        of the sources in k out of smooth functions; row i*ntau + j is (k_i, τ_j)."""
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        th = 2 * (np.asarray(theta) - BOX[:, 0]) / (BOX[:, 1] - BOX[:, 0]) - 1
        lk = 2 * (np.log(ks) - self.logk[0]) / (self.logk[1] - self.logk[0]) - 1
        lt = 2 * (np.log(taus) - LOGTAU[0]) / (LOGTAU[1] - LOGTAU[0]) - 1
        nk, nt = len(ks), len(taus)
        X = np.empty((nk * nt, self.NIN), dtype=np.float32)
        X[:, :6] = th
        X[:, 6] = np.repeat(lk, nt)
        X[:, 7] = np.tile(lt, nk)
        ph = np.outer(ks, vis[4]).ravel()
        X[:, 8] = np.sin(ph)
        X[:, 9] = np.cos(ph)
        return X

    @staticmethod
    def sound_horizon(bg, c, theta, taus):
        """Photon-baryon sound horizon r_s(τ) = ∫ dτ' / sqrt(3 (1 + R)), R = 3 ω_b a / (4 ω_γ) (T0 =
        2.7255 K, ω_γ = 2.4728e-5), from the background's a(τ) on 2048 log-spaced times (trapezoid;
        r_s = τ/√3 before the first), at taus.  An input feature, so approximate is enough."""
        p = box_params(theta)
        wb = p["Omega_b"] * p["h"] ** 2
        t = bg.t(c)
        tf = np.geomspace(max(float(t[t > 0][0]), 1e-6), float(bg.tau0[c]), 2048)
        a = bg.coefficients(tf, c)[:, 0]
        cs = 1.0 / np.sqrt(3.0 * (1.0 + 0.75 * wb / 2.4728e-5 * a))
        rs = tf[0] / np.sqrt(3.0) + np.concatenate([[0.0], np.cumsum(0.5 * (cs[1:] + cs[:-1]) * np.diff(tf))])
        return np.interp(taus, tf, rs)

    def background_rows(self, bg, c, theta, taus):
        """v, v̇, v̈, e^{-κ} and r_s on taus: the rows of vis."""
        return np.vstack([self.visibility(bg.coefficients(taus, c)), self.sound_horizon(bg, c, theta, taus)[None]])

    @staticmethod
    def visibility(coef):
        """v, v̇, v̈, e^{-κ} from the GPU coefficient columns (a, ℋ, κ̇, c_s², e^{-κ}, κ̈, κ⃛), the
        same expressions the perturbation kernel evaluates."""
        kd, ek, kdd, kddd = coef[:, 2], coef[:, 4], coef[:, 5], coef[:, 6]
        v = -kd * ek
        vd = (kd * kd - kdd) * ek
        vdd = (-kd * kd * kd + 3 * kd * kdd - kddd) * ek
        return np.stack([v, vd, vdd, ek])

    @staticmethod
    def taper(vis):
        """Normalised visibility envelope (|v| + a|v̇| + b|v̈|)/max ∈ [0, 1]: zero where no source
        term sees the visibility-carried factors (before recombination), so their stiff early-time
        transients do not enter the loss."""
        v, vd, vdd = np.abs(vis[0]), np.abs(vis[1]), np.abs(vis[2])
        d1 = v.max() / max(vd.max(), 1e-300)
        d2 = v.max() / max(vdd.max(), 1e-300)
        t = v + d1 * vd + d2 * vdd
        return t / t.max()

    def solve_factors(self, thetas, precision="mixed", ks=None):
        """Solver factors [ncos][nk][ntau][7] on (ks or the coarse grid) × each cosmology's τ grid,
        with taus [ncos][ntau], background rows [ncos][5][ntau] (v, v̇, v̈, e^{-κ}, r_s) and the problem."""
        from . import CosmologyProblem, solvept
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        prob = CosmologyProblem(self.M, [box_params(t) for t in thetas], precision=precision, pt_rtol=self.pt_rtol,
                                pt_atol=self.pt_atol)
        bg = prob.solvebg()
        if np.any(bg.status != 0):
            raise L.SbzError("background failed for a cosmology of the box")
        taus = np.stack([cmb_taus(bg.t(c), bg.tau0[c], self.ntau) for c in range(len(thetas))])
        nk = len(ks)
        cos = np.repeat(np.arange(len(thetas)), nk)
        out, st, _ = solvept(prob, np.tile(ks, len(thetas)), prob.opts.tau_ini, saveat=taus, output="factors", cosmo=cos)
        if np.any(st != 0):
            raise L.SbzError(f"{int(np.count_nonzero(st))} modes failed")
        vis = np.stack([self.background_rows(bg, c, thetas[c], taus[c]) for c in range(len(thetas))])
        return out.reshape(len(thetas), nk, self.ntau, 7), taus, vis, prob

    def backgrounds(self, thetas):
        """Times [ncos][ntau], background rows [ncos][5][ntau] (v, v̇, v̈, e^{-κ}, r_s) and the problem of the given parameter
        points from their backgrounds alone (no perturbation modes solved)."""
        from . import CosmologyProblem
        prob = CosmologyProblem(self.M, [box_params(t) for t in thetas], pt_rtol=self.pt_rtol, pt_atol=self.pt_atol)
        bg = prob.solvebg()
        if np.any(bg.status != 0):
            raise L.SbzError("background failed for a cosmology of the box")
        taus = np.stack([cmb_taus(bg.t(c), bg.tau0[c], self.ntau) for c in range(len(thetas))])
        vis = np.stack([self.background_rows(bg, c, thetas[c], taus[c]) for c in range(len(thetas))])
        return taus, vis, prob

    def weights(self, vis):
        """Per-time multipliers of the learned factors: the visibility envelope for f0, f2..f6 and
        e^{-κ} for the ISW factor f1."""
        w = np.repeat(self.taper(vis)[:, None], 7, axis=1)
        w[:, 1] = vis[3]
        return w

    def to_targets(self, F, ks, vis):
        with np.errstate(over="ignore", invalid="ignore"):
            G = F / ks[:, None, None] ** self.KPOW * self.weights(vis)[None]
        return np.where(self.weights(vis)[None] > 0, G, 0.0)

    def from_targets(self, G, ks, vis):
        w = self.weights(vis)[None]
        F = np.where(w > 1e-12, G / np.where(w > 1e-12, w, 1.0), 0.0)  # sources there carry v ≈ 0 or e^{-κ} ≈ 0
        return F * ks[:, None, None] ** self.KPOW

    @staticmethod
    def sources(F, ks, taus, vis):
        """(k S_T, k² S_E, S_ψ = 0) [nk][ntau][3] from factors; zero at χ = 0 (angular.jl:296)."""
        v, vd, vdd, ek = (x[None, :] for x in vis[:4])
        k = ks[:, None]
        f = [F[..., j] for j in range(7)]
        sT = v * f[0] + ek * f[1] + (vd * f[2] + v * f[3]) / k**2 + 3.0 / (16.0 * k**2) * (vdd * f[4] + 2 * vd * f[5] + v * f[6])
        chi2 = (taus[-1] - taus)[None, :] ** 2
        out = np.zeros(F.shape[:2] + (3,))
        out[..., 0] = k * sT
        out[..., 1] = np.where(chi2 > 0, 3.0 / 16.0 * v * f[4] / np.where(chi2 > 0, chi2, 1.0), 0.0)
        out[:, -1, :] = 0.0
        return out

    def dataset(self, thetas):
        """(X, Y, taus) training arrays from the solver for the given parameter points."""
        F, taus, vis, _ = self.solve_factors(thetas)
        X = np.concatenate([self.features(t, taus[c], vis[c]) for c, t in enumerate(thetas)])
        Y = np.concatenate([self.to_targets(F[c], self.ks, vis[c]).reshape(-1, 7) for c in range(len(thetas))])
        return X, Y, taus

    # ---- training ---------------------------------------------------------------------------
    def envelope(self, lk):
        """RMS amplitude of each target at the log-k features lk [n, 7] (log-linear between the
        training grid's k), so the network learns every k to the same relative accuracy: the
        Silk-damped high-k factors are orders of magnitude below the low-k ones."""
        return np.exp(np.stack([np.interp(lk, self.env_lk, self.env_la[:, j]) for j in range(7)], axis=1))

    def normalise(self, X, Y):
        return (Y / self.envelope(X[:, 6]) - self.mean) / self.scale

    def fit(self, X, Y, steps, lr=1e-3, lr_final=1e-5, chunks=20):
        """Divide the targets by their k envelope, standardise, and train `steps` Adam steps with an
        exponential learning-rate decay from lr to lr_final; returns the loss after each chunk."""
        lk, inv = np.unique(X[:, 6].astype(np.float64), return_inverse=True)
        cnt = np.bincount(inv, minlength=len(lk)).astype(np.float64)
        ms = np.stack([np.bincount(inv, weights=Y[:, j].astype(np.float64) ** 2, minlength=len(lk)) for j in range(7)], axis=1) / cnt[:, None]
        rms = np.sqrt(ms)
        rms = np.maximum(rms, 1e-12 * rms.max(axis=0, keepdims=True) + 1e-300)
        self.env_lk, self.env_la = lk, np.log(rms)
        Z = Y / self.envelope(X[:, 6])
        self.mean = Z.mean(axis=0)
        self.scale = Z.std(axis=0) + 1e-30
        Zn = ((Z - self.mean) / self.scale).astype(np.float32)
        losses = []
        for net in self.nets:
            net.set_data(X, Zn)
            per = max(1, steps // chunks)
            done = 0
            lm = []
            while done < steps:
                n = min(per, steps - done)
                rate = lr * (lr_final / lr) ** (done / max(1, steps))
                lm.append(net.train(n, rate))
                done += n
            losses.append(lm)
        return losses[0] if len(losses) == 1 else losses

    def mse(self, X, Y):
        """Mean squared error of the members' mean on (X, Y) in standardised units (all rows)."""
        P = np.mean([net.infer(X).astype(np.float64) for net in self.nets], axis=0)
        return float(np.mean((P - self.normalise(X, Y)) ** 2))

    # ---- prediction ------------------------------------------------------------------------
    def predict_factors(self, theta, taus, vis, ks=None, member=None):
        """Factors from one member's network, or from the members' mean (member None)."""
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        X = self.features(theta, taus, vis, ks)
        nets = self.nets if member is None else [self.nets[member]]
        Z = np.mean([net.infer(X).astype(np.float64) for net in nets], axis=0)
        G = ((Z * self.scale + self.mean) * self.envelope(X[:, 6])).reshape(len(ks), len(taus), 7)
        return self.from_targets(G, ks, vis)

    def predict_sources(self, theta, taus, vis, ks=None, member=None):
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        return self.sources(self.predict_factors(theta, taus, vis, ks, member), ks, taus, vis)

    def save(self, path):
        """Weights of every member (path, path.1, ...) and the normalisation (path.norm.npz)."""
        for m, net in enumerate(self.nets):
            net.save(path if m == 0 else f"{path}.{m}")
        np.savez(str(path) + ".norm.npz", mean=self.mean, scale=self.scale, env_lk=self.env_lk, env_la=self.env_la, ks=self.ks,
                 ntau=self.ntau)

    @staticmethod
    def cl_error(D, ref):
        """Largest relative difference of D_ℓ [nl, 3] (TT, TE, EE) from ref over ℓ and modes, TE
        relative to sqrt(TT EE) — the metric the C_ℓ tolerance is stated in."""
        den = np.stack([np.abs(ref[:, 0]), np.sqrt(np.abs(ref[:, 0] * ref[:, 2])), np.abs(ref[:, 2])], axis=1)
        return float(np.max(np.abs(D - ref) / np.where(den > 0, den, np.inf)))

    def probe_kgrid(self, nprobe=48):
        """Probe modes: an even subset of the coarse grid, both ends included."""
        idx = np.unique(np.round(np.linspace(0, len(self.ks) - 1, nprobe)).astype(int))
        return self.ks[idx]

    def probe_error(self, theta, taus, vis, F_true, kprobe, prob, cosmo, jl, ls_out):
        """Held-out error estimate in the C_ℓ metric: D_ℓ from the surrogate's sources and from the
        solver's sources at the probe modes, both through the same line-of-sight pipeline on the
        probe grid (its coarseness is common to both and cancels in the difference)."""
        from . import CubicSplineInterpolator, spectrum_cmb
        kin = CubicSplineInterpolator(kprobe, f=np.log)
        run = lambda src: spectrum_cmb(["TT", "TE", "EE"], prob, jl, ls_out, kinterp=kin, taus=taus, cosmo=cosmo,  # noqa: E731
                                       normalization="Dl", sources=src)
        ref = run(self.sources(F_true, kprobe, taus, vis))
        return self.cl_error(run(self.predict_sources(theta, taus, vis, kprobe)), ref)

    def spectra(self, thetas, jl, ls_out, kinterp, modes=("TT", "TE", "EE"), tol=1e-3, kprobe=None, fallback=True,
                estimator="ensemble", return_timings=False):
        """C_ℓ (D_ℓ) for each θ from the surrogate's sources through the line-of-sight pipeline; the
        cosmologies whose error estimate (relative D_ℓ, the metric of tol) is above tol or not a number
        are recomputed by the solver, all of their modes in one perturbation launch.

        estimator "ensemble" (needs two members): D_ℓ of the first member's sources against D_ℓ of
        the members' mean, doubled (≈ the members' disagreement), no mode solved; "probe": D_ℓ from
        the surrogate's and the solver's sources at 48 probe modes.  fallback=False: the surrogate
        alone (no estimate, errors NaN).  Returns (Dl [ncos][nl][nmodes], error estimates, fallback
        mask) and, with return_timings, a dict of phase wall times (s)."""
        import time
        from . import solvept, spectrum_cmb
        tm = {}
        t0 = time.perf_counter()
        if fallback and estimator == "probe":
            kprobe = self.probe_kgrid() if kprobe is None else np.asarray(kprobe)
            Fp, taus, vis, prob = self.solve_factors(thetas, ks=kprobe)
        else:
            taus, vis, prob = self.backgrounds(thetas)

        def pipe(c, src):
            return spectrum_cmb(list(modes), prob, jl, ls_out, kinterp=kinterp, taus=taus[c], cosmo=c, normalization="Dl",
                                sources=src)

        tm["backgrounds"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        out, errs = [], np.full(len(thetas), np.nan)
        for c, t in enumerate(thetas):
            D = pipe(c, self.predict_sources(t, taus[c], vis[c], ks=kinterp.xs))
            if fallback and estimator == "ensemble":
                if len(self.nets) < 2:
                    raise ValueError("the ensemble estimate needs a surrogate with two or more members")
                errs[c] = 2 * self.cl_error(pipe(c, self.predict_sources(t, taus[c], vis[c], ks=kinterp.xs, member=0)), D)
            elif fallback:
                errs[c] = self.probe_error(t, taus[c], vis[c], Fp[c], kprobe, prob, c, jl, ls_out)
            out.append(D)
        tm["surrogate"] = time.perf_counter() - t0
        fb = needs_solver(errs, tol) if fallback else np.zeros(len(thetas), dtype=bool)
        t0 = time.perf_counter()
        flagged = np.flatnonzero(fb)
        if len(flagged):
            # every flagged cosmology's modes in one launch, then each through the same pipeline
            xs = np.asarray(kinterp.xs, dtype=np.float64)
            src, st, _ = solvept(prob, np.tile(xs, len(flagged)), prob.opts.tau_ini, saveat=taus, output="sources",
                                 cosmo=np.repeat(flagged, len(xs)))
            if np.any(st != 0):
                raise L.SbzError(f"{int(np.count_nonzero(st))} fallback modes failed")
            src = src.reshape(len(flagged), len(xs), taus.shape[1], 3)
            for j, c in enumerate(flagged):
                out[c] = pipe(c, src[j])
        tm["fallback"] = time.perf_counter() - t0
        res = (np.stack(out), errs, fb)
        return res + (tm,) if return_timings else res


class MatterSurrogate:
    """P(k) at z = 0 from an MLP of (θ, log k) to ln Δ_m(τ0)² (spectrum_matter's transfer factor,
    src/observables/fourier.jl:79-101; P = P0 Δ_m²), standardised; like SourceSurrogate it keeps two
    members and estimates each cosmology's error from their disagreement, and the solver (Δ_m output,
    one launch for all flagged cosmologies) is its fallback."""

    def __init__(self, M, ks, width=256, nhidden=3, batch=8192, seed=0, members=2, pt_rtol=1e-5, pt_atol=1e-5):
        self.M, self.ks = M, np.asarray(ks, dtype=np.float64)
        self.logk = (np.log(self.ks.min()), np.log(self.ks.max()))
        self.nets = [MLP(7, width, nhidden, 1, batch, seed + 104729 * i) for i in range(max(1, members))]
        self.pt_rtol, self.pt_atol = pt_rtol, pt_atol
        self.mean, self.scale = 0.0, 1.0

    def features(self, theta, ks=None):
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        X = np.empty((len(ks), 7), dtype=np.float32)
        X[:, :6] = 2 * (np.asarray(theta) - BOX[:, 0]) / (BOX[:, 1] - BOX[:, 0]) - 1
        X[:, 6] = 2 * (np.log(ks) - self.logk[0]) / (self.logk[1] - self.logk[0]) - 1
        return X

    def problem(self, thetas):
        from . import CosmologyProblem
        prob = CosmologyProblem(self.M, [box_params(t) for t in thetas], pt_rtol=self.pt_rtol, pt_atol=self.pt_atol)
        if np.any(prob.solvebg().status != 0):
            raise L.SbzError("background failed for a cosmology of the box")
        return prob

    def solve(self, thetas, prob=None, which=None):
        """Δ_m(τ0) [ncos][nk] from the solver: every mode of the cosmologies `which` (default all) in
        one launch, spectrum_matter's initial times."""
        from . import solvept
        prob = self.problem(thetas) if prob is None else prob
        which = np.arange(len(thetas)) if which is None else np.asarray(which)
        nk = len(self.ks)
        dm, st, _ = solvept(prob, np.tile(self.ks, len(which)), lambda k: np.minimum(1e-2 / k, 1e-4), output="delta_m",
                            cosmo=np.repeat(which, nk))
        if np.any(st != 0):
            raise L.SbzError(f"{int(np.count_nonzero(st))} modes failed")
        return dm.reshape(len(which), nk)

    def dataset(self, thetas):
        dm = self.solve(thetas)
        X = np.concatenate([self.features(t) for t in thetas])
        Y = np.log(dm.reshape(-1, 1) ** 2)
        return X, Y

    def fit(self, X, Y, steps, lr=1e-3, lr_final=1e-5, chunks=20):
        self.mean, self.scale = float(Y.mean()), float(Y.std()) + 1e-30
        Z = ((Y - self.mean) / self.scale).astype(np.float32)
        losses = []
        for net in self.nets:
            net.set_data(X, Z)
            per, done, lm = max(1, steps // chunks), 0, []
            while done < steps:
                n = min(per, steps - done)
                lm.append(net.train(n, lr * (lr_final / lr) ** (done / max(1, steps))))
                done += n
            losses.append(lm)
        return losses

    def transfer2(self, theta, member=None):
        """Δ_m² on the k grid from one member or the members' mean (in ln Δ_m²)."""
        X = self.features(theta)
        nets = self.nets if member is None else [self.nets[member]]
        Z = np.mean([net.infer(X).astype(np.float64)[:, 0] for net in nets], axis=0)
        return np.exp(Z * self.scale + self.mean)

    def spectra(self, thetas, tol=1e-3, fallback=True, prob=None):
        """P(k) [ncos][nk] at z = 0, surrogate or (estimate above tol or not a number) the solver;
        returns (P, error estimates, fallback mask)."""
        from . import spectrum_primordial
        prob = self.problem(thetas) if prob is None else prob
        T2 = np.stack([self.transfer2(t) for t in thetas])
        errs = np.full(len(thetas), np.nan)
        if fallback:
            if len(self.nets) < 2:
                raise ValueError("the ensemble estimate needs two or more members")
            for c, t in enumerate(thetas):
                errs[c] = 2 * float(np.max(np.abs(self.transfer2(t, member=0) / T2[c] - 1)))
        fb = needs_solver(errs, tol) if fallback else np.zeros(len(thetas), dtype=bool)
        flagged = np.flatnonzero(fb)
        if len(flagged):
            T2[flagged] = self.solve(thetas, prob=prob, which=flagged) ** 2
        P = np.stack([spectrum_primordial(self.ks, prob, c) for c in range(len(thetas))]) * T2
        return P, errs, fb
