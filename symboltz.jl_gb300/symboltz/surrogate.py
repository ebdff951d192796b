"""Learned source surrogate with solver fallback.

An MLP maps (six cosmological parameters, log k, log τ) to the four line-of-sight source terms
(k(S_SW + S_ISW), k S_Doppler, k S_polarisation, k² S_E; src/models/cosmologies.jl:99-104).  It is
trained on sources computed by the GPU perturbation solver (output "sources4") with the library's
own BF16 tensor-core forward/backward kernels (``sbz_surrogate_*``), and evaluated the same way.
Its sources go through the regular k-interpolation → line-of-sight → C_ℓ pipeline
(``sbz_spectrum_cmb_sources``).  Each cosmology gets an error estimate from a few probe modes that
are also solved with the real solver; a cosmology whose probes disagree by more than the tolerance is
recomputed with the solver (fallback), which therefore remains the judge of every result.
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
    """Sources on a fixed coarse k grid and per-cosmology τ grids, learned by an MLP.

    ks: coarse k grid (H0/c) shared by all cosmologies; ntau: times per cosmology."""

    def __init__(self, M, ks, ntau=500, width=512, nhidden=4, batch=65536, seed=0):
        self.M, self.ks, self.ntau = M, np.asarray(ks, dtype=np.float64), ntau
        self.logk = (np.log(self.ks.min()), np.log(self.ks.max()))
        self.net = MLP(8, width, nhidden, 4, batch, seed)
        self.mean = np.zeros(4)
        self.scale = np.ones(4)

    # ---- features and targets -------------------------------------------------------------
    def features(self, theta, taus):
        """[nk * ntau, 8] inputs for one cosmology: θ mapped to [-1, 1] by the box, log k and log τ to
        [-1, 1]; row i*ntau + j is (k_i, τ_j)."""
        th = 2 * (np.asarray(theta) - BOX[:, 0]) / (BOX[:, 1] - BOX[:, 0]) - 1
        lk = 2 * (np.log(self.ks) - self.logk[0]) / (self.logk[1] - self.logk[0]) - 1
        lt = 2 * (np.log(taus) - LOGTAU[0]) / (LOGTAU[1] - LOGTAU[0]) - 1
        nk, nt = len(self.ks), len(taus)
        X = np.empty((nk * nt, 8), dtype=np.float32)
        X[:, :6] = th
        X[:, 6] = np.repeat(lk, nt)
        X[:, 7] = np.tile(lt, nk)
        return X

    def solve_sources(self, thetas, precision="mixed", ks=None):
        """Solver sources4 for each θ on (ks or the coarse grid) × its own τ grid:
        returns (sources [ncos][nk][ntau][4], taus [ncos][ntau], envelopes [ncos][ntau], problem)."""
        from . import CosmologyProblem, solvept
        ks = self.ks if ks is None else np.asarray(ks, dtype=np.float64)
        prob = CosmologyProblem(self.M, [box_params(t) for t in thetas], precision=precision)
        bg = prob.solvebg()
        if np.any(bg.status != 0):
            raise L.SbzError("background failed for a cosmology of the box")
        taus = np.stack([cmb_taus(bg.t(c), bg.tau0[c], self.ntau) for c in range(len(thetas))])
        nk = len(ks)
        cos = np.repeat(np.arange(len(thetas)), nk)
        out, st, _ = solvept(prob, np.tile(ks, len(thetas)), prob.opts.tau_ini, saveat=taus, output="sources4", cosmo=cos)
        if np.any(st != 0):
            raise L.SbzError(f"{int(np.count_nonzero(st))} training modes failed")
        out = out.reshape(len(thetas), nk, self.ntau, 4)
        out[:, :, -1, :] = 0.0  # χ = 0: zeroed, as the line of sight does (src/observables/angular.jl:296)
        env = np.stack([self.envelope(bg.eval(taus[c], c)) for c in range(len(thetas))])
        return out, taus, env, prob

    @staticmethod
    def envelope(bgv):
        """|v| + e^{-κ} + 1e-3 max|v| from background columns (…, κ, v, …): the visibility and
        transparency factors the sources carry, so that sources / envelope are smooth in τ."""
        v, kappa = bgv[:, 4], bgv[:, 3]
        return np.abs(v) + np.exp(-kappa) + 1e-3 * np.max(np.abs(v))

    @staticmethod
    def _chi2(taus):
        return (taus[-1] - taus) ** 2  # χ² = (τ0 - τ)²

    def to_targets(self, S4, taus, env):
        """Learned quantities for sources4 [nk][ntau][4] on one cosmology's τ grid: the three
        temperature terms and χ² k² S_E = (3/16) v Π (removing the 1/χ² of S_E), each divided by the
        cosmology's visibility envelope (the sharp recombination peak is known exactly from the
        background; the network learns the smooth factors multiplying it)."""
        Y = S4.copy()
        Y[..., 3] *= self._chi2(taus)
        return Y / env[None, :, None]

    def from_targets(self, Y, taus, env):
        S4 = Y * env[None, :, None]
        chi2 = self._chi2(taus)
        S4[..., 3] = np.where(chi2 > 0, S4[..., 3] / np.where(chi2 > 0, chi2, 1.0), 0.0)
        S4[:, -1, :] = 0.0
        return S4

    def dataset(self, thetas):
        """(X, Y, taus) training arrays from the solver for the given parameter points."""
        S, taus, env, _ = self.solve_sources(thetas)
        X = np.concatenate([self.features(t, taus[c]) for c, t in enumerate(thetas)])
        Y = np.concatenate([self.to_targets(S[c], taus[c], env[c]).reshape(-1, 4) for c in range(len(thetas))])
        return X, Y, taus

    # ---- training ---------------------------------------------------------------------------
    def fit(self, X, Y, steps, lr=1e-3, lr_final=1e-5, chunks=20):
        """Standardise the targets and train `steps` Adam steps with an exponential learning-rate
        decay from lr to lr_final; returns the loss after each chunk."""
        self.mean = Y.mean(axis=0)
        self.scale = Y.std(axis=0) + 1e-30
        self.net.set_data(X, (Y - self.mean) / self.scale)
        losses = []
        per = max(1, steps // chunks)
        done = 0
        while done < steps:
            n = min(per, steps - done)
            rate = lr * (lr_final / lr) ** (done / max(1, steps))
            losses.append(self.net.train(n, rate))
            done += n
        return losses

    def mse(self, X, Y):
        """Mean squared error of the network on (X, Y) in standardised units (all rows)."""
        P = self.net.infer(X).astype(np.float64)
        return float(np.mean((P - (Y - self.mean) / self.scale) ** 2))

    # ---- prediction ------------------------------------------------------------------------
    def predict(self, theta, taus, env, ks=None):
        """Sources4 [nk][ntau][4] for one cosmology (physical units); env: its visibility envelope."""
        if ks is not None:
            keep, self.ks = self.ks, np.asarray(ks, dtype=np.float64)
            try:
                X = self.features(theta, taus)
            finally:
                self.ks = keep
        else:
            X = self.features(theta, taus)
        Y = (self.net.infer(X).astype(np.float64) * self.scale + self.mean).reshape(-1, len(taus), 4)
        return self.from_targets(Y, taus, env)

    @staticmethod
    def los_sources(S4):
        """(k S_T, k² S_E, S_ψ = 0) in the layout of the line-of-sight pipeline."""
        out = np.zeros(S4.shape[:2] + (3,))
        out[..., 0] = S4[..., 0] + S4[..., 1] + S4[..., 2]
        out[..., 1] = S4[..., 3]
        return out

    def save(self, path):
        self.net.save(path)
        np.savez(str(path) + ".norm.npz", mean=self.mean, scale=self.scale, ks=self.ks, ntau=self.ntau)

    def probe_error(self, theta, taus, env, S4_true, kprobe):
        """Relative L2 error of the predicted sources against solver sources at the probe modes."""
        P = self.predict(theta, taus, env, ks=kprobe)
        return float(np.linalg.norm(P - S4_true) / (np.linalg.norm(S4_true) + 1e-300))

    def spectra(self, thetas, jl, ls_out, kinterp, modes=("TT", "TE", "EE"), tol=0.05, kprobe=None, fallback=True):
        """C_ℓ for each θ: surrogate sources through the line-of-sight pipeline, or the solver for
        cosmologies whose probe-mode error exceeds tol.  Returns (Dl [ncos][nl][nmodes],
        probe errors, fallback mask)."""
        from . import CosmologyProblem, spectrum_cmb
        kprobe = np.geomspace(self.ks.min() * 10, self.ks.max() / 3, 4) if kprobe is None else np.asarray(kprobe)
        S4p, taus, env, prob = self.solve_sources(thetas, ks=kprobe)
        errs = np.array([self.probe_error(t, taus[c], env[c], S4p[c], kprobe) for c, t in enumerate(thetas)])
        fb = (errs > tol) if fallback else np.zeros(len(thetas), dtype=bool)
        out = []
        for c, t in enumerate(thetas):
            if fb[c]:
                p1 = CosmologyProblem(self.M, box_params(t))
                out.append(spectrum_cmb(list(modes), p1, jl, ls_out, kinterp=kinterp, taus=taus[c], normalization="Dl"))
            else:
                src = self.los_sources(self.predict(t, taus[c], env[c], ks=kinterp.xs))
                out.append(spectrum_cmb(list(modes), prob, jl, ls_out, kinterp=kinterp, taus=taus[c], cosmo=c, normalization="Dl",
                                        sources=src))
        return np.stack(out), errs, fb
