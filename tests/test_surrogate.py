"""Source surrogate: the device MLP (BF16 tensor-core forward/backward, FP32 accumulation) against the
CPU oracle (oracle/mlp.py), training, weight files, and the surrogate → line-of-sight path with its
solver fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = dict(nin=8, width=128, nhidden=2, nout=4)


def _mlp(batch=256, seed=1):
    from symboltz.surrogate import MLP
    return MLP(SIZES["nin"], SIZES["width"], SIZES["nhidden"], SIZES["nout"], batch, seed)


def _layers():
    import mlp as MO
    return MO.layer_sizes(SIZES["nin"], SIZES["width"], SIZES["nhidden"], SIZES["nout"])


def _rel(a, b):
    return float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-300))


def test_gradients_match_oracle():
    """Loss and every layer's gradient against FP64 backpropagation on the same BF16-rounded
    operands; the remaining difference is the device's BF16 activations (relative ~1e-2)."""
    import mlp as MO
    net = _mlp()
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (256, 8)).astype(np.float32)
    Y = rng.normal(size=(256, 4)).astype(np.float32)
    p = net.get_params().astype(np.float64)
    loss, g = net.gradients(X, Y)
    lo, go = MO.loss_and_grad(p, X, Y, _layers(), bf16_operands=True)
    assert abs(loss - lo) / lo < 1e-2
    o = 0
    for a, b in zip(_layers()[:-1], _layers()[1:]):
        for n in (a * b, b):
            assert _rel(g[o:o + n], go[o:o + n]) < 3e-2, (a, b, n)
            o += n
    assert o == len(g)


def test_inference_matches_oracle_forward():
    import mlp as MO
    net = _mlp()
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (1000, 8)).astype(np.float32)  # not a multiple of 128: padded rows are dropped
    got = net.infer(X)
    xs, _ = MO.forward(net.get_params().astype(np.float64), X, _layers(), bf16_operands=True)
    assert _rel(got, xs[-1]) < 2e-2


def test_training_reduces_loss_and_weights_round_trip(tmp_path):
    net = _mlp(batch=512, seed=2)
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, (20000, 8)).astype(np.float32)
    Y = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], np.cos(X[:, 2] + X[:, 3]), X[:, 4] ** 2, X[:, 5] - X[:, 6] * X[:, 7]], axis=1)
    net.set_data(X, Y.astype(np.float32))
    first = net.train(1, 1e-3)
    last = net.train(600, 2e-3)
    assert last < 0.2 * first, (first, last)
    from symboltz.surrogate import MLP
    path = tmp_path / "w.bin"
    net.save(path)
    back = MLP.load(path, batch=512)
    np.testing.assert_array_equal(back.get_params(), net.get_params())
    np.testing.assert_array_equal(back.infer(X[:300]), net.infer(X[:300]))


def test_surrogate_sources_through_the_line_of_sight_with_fallback():
    """A small surrogate end to end: trained on solver sources of a few cosmologies, its sources feed
    the line-of-sight pipeline; with tolerance 0 every cosmology falls back to the solver and the
    spectra equal the solver's."""
    import symboltz as S
    from symboltz.surrogate import SourceSurrogate, box_params, sample_box
    M = S.ΛCDM(lmax=5)
    ks = S.k_from_hMpc(S.loggrid(1e-4, 0.3, length=32))
    sur = SourceSurrogate(M, ks, ntau=48, width=128, nhidden=2, batch=1024, seed=3)
    train = sample_box(4, seed=0)
    X, Y, _ = sur.dataset(train)
    assert X.shape == (4 * 32 * 48, SourceSurrogate.NIN) and Y.shape == (4 * 32 * 48, 7) and np.all(np.isfinite(Y))
    sur.fit(X, Y, steps=1, lr=1e-4)
    before = sur.mse(X, Y)
    sur.fit(X, Y, steps=400, lr=2e-3, lr_final=2e-4, chunks=4)
    assert sur.mse(X, Y) < before  # learning quality is measured at full resolution (bench); here the plumbing
    test = sample_box(2, seed=1)
    jl = S.SphericalBesselCache(np.arange(2, 401, 10))
    kin = S.CubicSplineInterpolator(ks, f=np.log)
    ls = np.arange(2, 393)
    Dl, err, fb = sur.spectra(test, jl, ls, kin, tol=np.inf)
    assert not fb.any() and np.all(np.isfinite(Dl)) and np.all(np.isfinite(err))
    Draw, err_raw, fb_raw = sur.spectra(test, jl, ls, kin, fallback=False)  # no probe modes solved
    assert not fb_raw.any() and np.all(np.isnan(err_raw))
    np.testing.assert_allclose(Draw, Dl, rtol=1e-12)
    Dfb, err2, fb2 = sur.spectra(test, jl, ls, kin, tol=0.0)
    assert fb2.all()
    np.testing.assert_allclose(err2, err)
    _, taus, _, _ = sur.solve_factors(test[:1])
    ref = S.spectrum_cmb(["TT", "TE", "EE"], S.CosmologyProblem(M, box_params(test[0])), jl, ls, kinterp=kin, taus=taus[0],
                         normalization="Dl")
    np.testing.assert_allclose(Dfb[0], ref, rtol=1e-12)


def test_factors_rebuild_the_solver_sources():
    """Sources assembled from the solver's factors and the background visibility equal the solver's
    own sources (same operator, same coefficient table)."""
    import symboltz as S
    from symboltz.surrogate import SourceSurrogate, sample_box
    M = S.ΛCDM(lmax=5)
    ks = S.k_from_hMpc(S.loggrid(1e-4, 0.3, length=16))
    sur = SourceSurrogate(M, ks, ntau=40, width=128, nhidden=1, batch=128)
    F, taus, vis, prob = sur.solve_factors(sample_box(1, seed=5))
    rebuilt = sur.sources(F[0], ks, taus[0], vis[0])
    direct, st, _ = S.solvept(prob, ks, prob.opts.tau_ini, saveat=taus[0], output="sources")
    assert np.all(st == 0)
    direct[:, -1, :] = 0.0
    for s in range(2):
        scale = np.max(np.abs(direct[..., s]))
        np.testing.assert_allclose(rebuilt[..., s], direct[..., s], rtol=0, atol=1e-9 * scale)
