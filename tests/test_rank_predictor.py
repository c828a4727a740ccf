"""Learned ACA-rank predictor: the network's gradients against the float64
oracle, training on the GPU, and rank-hinted assembly (identical ranks with a
smaller ACA workspace than the fixed-capacity default)."""
import numpy as np
import pytest

from ahmed_gb300 import HMatrix, RankPredictor, mean_nn, training_set
from ahmed_gb300.geometry import ellipsoid_surface, fibonacci_sphere
import mlp_ref


def _random_params(rng):
    p = rng.standard_normal(mlp_ref.NPARAMS) * 0.3
    return p.astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _random_params(rng).astype(np.float64)
    X = rng.standard_normal((40, 8))
    y = rng.standard_normal(40)
    mean, std = X.mean(0), X.std(0)
    loss, g = mlp_ref.loss_and_grad(p, X, y, mean, std)
    idx = rng.choice(mlp_ref.NPARAMS, 60, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        lp, _ = mlp_ref.loss_and_grad(p + e, X, y, mean, std)
        lm, _ = mlp_ref.loss_and_grad(p - e, X, y, mean, std)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * (1 + abs(g[i])), (i, fd, g[i])


def test_leaf_features_host():
    pts = fibonacci_sphere(2000)
    H = HMatrix(pts, tree="pca", bmin=32, eta=0.8)
    F = H.features(1e-6)
    lv = H.leaves()
    assert F.shape == (H.nleaves, 8)
    assert np.all(np.isfinite(F))
    np.testing.assert_allclose(F[:, 4], np.log(lv[:, 1]), rtol=1e-6)
    np.testing.assert_allclose(F[:, 5], np.log(lv[:, 3]), rtol=1e-6)
    np.testing.assert_allclose(F[:, 7], 6.0, rtol=1e-6)
    assert np.all(F[:, 6] == 0)
    adm = lv[:, 4] == 1
    # admissible leaves are separated: min(diam)/dist is bounded by eta for PCA trees
    assert np.all(F[adm, 3] < 1.0)
    H.close()


def _mats(sizes, tree="bbx"):
    out = []
    for n, shape in sizes:
        pts = fibonacci_sphere(n) if shape == "sphere" else ellipsoid_surface(n, seed=n)
        out.append((pts, HMatrix(pts, tree=tree, bmin=32, eta=0.8)))
    return out


@pytest.mark.gpu
def test_gpu_gradients_match_oracle():
    rng = np.random.default_rng(7)
    M = RankPredictor(seed=1)
    p = _random_params(rng)
    M.params = p
    np.testing.assert_array_equal(M.params, p)
    X = (rng.standard_normal((3000, 8)) * 2 + 1).astype(np.float32)
    y = rng.standard_normal(3000).astype(np.float32)
    mean, std = X.mean(0), X.std(0)
    M.set_norm(mean, std)
    g, loss = M.gradients(X, y)
    lo, go = mlp_ref.loss_and_grad(p, X, y, mean.astype(np.float64), std.astype(np.float64))
    # FP32 arithmetic over 3000 samples: norm-wise relative error well below 1e-4
    assert abs(loss - lo) <= 1e-4 * lo
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    # the forward pass alone
    out = M.predict_log(X[:500])
    ref = mlp_ref.forward(p, X[:500], mean.astype(np.float64), std.astype(np.float64))[-1]
    np.testing.assert_allclose(out, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    M.close()


@pytest.mark.gpu
def test_gpu_training_and_hinted_assembly():
    eps = 1e-6
    train = _mats([(3000, "sphere"), (5000, "ellipsoid"), (8000, "sphere")])
    for pts, H in train:
        H.matgenGeH_omp(mean_nn(pts), eps)
    X, r = training_set([H for _, H in train], eps)
    M = RankPredictor(seed=0)
    losses = M.fit(X, r, epochs=60, batch=512, lr=3e-3)
    assert losses[-1] < 0.25 * losses[0]
    assert losses[-1] < 0.05  # mean squared error of log(1 + rank)

    # held-out geometry
    pts = ellipsoid_surface(12000, seed=5, axes=(1.0, 0.7, 0.4))
    h = mean_nn(pts)
    H0 = HMatrix(pts, tree="bbx", bmin=32, eta=0.8).matgenGeH_omp(h, eps)
    r0, a0 = H0.ranks(), H0.aca_ranks()
    ws0 = H0.assembly_stats()[0]
    F = H0.features(eps)
    pred = M.predict(F)
    adm = (H0.leaves()[:, 4] == 1) & (a0 >= 0)
    rel = np.abs(pred[adm] - a0[adm]) / np.maximum(a0[adm], 1)
    assert np.median(rel) < 0.25

    H1 = HMatrix(pts, tree="bbx", bmin=32, eta=0.8)
    H1.assemble_hinted(h, eps, np.where(H1.leaves()[:, 4] == 1, pred, -1.0))
    # the hints size the workspace only: every rank is the one ACA chooses
    np.testing.assert_array_equal(H1.aca_ranks(), a0)
    np.testing.assert_array_equal(H1.ranks(), r0)
    ws1, retries1, _ = H1.assembly_stats()
    assert ws1 < 0.7 * ws0, (ws1, ws0)
    assert retries1 <= 0.02 * adm.sum()
    x = np.random.default_rng(0).standard_normal(len(pts))
    y0 = np.zeros_like(x)
    y1 = np.zeros_like(x)
    H0.mltaGeHVec(1.0, x, y0)
    H1.mltaGeHVec(1.0, x, y1)
    assert np.linalg.norm(y1 - y0) <= 1e-13 * np.linalg.norm(y0)
    for _, H in train:
        H.close()
    H0.close()
    H1.close()
    M.close()
