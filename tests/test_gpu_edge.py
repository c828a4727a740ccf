"""Edge cases on the GPU: one and two points, a tree of exactly one leaf (n = bmin)
and one leaf past it (n = bmin + 1), duplicate points, for the general and the
symmetric trees, every product precision, GMRES, save/load and agglomeration.
The dense product of the generator (diagonal 1/(4 pi h)) is the reference."""
import numpy as np
import pytest

import ahmed_gb300 as A

pytestmark = pytest.mark.gpu


def _dense(P, op, h):
    Q = P[op]
    d = np.sqrt(((Q[:, None, :] - Q[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(d, h)
    return 1.0 / (4.0 * np.pi * d)


def _points(n):
    if n <= 2:
        return np.array([[0.0, 0.0, 0.0], [1.0, 0.5, 0.25]][:n])
    return A.geometry.fibonacci_sphere(n)


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("n", [1, 2, 32, 33, 100])
def test_small_trees_all_precisions(n, symmetric, tmp_path):
    P = _points(n)
    h = 0.05
    H = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H.matgenGeH_omp(h, 1e-6)
    op, _ = H.perm()
    D = _dense(P, op, h)
    X = np.random.default_rng(n).uniform(-1, 1, (3, n))
    ref = (D @ X.T).T
    for prec, tol in (("fp64", 1e-6), ("df64", 1e-6), ("fp32", 1e-5), ("bf16", 3e-2)):
        for p in (1, 3):
            Y = H.mltaGeHVec(1.0, X[:p].copy(), np.zeros((p, n)), precision=prec)
            err = np.linalg.norm(Y - ref[:p]) / np.linalg.norm(ref[:p])
            assert err <= tol, (prec, p, err)
    # GMRES on the diagonally dominant variant
    H2 = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H2.matgenGeH_omp(1e-3, 1e-6)
    b = np.random.default_rng(1).standard_normal(n)
    x = np.zeros(n)
    ret, eps, its = H2.GMRes(b, x, 1e-10, 10, 100)
    assert ret == 0
    # save / load round trip
    path = str(tmp_path / "t.mbls")
    H.save(path)
    H3 = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H3.load(path)
    for l in range(H.nleaves):
        assert np.array_equal(H3.leaf_data(l), H.leaf_data(l))


def test_duplicate_points():
    """Coincident points: distance 0 off the diagonal gives infinite entries in the
    generator; the tree and the product still run, and the dense leaves hold inf."""
    P = np.zeros((40, 3))
    P[20:] = 1.0
    H = A.HMatrix(P, "bbx", bmin=32)
    assert H.nleaves >= 1
    L = H.leaves()
    assert (L[:, 1].astype(np.int64) * L[:, 3]).sum() == 40 * 40


def test_agglomeration_on_a_single_leaf():
    H = A.HMatrix(_points(2), "bbx", bmin=32)
    H.matgenGeH_omp(0.05, 1e-6)
    assert H.agglH(1e-6) == 0 and H.nleaves == 1


def _zdense(P, op, h, k):
    Q = P[op]
    d = np.sqrt(((Q[:, None, :] - Q[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(d, h)
    return np.exp(1j * k * d) / (4.0 * np.pi * d)


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("n", [1, 2, 32, 33, 100])
def test_small_trees_helmholtz(n, symmetric, tmp_path):
    """The Helmholtz leaves on the same small trees: A, A^H, A^T with complex128 and
    complex64 leaves, complex GMRES, save / load, agglomeration of a tiny tree."""
    P = _points(n)
    h, k = 0.05, 7.0
    H = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H.helmholtz_assemble(k, h, 1e-6)
    op, _ = H.perm()
    D = _zdense(P, op, h, k)
    rng = np.random.default_rng(n)
    X = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    for prec, tol in (("fp64", 1e-6), ("fp32", 1e-5)):
        for o, M in ((0, D), (1, D.conj().T), (2, D.T)):
            for p in (1, 3):
                Y = np.zeros((p, n), np.complex128)
                H._helm_product(o, 0.5 - 0.25j, p, X[:p].copy(), n, Y, n, prec)
                ref = (0.5 - 0.25j) * (M @ X[:p].T).T
                err = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
                assert err <= tol, (prec, o, p, err)
    H2 = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H2.helmholtz_assemble(k, 1e-3, 1e-6)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for prec in ("fp64", "fp32"):
        x = np.zeros(n, np.complex128)
        ret, eps, its = H2.GMRes(b, x, 1e-10, 10, 100, precision=prec)
        assert ret == 0, (prec, eps)
    path = str(tmp_path / "z.mbls")
    H.helm_save(path)
    H3 = A.HMatrix(P, "bbx", bmin=32, symmetric=symmetric)
    H3.helm_load(path)
    for l in range(H.nleaves):
        assert np.array_equal(H3.helm_leaf_data(l), H.helm_leaf_data(l))
    if not symmetric:
        H.helm_agglH(1e-6)  # nothing or little to merge on a tiny tree; must not fail
        Y = np.zeros((1, n), np.complex128)
        H.mltaGeHVec(1.0, X[:1].copy(), Y)
        ref = (D @ X[:1].T).T
        assert np.linalg.norm(Y - ref) <= 1e-5 * np.linalg.norm(ref)
