"""Helmholtz (complex) H-matrix: assembly, products A / A^H / A^T, GMRES.

Fixtures (tests/golden/make_golden.py zhmat) hold the reference's own results
with T = dcomp: the mblock<dcomp> ranks of every leaf after ACA<dcomp> and
addtrll, Y0 + d op(A) X for its mltaGeHGeM / mltaGeHhGeM / mltaGeHtGeM, the
factors of 40 low-rank leaves, and the solution of its complex GMRes; zhs_*:
the complex symmetric form on the symmetric block tree (matgenSyH_omp: ACAr,
packed symmetric diagonal blocks; mltaSyHGeM).  The CPU tests pin the fixtures
to the dense complex matrix; the GPU tests compare the library with them."""
import numpy as np
import pytest

import ahmed_gb300 as A

CASES = ["zh_fib4096", "zh_ell2500", "zhs_fib4096", "zhs_ell2500"]
TREE = {0: "bbx", 1: "pca"}


def dense(g, h):
    P = g["points"][g["op_perm"]]
    D = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, h)
    return np.exp(1j * float(g["k"]) * D) / (4.0 * np.pi * D)


def ops(M):
    return {0: M, 1: M.conj().T, 2: M.T}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


# ---------------------------------------------------------------- CPU: fixtures
@pytest.mark.parametrize("name", CASES)
def test_fixture_products_match_dense(golden, name):
    g = golden(name)
    M = dense(g, float(g["h"]))
    d = complex(g["d"])
    for op, Mo in ops(M).items():
        want = g["Y0"] + d * (Mo @ g["X"].T).T
        assert rel(g[f"Y_op{op}"], want) < 5e-6, op


@pytest.mark.parametrize("name", CASES)
def test_fixture_gmres_solution(golden, name):
    g = golden(name)
    M = dense(g, float(g["gm_h"]))
    assert rel(M @ g["gm_x"], g["gm_b"]) < 1e-6  # the H-matrix approximates M to about eps
    assert g["gm_resid"] < 1e-8


@pytest.mark.parametrize("name", CASES)
def test_fixture_leaves(golden, name):
    g = golden(name)
    L = g["leaves"]
    r = g["ranks"]
    assert np.all(r[L[:, 4] == 0] == -1)  # inadmissible leaves are dense
    assert (r >= 0).sum() > 0
    M = dense(g, float(g["h"]))
    for q, l in enumerate(g.get("sym_leaves", [])):  # packed upper triangles
        b1, n1 = int(L[l, 0]), int(L[l, 1])
        iu = np.triu_indices(n1)
        want = M[b1:b1 + n1, b1:b1 + n1].T[np.tril_indices(n1)]  # column by column, rows <= column
        assert rel(g[f"sym_data{q}"], want) < 1e-14
        assert iu[0].size == g[f"sym_data{q}"].size
    if "data" not in g:
        return
    for q, l in enumerate(g["data_leaves"]):
        b1, n1, b2, n2 = (int(v) for v in L[l, :4])
        k = int(r[l])
        c = g["data"][int(g["offsets"][q]):int(g["offsets"][q + 1])]
        U = c[:n1 * k].reshape(k, n1).T
        V = c[n1 * k:].reshape(k, n2).T
        blk = M[b1:b1 + n1, b2:b2 + n2]
        assert rel(U @ V.conj().T, blk) < 2e-5, l


@pytest.mark.parametrize("name", CASES)
def test_fixture_trees_match(golden, name):
    g = golden(name)
    H = A.HMatrix(g["points"], TREE[int(g["kind"])], bmin=int(g["bmin"]), eta=float(g["eta"]),
                  symmetric=bool(g["sym"]))
    np.testing.assert_array_equal(H.leaves(), g["leaves"])
    np.testing.assert_array_equal(H.perm()[0], g["op_perm"])
    H.close()


# ---------------------------------------------------------------- GPU
def _hmat(g, h=None):
    H = A.HMatrix(g["points"], TREE[int(g["kind"])], bmin=int(g["bmin"]), eta=float(g["eta"]),
                  symmetric=bool(g["sym"]))
    H.helmholtz_assemble(float(g["k"]), float(g["h"] if h is None else h), float(g["eps"]))
    return H


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_ranks_match_reference(golden, name):
    g = golden(name)
    H = _hmat(g)
    got, ref = H.helm_ranks(), g["ranks"]
    np.testing.assert_array_equal(got < 0, ref < 0)  # the same dense leaves
    lr = ref >= 0
    assert (got[lr] == ref[lr]).mean() >= 0.95, (got[lr] != ref[lr]).sum()
    assert np.abs(got[lr] - ref[lr]).max() <= 2
    # leaf data: U V^H of the sampled leaves against the reference's
    L = g["leaves"]
    for q, l in enumerate(g.get("data_leaves", [])):
        b1, n1, b2, n2 = (int(v) for v in L[l, :4])
        c = g["data"][int(g["offsets"][q]):int(g["offsets"][q + 1])]
        k = int(ref[l])
        Ur, Vr = c[:n1 * k].reshape(k, n1).T, c[n1 * k:].reshape(k, n2).T
        mine = H.helm_leaf_data(int(l))
        kg = int(got[l])
        assert mine.size == kg * (n1 + n2)
        Ug, Vg = mine[:n1 * kg].reshape(kg, n1).T, mine[n1 * kg:].reshape(kg, n2).T
        want = Ur @ Vr.conj().T
        assert rel(Ug @ Vg.conj().T, want) < 1e-5, l
    for q, l in enumerate(g.get("sym_leaves", [])):  # packed symmetric diagonal blocks
        assert rel(H.helm_leaf_data(int(l)), g[f"sym_data{q}"]) < 1e-14
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_products_match_reference(golden, name):
    g = golden(name)
    H = _hmat(g)
    d = complex(g["d"])
    X = np.ascontiguousarray(g["X"])
    M = dense(g, float(g["h"]))
    for op, Mo in ops(M).items():
        Y = np.ascontiguousarray(g["Y0"]).copy()
        if op == 0:
            H.mltaGeHVec(d, X, Y)
        elif op == 1:
            H.mltaGeHhVec(d, X, Y)
        else:
            H.mltaGeHtVec(d, X, Y)
        assert rel(Y, g[f"Y_op{op}"]) < 1e-5, op  # the reference's product
        exact = g["Y0"] + d * (Mo @ X.T).T
        assert rel(Y, exact) < 5e-6, op  # the dense matrix
        # complex64 leaves
        Y32 = np.ascontiguousarray(g["Y0"]).copy()
        H._helm_product(op, d, X.shape[0], X, H.n, Y32, H.n, "fp32")
        assert rel(Y32, Y) < 2e-5, op
    H.close()


@pytest.mark.gpu
def test_product_device_pointers_and_many_rhs(golden):
    import torch

    g = golden("zh_fib4096")
    H = _hmat(g)
    n = H.n
    rng = np.random.default_rng(5)
    for p in (1, 3, 9):
        X = rng.standard_normal((p, n)) + 1j * rng.standard_normal((p, n))
        Yh = np.zeros((p, n), np.complex128)
        H.mltaGeHVec(0.5 + 0.25j, X, Yh)
        Xd = torch.from_numpy(X).cuda()
        Yd = torch.zeros((p, n), dtype=torch.complex128, device="cuda")
        H.mltaGeHVec(0.5 + 0.25j, Xd, Yd)
        torch.cuda.synchronize()
        assert rel(Yd.cpu().numpy(), Yh) < 1e-13
        # columns are independent: one at a time gives the same
        for c in range(p):
            y1 = np.zeros(n, np.complex128)
            H.mltaGeHVec(0.5 + 0.25j, X[c], y1)
            assert rel(y1, Yh[c]) < 1e-13
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gmres_matches_reference(golden, name):
    g = golden(name)
    H = _hmat(g, h=float(g["gm_h"]))
    b = np.ascontiguousarray(g["gm_b"])
    x = np.zeros_like(b)
    st, res, its = H.GMRes(b, x, 1e-8, int(g["gm_m"]), int(g["gm_m"]))
    assert st == 0 and res[0] < 1e-8
    assert abs(int(its[0]) - int(g["gm_iters"])) <= 2, (its, g["gm_iters"])
    assert rel(x, g["gm_x"]) < 1e-6
    # true residual with the dense matrix
    M = dense(g, float(g["gm_h"]))
    assert rel(M @ x, b) < 1e-6
    # complex64 leaves with FP64 refinement reach the same tolerance
    x32 = np.zeros_like(b)
    st32, res32, its32 = H.GMRes(b, x32, 1e-8, 30, 500, precision="fp32")
    assert st32 == 0 and res32[0] < 1e-8
    assert rel(M @ x32, b) < 1e-6
    H.close()


@pytest.mark.gpu
def test_gmres_restart_and_limits(golden):
    """Restarted cycles (m smaller than the steps needed) converge from the true
    residual; an iteration limit below that reports not converged."""
    g = golden("zh_fib4096")
    H = _hmat(g, h=float(g["gm_h"]))
    b = np.ascontiguousarray(g["gm_b"])
    x = np.zeros_like(b)
    st, res, its = H.GMRes(b, x, 1e-8, 10, 400)
    assert st == 0 and res[0] < 1e-8
    M = dense(g, float(g["gm_h"]))
    assert rel(M @ x, b) < 1e-6
    x2 = np.zeros_like(b)
    st2, res2, its2 = H.GMRes(b, x2, 1e-8, 10, 5)
    assert st2 == 1 and its2[0] == 5 and res2[0] > 1e-8
    # zero right-hand side: x = 0, no steps
    z = np.zeros_like(b)
    xz = np.ones_like(b)
    st3, res3, its3 = H.GMRes(z, xz, 1e-8, 10, 10)
    assert st3 == 0 and its3[0] == 0 and not xz.any()
    H.close()


@pytest.mark.gpu
def test_errors(golden):
    from ahmed_gb300._capi import AHX_ERR_ARG, AHX_ERR_STATE, lib, ptr

    g = golden("zh_ell2500")
    H = A.HMatrix(g["points"], "pca", bmin=int(g["bmin"]), eta=float(g["eta"]))
    X = np.zeros(H.n, np.complex128)
    Y = np.zeros(H.n, np.complex128)
    assert lib().ahx_helm_matvec(H.handle, 0, 0, 1.0, 0.0, 1, ptr(X), H.n, ptr(Y), H.n) == AHX_ERR_STATE
    H.helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
    assert lib().ahx_helm_matvec(H.handle, 2, 0, 1.0, 0.0, 1, ptr(X), H.n, ptr(Y), H.n) == AHX_ERR_ARG  # bf16
    assert lib().ahx_helm_matvec(H.handle, 0, 3, 1.0, 0.0, 1, ptr(X), H.n, ptr(Y), H.n) == AHX_ERR_ARG  # op
    assert lib().ahx_helm_assemble(H.handle, 5.0, -1.0, 1e-6, 2**32 - 1) == AHX_ERR_ARG  # h <= 0
    assert lib().ahx_helm_assemble(H.handle, float("nan"), 1.0, 1e-6, 2**32 - 1) == AHX_ERR_ARG
    H.close()
