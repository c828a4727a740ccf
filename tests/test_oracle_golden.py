"""The CPU oracle against golden vectors produced by the reference library.

Bit-exact: cluster-tree permutations and the DFS leaf list (b1,n1,b2,n2,adm,idx,i0).
Toleranced: ACA ranks after recompression, products, GMRES.
"""
import numpy as np
import pytest

import oracle as O

CASES = ["fib4096", "cube3000", "ell2500", "sph360", "fib50"]
KINDS = [("bbx", O.TREE_BBX), ("pca", O.TREE_PCA)]


def _oracle(g, kind, h=None):
    return O.OracleH(g["points"], kind, int(g["bmin"]), float(g["eta"]),
                     float(g["h"]) if h is None else h)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kname,kind", KINDS)
def test_tree_bit_exact(golden, case, kname, kind):
    g = golden(case)
    H = _oracle(g, kind)
    op, po = H.perm()
    assert np.array_equal(op, g[f"{kname}_op_perm"])
    assert np.array_equal(po, g[f"{kname}_po_perm"])
    assert np.array_equal(H.leaves(), g[f"{kname}_leaves"])


def test_mean_nn_matches_golden_h(golden):
    g = golden("fib4096")
    assert O.mean_nn(g["points"]) == float(g["h"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kname,kind", KINDS)
def test_assembly_and_product(golden, case, kname, kind):
    g = golden(case)
    H = _oracle(g, kind)
    H.assemble(float(g["eps"]), nthreads=2)
    ranks = H.ranks()
    ref = g[f"{kname}_ranks"]
    # dense/low-rank decisions identical, truncated ranks identical on >= 99% of leaves
    assert np.array_equal(ranks >= 0, ref >= 0)
    assert (ranks == ref).mean() >= 0.99
    assert np.abs(ranks - ref).max() <= 1
    n = H.n
    y = H.matvec(g["x"], np.zeros(n))
    yr = g[f"{kname}_y"]
    assert np.linalg.norm(y - yr) <= 1e-8 * np.linalg.norm(yr)
    Y = H.matvec(g["X4"], np.zeros((4, n)), d=-0.5)
    Yr = g[f"{kname}_Y4"]
    for r in range(4):
        assert np.linalg.norm(Y[r] - Yr[r]) <= 1e-8 * np.linalg.norm(Yr[r])


@pytest.mark.parametrize("kname,kind", KINDS)
def test_product_on_reference_leaves(golden, kname, kind):
    """Oracle product on the reference's own leaf data reproduces mltaGeHVec to 1e-13."""
    g = golden("sph360")
    H = _oracle(g, kind)
    offs = g[f"{kname}_offsets"]
    data = g[f"{kname}_data"]
    for l, rk in enumerate(g[f"{kname}_ranks"]):
        H.set_leaf(l, int(rk), data[offs[l]:offs[l + 1]])
    n = H.n
    y = H.matvec(g["x"], np.zeros(n))
    yr = g[f"{kname}_y"]
    assert np.linalg.norm(y - yr) <= 1e-13 * np.linalg.norm(yr)
    Y = H.matvec(g["X4"], np.zeros((4, n)), d=-0.5)
    for r in range(4):
        assert np.linalg.norm(Y[r] - g[f"{kname}_Y4"][r]) <= 1e-13 * np.linalg.norm(g[f"{kname}_Y4"][r])


def test_block_errors_within_check_error_bound(golden):
    """apprx.h:47 criterion: every low-rank leaf within 20*eps of its dense block."""
    g = golden("ell2500")
    H = _oracle(g, O.TREE_PCA)
    eps = float(g["eps"])
    H.assemble(eps, nthreads=2)
    K = H.dense()
    lv = H.leaves()
    ranks = H.ranks()
    for l in np.nonzero(ranks > 0)[0]:
        b1, n1, b2, n2 = (int(v) for v in lv[l, :4])
        k = int(ranks[l])
        d = H.leaf_data(l)
        U = d[: n1 * k].reshape(k, n1).T
        V = d[n1 * k:].reshape(k, n2).T
        B = K[b1:b1 + n1, b2:b2 + n2]
        assert np.linalg.norm(U @ V.T - B) <= 20 * eps * np.linalg.norm(B)


@pytest.mark.parametrize("case,tag", [("fib4096", "spec"), ("fib4096", "spd"),
                                      ("cube3000", "spec"), ("cube3000", "spd")])
def test_gmres_matches_reference(golden, case, tag):
    g = golden(case)
    H = _oracle(g, O.TREE_BBX, h=float(g[f"gmres_{tag}_h"]))
    H.assemble(float(g["eps"]), nthreads=2)
    ret_r, eps_r, ns_r = g[f"gmres_{tag}"]
    x = np.zeros(H.n)
    ret, eps, ns = H.gmres(g["gmres_b"], x, 1e-8, 30, 150, nthreads=2)
    assert ret == int(ret_r)
    if ret == 0:
        assert abs(int(ns) - int(ns_r)) <= 2
        assert eps < 1e-8
        xr = g[f"gmres_{tag}_x"]
        assert np.linalg.norm(x - xr) <= 1e-5 * np.linalg.norm(xr)
    else:
        assert ns == int(ns_r)
        assert abs(eps - eps_r) <= 1e-3 * eps_r


@pytest.mark.parametrize("case", ["fib4096", "cube3000"])
@pytest.mark.parametrize("tag,steps", [("conv", 300), ("cap", 8)])
def test_cg_matches_reference(golden, case, tag, steps):
    """The oracle's CG (solvers/CG.cpp:31-113) against the reference's own CG on its
    own assembly: a converging solve and one stopped by the step limit."""
    g, c = golden(case), golden("cg")
    H = _oracle(g, O.TREE_BBX, h=float(c[f"{case}_h"]))
    H.assemble(float(g["eps"]), nthreads=2)
    ret_r, eps_r, ns_r = c[f"{case}_{tag}"]
    x = np.zeros(H.n)
    ret, eps, ns = H.cg(c[f"{case}_b"], x, 1e-8, steps, nthreads=2)
    assert ret == int(ret_r)
    xr = c[f"{case}_{tag}_x"]
    if ret == 0:
        assert abs(int(ns) - int(ns_r)) <= 2
        assert eps < 1e-8
        assert np.linalg.norm(x - xr) <= 1e-5 * np.linalg.norm(xr)
    else:
        assert ns == int(ns_r)
        assert abs(eps - eps_r) <= 1e-3 * eps_r
        assert np.linalg.norm(x - xr) <= 1e-4 * np.linalg.norm(xr)
