"""Agglomeration of Helmholtz (mblock<dcomp>) leaves: agglH with T = dcomp
(H/agglH.cpp:291-305) against the compiled reference (tests/golden/make_golden.py
zaggl).  As for real leaves, the sons are united pairwise as in the reference
(block rows first, truncating after each step).  Checked: the leaves tile the
matrix, the product stays within the assembly accuracy of the reference's
agglomerated product, the same leaves as the reference's (99% or more, count
and storage within 1%), indices compacted; the real leaves of the handle are
dropped; save/load and complex64 products on the new leaves."""
import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

CASES = ["zaggl_fib4096", "zaggl_ell2500"]
TREE = {0: "bbx", 1: "pca"}


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _dense(g):
    P = g["points"][g["op_perm"]]
    D = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, float(g["h"]))
    return np.exp(1j * float(g["k"]) * D) / (4.0 * np.pi * D)


@pytest.mark.parametrize("name", CASES)
def test_fixture_product_matches_dense(golden, name):
    g = golden(name)
    M = _dense(g)
    assert _rel(g["y"], M @ g["x"]) < 2e-5
    L = g["leaves"]
    n = len(g["x"])
    assert (L[:, 1].astype(np.int64) * L[:, 3]).sum() == n * n
    assert len(L) < int(g["nleaves_before"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_agglomeration_against_reference(golden, name, tmp_path):
    g = golden(name)
    H = A.HMatrix(g["points"], TREE[int(g["kind"])], bmin=int(g["bmin"]), eta=float(g["eta"]))
    H.matgenGeH_omp(float(g["h"]), float(g["eps"]))  # real leaves, dropped below
    H.helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
    x = g["x"]
    y0 = H.mltaGeHVec(1.0, x, np.zeros_like(x))
    n_before = H.nleaves
    merged = H.helm_agglH(float(g["eps"]))
    assert merged > 0 and H.nleaves < n_before
    L = H.leaves()
    n = H.n
    assert (L[:, 1].astype(np.int64) * L[:, 3]).sum() == n * n
    assert np.array_equal(L[:, 5], np.arange(H.nleaves))
    y = H.mltaGeHVec(1.0, x, np.zeros_like(x))
    assert _rel(y, y0) <= 1e-5
    assert _rel(y, g["y"]) <= 1e-5
    ref = g["leaves"]
    assert abs(H.nleaves - len(ref)) <= 0.01 * len(ref)
    stored = sum(H.helm_leaf_data(l).size for l in range(H.nleaves))
    assert abs(stored - int(g["stored"])) <= 0.01 * int(g["stored"])
    ours = {tuple(r) for r in L[:, :4].tolist()}
    theirs = {tuple(r) for r in ref[:, :4].tolist()}
    assert len(ours & theirs) >= 0.99 * len(theirs)
    # the real leaves belonged to the old block tree
    with pytest.raises(_capi.AhxError, match="not assembled"):
        H.mltaGeHVec(1.0, np.zeros(n), np.zeros(n))
    # complex64 products and a file round trip on the new leaves
    y32 = H.mltaGeHVec(1.0, x, np.zeros_like(x), precision="fp32")
    assert _rel(y32, y) <= 2e-5
    path = str(tmp_path / "aggl.mbls")
    H.helm_save(path)
    G = A.HMatrix(g["points"], TREE[int(g["kind"])], bmin=int(g["bmin"]), eta=float(g["eta"]))
    with pytest.raises(_capi.AhxError, match="leaves"):
        G.helm_load(path)  # the file holds the agglomerated leaf list, not this tree's
    G.close()
    H.close()


@pytest.mark.gpu
def test_real_agglomeration_drops_helmholtz_leaves(golden):
    g = golden("zaggl_ell2500")
    H = A.HMatrix(g["points"], "pca", bmin=int(g["bmin"]), eta=float(g["eta"]))
    H.helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
    H.matgenGeH_omp(float(g["h"]), float(g["eps"]))
    assert H.agglH(float(g["eps"])) > 0
    with pytest.raises(_capi.AhxError, match="not assembled"):
        H.mltaGeHVec(1.0, g["x"], np.zeros_like(g["x"]))
    # Helmholtz leaves assembled on the agglomerated tree work again
    H.helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
    y = H.mltaGeHVec(1.0, g["x"], np.zeros_like(g["x"]))
    assert _rel(y, g["y"]) <= 1e-5
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cplx", [False, True])
def test_symmetric_tree_agglomeration(golden, cplx):
    """Symmetric block trees (upper blocks only): the unions stay above the diagonal,
    the product of the agglomerated matrix stays within the assembly accuracy and the
    storage shrinks, for real (HeH) and complex symmetric (SyH) leaves."""
    g = golden("zaggl_fib4096")
    H = A.HMatrix(g["points"], "bbx", bmin=int(g["bmin"]), eta=float(g["eta"]), symmetric=True)
    x = g["x"] if cplx else g["x"].real.copy()
    if cplx:
        H.helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
        stored0 = sum(H.helm_leaf_data(l).size for l in range(H.nleaves))
    else:
        H.matgenGeH_omp(float(g["h"]), float(g["eps"]))
        stored0 = sum(H.leaf_data(l).size for l in range(H.nleaves))
    y0 = H.mltaGeHVec(1.0, x, np.zeros_like(x))
    n0 = H.nleaves
    merged = H.helm_agglH(float(g["eps"])) if cplx else H.agglH(float(g["eps"]))
    assert merged > 0 and H.nleaves < n0
    L = H.leaves()
    assert np.all(L[:, 0] <= L[:, 2])  # upper blocks only
    y = H.mltaGeHVec(1.0, x, np.zeros_like(x))
    assert _rel(y, y0) <= 1e-5
    stored = sum((H.helm_leaf_data(l) if cplx else H.leaf_data(l)).size for l in range(H.nleaves))
    assert stored < stored0
    H.close()
