"""Symmetric H-matrices: the symmetric block tree (blcluster::subdivide_sym,
cluster/blcluster.cpp:90-113), the HeH assembly (matgenHeH_omp, ACAr,
Include/ACA.h:579-720, Include/apprx.h:86-132) and products (mltaHeHVec /
mltaHeHGeM, H/mltaGeHVec.cpp:421-475), against fixtures from the compiled
reference (tests/golden/make_golden.py sym).

CPU: trees bit-exact.  GPU: the product on the reference's own leaves within
1e-12, the GPU assembly's ranks and products against the reference's, mixed and
double-float products, GMRES with refinement, save/load with Hermitian records.
"""
import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

import mbls_format as F

CASES = ["sym_fib4096", "sym_sph360"]


def _relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _tree(g, kind):
    return A.HMatrix(g["points"], kind, bmin=int(g["bmin"]), eta=float(g["eta"]), symmetric=True)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_symmetric_tree_matches_reference(golden, case, kind):
    g = golden(case)
    H = _tree(g, kind)
    L = H.leaves()
    assert np.array_equal(L, g[f"{kind}_leaves"])
    n = H.n
    # diagonal and upper blocks only; diagonal blocks inadmissible; the upper
    # blocks twice plus the diagonal ones tile the matrix
    assert (L[:, 0] <= L[:, 2]).all()
    diag = L[:, 0] == L[:, 2]
    assert (L[diag, 4] == 0).all() and (L[diag, 1] == L[diag, 3]).all()
    area = 2 * (L[~diag, 1].astype(np.int64) * L[~diag, 3]).sum() + (L[diag, 1].astype(np.int64) ** 2).sum()
    assert area == n * n
    assert H.symmetric and _capi.lib().ahx_hmat_symmetric(H.handle) == 1


# ---------------------------------------------------------------- GPU ----

@pytest.mark.gpu
def test_symmetric_product_on_reference_leaves(golden):
    """The reference's HeH leaves (Hermitian diagonal blocks packed) uploaded as
    they are: y = A x within 1e-12 of its mltaHeHVec / mltaHeHGeM."""
    g = golden("sym_sph360")
    H = _tree(g, "pca")
    H.set_leaves(g["pca_ranks"], g["pca_data"], g["pca_offsets"])
    offs = g["pca_offsets"]
    for l in range(H.nleaves):   # getdata layout, packed for the Hermitian blocks
        assert np.array_equal(H.leaf_data(l), g["pca_data"][offs[l]:offs[l + 1]])
    y = H.mltaHeHVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(y, g["pca_y"]) <= 1e-12
    Y = H.mltaHeHVec(-0.5, g["X4"], np.zeros((4, H.n)))
    for r in range(4):
        assert _relerr(Y[r], g["pca_Y4"][r]) <= 1e-12
    # A^T = A
    yt = H.mltaGeHtVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(yt, y) <= 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_symmetric_assembly_matches_reference(golden, kind):
    g = golden("sym_fib4096")
    H = _tree(g, kind)
    H.matgenHeH_omp(float(g["h"]), float(g["eps"]))
    r, rr = H.ranks(), g[f"{kind}_ranks"]
    assert np.array_equal(r < 0, rr < 0)               # the same dense / low-rank decisions
    assert (r == rr).mean() >= 0.98 and np.abs(r - rr).max() <= 2
    y = H.mltaHeHVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(y, g[f"{kind}_y"]) <= 1e-6          # both approximate A to eps = 1e-6
    # the general assembly of the same matrix
    G = A.HMatrix(g["points"], kind, bmin=int(g["bmin"]), eta=float(g["eta"]))
    G.matgenGeH_omp(float(g["h"]), float(g["eps"]))
    y2 = G.mltaGeHVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(y, y2) <= 2e-6
    assert H.storage_bytes("fp64") < 0.62 * G.storage_bytes("fp64")   # upper blocks once


@pytest.mark.gpu
@pytest.mark.parametrize("p", [1, 16])
def test_symmetric_mixed_and_df64_products(golden, p):
    g = golden("sym_fib4096")
    H = _tree(g, "bbx")
    H.matgenHeH_omp(float(g["h"]), float(g["eps"]))
    X = np.random.default_rng(3).uniform(-1, 1, (p, H.n))
    Y64 = H.mltaHeHVec(1.0, X, np.zeros((p, H.n)))
    for prec, tol in (("fp32", 2e-6), ("bf16", 2e-2), ("df64", 1e-13)):
        Y = H.mltaHeHVec(1.0, X, np.zeros((p, H.n)), precision=prec)
        for r in range(p):
            assert _relerr(Y[r], Y64[r]) <= tol, (prec, r)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "bf16"])
def test_symmetric_gmres(golden, prec):
    g = golden("sym_fib4096")
    H = A.HMatrix(g["points"], "bbx", symmetric=True)
    H.matgenHeH_omp(float(g["h"]) / 2.0, 1e-6)       # diagonal 2/(4 pi h): positive definite
    b = np.random.default_rng(4).standard_normal(H.n)
    x = np.zeros(H.n)
    ret, eps, its = H.GMRes(b, x, 1e-8, 30, 300, precision=prec)
    assert ret == 0
    r = b - H.mltaHeHVec(1.0, x, np.zeros(H.n))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-8


@pytest.mark.gpu
def test_symmetric_save_load(golden, tmp_path):
    g = golden("sym_fib4096")
    H = _tree(g, "pca")
    H.matgenHeH_omp(float(g["h"]), float(g["eps"]))
    path = str(tmp_path / "sym.mbls")
    H.save(path)
    _, _, recs = F.read(path)
    L = H.leaves()
    for l, rec in enumerate(recs):
        if L[l, 0] == L[l, 2]:
            assert rec[2] == F.HERM and rec[4].size == L[l, 1] * (L[l, 1] + 1) // 2
    H2 = _tree(g, "pca")
    H2.load(path)
    for l in range(H.nleaves):
        assert np.array_equal(H2.leaf_data(l), H.leaf_data(l))
    x = g["x"]
    assert _relerr(H2.mltaHeHVec(1.0, x, np.zeros(H.n)), H.mltaHeHVec(1.0, x, np.zeros(H.n))) <= 1e-14


@pytest.mark.gpu
def test_symmetric_handles_are_not_batched(golden):
    g = golden("sym_sph360")
    H = _tree(g, "pca")
    H.set_leaves(g["pca_ranks"], g["pca_data"], g["pca_offsets"])
    with pytest.raises(_capi.AhxError, match="symmetric"):
        A.HBatch([H], precision="fp64")
