"""Agglomeration (agglH, H/agglH.cpp:111-272; matgenGeH_sqntl with recmpr,
Include/matgen_sqntl.h:32-55) against the compiled reference
(tests/golden/make_golden.py aggl).

The sons of a block are united pairwise as in the reference (the two sons of
each block row, then the two block rows, truncating after each step), with this
library's own QR + SVD recompression.  Checked: the leaves still tile the
matrix; the product is within the assembly accuracy of the reference's
agglomerated product; the same leaves as the reference's (99% or more, leaf
count within 1%) and storage within 1%; leaf indices compacted (0 .. n-1);
mixed products, save/load and a second call's error.
"""
import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

pytestmark = pytest.mark.gpu


def _relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _stored(H):
    return sum(H.leaf_data(l).size for l in range(H.nleaves))


@pytest.mark.parametrize("case", ["aggl_fib4096", "aggl_cube3000"])
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_agglomeration_against_reference(golden, case, kind):
    g = golden(case)
    H = A.HMatrix(g["points"], kind, bmin=int(g["bmin"]), eta=float(g["eta"]))
    H.matgenGeH_omp(float(g["h"]), float(g["eps"]))
    y0 = H.mltaGeHVec(1.0, g["x"], np.zeros(H.n))
    n_before = H.nleaves
    merged = H.agglH(float(g["eps"]))
    assert merged > 0 and H.nleaves < n_before
    L = H.leaves()
    n = H.n
    # a tiling of the matrix, indices 0 .. n-1
    assert (L[:, 1].astype(np.int64) * L[:, 3]).sum() == n * n
    assert np.array_equal(L[:, 5], np.arange(H.nleaves))
    y = H.mltaGeHVec(1.0, g["x"], np.zeros(n))
    assert _relerr(y, y0) <= 5e-6
    assert _relerr(y, g[f"{kind}_y"]) <= 5e-6
    ref_leaves = g[f"{kind}_leaves"]
    assert abs(H.nleaves - len(ref_leaves)) <= 0.01 * len(ref_leaves)
    assert abs(_stored(H) - int(g[f"{kind}_stored"])) <= 0.01 * int(g[f"{kind}_stored"])
    ours = {tuple(r) for r in L[:, :4].tolist()}
    theirs = {tuple(r) for r in ref_leaves[:, :4].tolist()}
    assert len(ours & theirs) >= 0.99 * len(theirs)
    # mixed products on the agglomerated leaves
    X = np.random.default_rng(5).uniform(-1, 1, (16, n))
    Y64 = H.mltaGeHVec(1.0, X, np.zeros((16, n)))
    Y32 = H.mltaGeHVec(1.0, X, np.zeros((16, n)), precision="fp32")
    for r in range(16):
        assert _relerr(Y32[r], Y64[r]) <= 2e-6
    # once per assembly
    with pytest.raises(_capi.AhxError, match="once per assembly"):
        H.agglH(float(g["eps"]))


def test_agglomeration_save_load_and_sqntl(golden, tmp_path):
    g = golden("aggl_fib4096")
    H = A.HMatrix(g["points"], "bbx").matgenGeH_sqntl(float(g["h"]), recmpr=True, eps=float(g["eps"]))
    path = str(tmp_path / "aggl.mbls")
    H.save(path)
    # a fresh tree agglomerated the same way loads the file
    H2 = A.HMatrix(g["points"], "bbx").matgenGeH_sqntl(float(g["h"]), recmpr=True, eps=float(g["eps"]))
    H2.load(path)
    assert np.array_equal(H2.ranks(), H.ranks())
    for l in range(0, H.nleaves, 5):
        assert np.array_equal(H2.leaf_data(l), H.leaf_data(l))
