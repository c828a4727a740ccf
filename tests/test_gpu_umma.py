"""The FP32 product on the fifth-generation tensor cores (tcgen05.mma, TMEM
accumulators; ahmed_gb300/csrc/ahx_matvec_umma.cu) through the C ABI.

Semantics: mltaGeHGeM (H/mltaGeHVec.cpp:38-59) over FP32 copies of the leaves.
Each case compares, per right-hand side, with the FP64 product of the same
leaves (error <= 2e-6 relative, the FP32 bar of this library) and with the
oracle's product of the reference's algorithm.  Cases cover the right-hand-side
passes (P = 16, 32, 64 and more than 64), both cluster trees, the V tiles split
along K (a small piece length, their pieces adding into zeroed T rows), leading
dimensions larger than n, accumulation into a non-zero Y with a scale d, and
the sweep timing instrumentation.
"""
import numpy as np
import pytest

import ahmed_gb300 as A
import oracle as O
from ahmed_gb300 import _capi

pytestmark = pytest.mark.gpu

TOL_FP32 = 2e-6


def _relerr_rows(a, b):
    return (np.linalg.norm(a - b, axis=-1) / np.linalg.norm(b, axis=-1)).max()


@pytest.fixture(scope="module")
def fib(golden):
    g = golden("fib4096")
    H = A.HMatrix(g["points"], "bbx", bmin=32, eta=0.8)
    H.matgenGeH_omp(float(g["h"]), 1e-6)
    return g, H


@pytest.mark.parametrize("p", [2, 5, 16, 17, 33, 64, 70])
def test_fp32_tcgen05_product_per_rhs(fib, p):
    g, H = fib
    X = np.random.default_rng(p).uniform(-1, 1, (p, H.n))
    Y64 = H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp64")
    Y32 = H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp32")
    assert _relerr_rows(Y32, Y64) <= TOL_FP32


def test_fp32_tcgen05_matches_oracle_and_accumulates(golden):
    g = golden("cube3000")
    Ho = O.OracleH(g["points"], O.TREE_PCA, 32, 0.8, float(g["h"]))
    Ho.assemble(1e-6, nthreads=4)
    H = A.HMatrix(g["points"], "pca", bmin=32, eta=0.8)
    chunks = [Ho.leaf_data(l) for l in range(Ho.nleaves)]
    offs = np.zeros(len(chunks) + 1, np.uint64)
    offs[1:] = np.cumsum([c.size for c in chunks])
    H.set_leaves(Ho.ranks(), np.concatenate(chunks), offs)
    n, p = H.n, 24
    X = np.random.default_rng(7).uniform(-1, 1, (p, n))
    Y0 = np.random.default_rng(8).uniform(-1, 1, (p, n))
    Yo = Ho.matvec(X, Y0.copy(), d=-0.75)
    # leading dimensions larger than n, through the C ABI
    ld = n + 5
    Xl = np.zeros((p, ld))
    Xl[:, :n] = X
    Yl = np.zeros((p, ld))
    Yl[:, :n] = Y0
    _capi.check(_capi.lib().ahx_matvec(H.handle, 1, -0.75, p, Xl.ctypes.data, ld, Yl.ctypes.data, ld))
    assert _relerr_rows(Yl[:, :n], Yo) <= TOL_FP32
    assert np.array_equal(Yl[:, n:], np.zeros((p, 5)))


def test_fp32_tcgen05_split_v_tiles(golden, monkeypatch):
    """V tiles split along K into 32-row pieces add into zeroed T rows."""
    monkeypatch.setenv("AHX_UM_KPIECE", "32")
    g = golden("fib4096")
    H = A.HMatrix(g["points"], "bbx", bmin=32, eta=0.8)
    H.matgenGeH_omp(float(g["h"]), 1e-6)
    X = np.random.default_rng(11).uniform(-1, 1, (64, H.n))
    Y64 = H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp64")
    for _ in range(2):  # the zeroed rows are zeroed again on every product
        Y32 = H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp32")
        assert _relerr_rows(Y32, Y64) <= TOL_FP32


def test_sweep_timing_counts_launches(fib):
    g, H = fib
    L = _capi.lib()
    X = np.random.default_rng(1).uniform(-1, 1, (16, H.n))
    H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp32")
    ms = np.zeros(2)
    cnt = np.zeros(2, np.uint64)
    L.ahx_timing_read(ms.ctypes.data, cnt.ctypes.data, 1)
    L.ahx_timing(1)
    try:
        for _ in range(3):
            H.mltaGeHVec(1.0, X, np.zeros_like(X), precision="fp32")
        L.ahx_timing_read(ms.ctypes.data, cnt.ctypes.data, 1)
    finally:
        L.ahx_timing(0)
    assert list(cnt) == [3, 3]
    assert ms[0] > 0 and ms[1] > 0
