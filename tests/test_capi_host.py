"""Host-side checks of libahx that need no GPU: exports, trees, permutations, h."""
import os
import re

import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["fib4096", "cube3000", "ell2500", "sph360", "fib50"]


def _declared():
    src = open(os.path.join(ROOT, "include", "ahx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ahx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _capi.lib()
    names = _declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    bound = {s[0] for s in _capi.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_version_and_error_channel():
    assert _capi.lib().ahx_version() >= 10000
    with pytest.raises(_capi.AhxError):
        A.HMatrix(np.zeros((0, 3)))


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_product_tree_matches_reference(golden, case, kind):
    g = golden(case)
    H = A.HMatrix(g["points"], kind, bmin=int(g["bmin"]), eta=float(g["eta"]))
    op, po = H.perm()
    assert np.array_equal(op, g[f"{kind}_op_perm"])
    assert np.array_equal(po, g[f"{kind}_po_perm"])
    assert np.array_equal(H.leaves(), g[f"{kind}_leaves"])


def test_mean_nn_matches_oracle_bitwise(golden):
    for case in ("fib4096", "cube3000", "ell2500"):
        g = golden(case)
        assert A.mean_nn(g["points"]) == float(g["h"])


def test_leaf_list_is_a_partition():
    """Every (row, col) pair of the matrix is covered by exactly one leaf."""
    P = A.geometry.cube_surface(1500, 3)
    for kind in ("bbx", "pca"):
        H = A.HMatrix(P, kind, bmin=16)
        lv = H.leaves().astype(np.int64)
        cover = np.zeros((H.n, H.n), np.int8)
        for b1, n1, b2, n2 in lv[:, :4]:
            cover[b1:b1 + n1, b2:b2 + n2] += 1
        assert (cover == 1).all()
        assert np.array_equal(lv[:, 5], np.arange(len(lv)))


def test_helmholtz_calls_before_assembly_fail_on_the_host(tmp_path):
    """The Helmholtz entry points check arguments and state before any device work,
    so a handle without assembled complex leaves gets status codes, not faults."""
    L = _capi.lib()
    P = A.geometry.fibonacci_sphere(512)
    H = A.HMatrix(P, "bbx", bmin=32, eta=0.8)
    h, n = H.handle, H.n
    X = np.zeros(n, np.complex128)
    Y = np.zeros(n, np.complex128)
    ptr = _capi.ptr
    ranks = np.zeros(H.nleaves, np.int32)
    assert L.ahx_helm_ranks(h, ptr(ranks)) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_leaf_size(h, 0) == 0
    assert L.ahx_helm_get_leaf(h, 0, ptr(X)) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_get_leaf(h, H.nleaves, ptr(X)) == _capi.AHX_ERR_ARG
    assert L.ahx_helm_storage_bytes(h, 0) == 0
    assert L.ahx_helm_matvec(h, 0, 0, 1.0, 0.0, 1, ptr(X), n, ptr(Y), n) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_matvec(h, 0, 0, 1.0, 0.0, 1, ptr(X), n - 1, ptr(Y), n) == _capi.AHX_ERR_ARG
    assert L.ahx_helm_matvec(h, 0, 7, 1.0, 0.0, 1, ptr(X), n, ptr(Y), n) == _capi.AHX_ERR_ARG
    its = np.zeros(1, np.uint32)
    res = np.zeros(1)
    assert L.ahx_helm_gmres(h, 0, 1, ptr(X), n, ptr(Y), n, 1e-8, 10, 10, ptr(its), ptr(res)) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_gmres(h, 0, 1, ptr(X), n, ptr(Y), n, 1e-8, 0, 10, ptr(its), ptr(res)) == _capi.AHX_ERR_ARG
    assert L.ahx_helm_save(h, 0.8, 32, os.fsencode(str(tmp_path / "z.mbls"))) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_agglomerate(h, 1e-6, 2**32 - 1, None) == _capi.AHX_ERR_STATE
    assert L.ahx_helm_assemble(h, 5.0, 0.0, 1e-6, 2**32 - 1) == _capi.AHX_ERR_ARG
    assert L.ahx_helm_assemble(h, 5.0, 0.05, -1.0, 2**32 - 1) == _capi.AHX_ERR_ARG
    assert L.ahx_helm_load(h, os.fsencode(str(tmp_path / "missing.mbls")), None, None) == _capi.AHX_ERR_ARG
    H.close()


def test_python_mirror_dispatches_by_element_type(monkeypatch):
    """Complex arrays go to the Helmholtz entry points (the reference's dcomp overloads),
    real ones to the real leaves: A, A^H, A^T and GMRes (a recording stand-in for the
    library, no device work)."""
    from ahmed_gb300 import hmatrix as HM

    P = A.geometry.fibonacci_sphere(256)
    H = A.HMatrix(P, "bbx", bmin=32, eta=0.8)
    calls = []

    class Rec:
        def __getattr__(self, name):
            def f(*args):
                calls.append((name, args[2] if name == "ahx_helm_matvec" else None))
                return 0
            return f

    monkeypatch.setattr(HM, "lib", lambda: Rec())
    n = H.n
    z = np.zeros(n, np.complex128)
    r = np.zeros(n)
    H.mltaGeHVec(1.0, z, z.copy())
    H.mltaGeHhVec(1.0, z, z.copy())
    H.mltaGeHtVec(1.0, z, z.copy())
    H.mltaSyHVec(1.0, z, z.copy())
    H.mltaGeHVec(1.0, r, r.copy())
    H.mltaGeHhVec(1.0, r, r.copy())
    H.GMRes(z, z.copy(), 1e-8, 10, 10)
    H.GMRes(r, r.copy(), 1e-8, 10, 10)
    assert calls == [("ahx_helm_matvec", 0), ("ahx_helm_matvec", 1), ("ahx_helm_matvec", 2),
                     ("ahx_helm_matvec", 0), ("ahx_matvec", None), ("ahx_matvec_transposed", None),
                     ("ahx_helm_gmres", None), ("ahx_gmres", None)]
    monkeypatch.undo()
    H.close()


def test_noalloc_refuses_oversized_blocks_before_device_work():
    """Sizes whose n1 + n2 wraps 32 bits, or rank bounds beyond the fixed scratch
    array, are refused with AHX_ERR_ARG before any CUDA call (no GPU needed)."""
    import ctypes as C

    L = _capi.lib()
    fake = C.c_void_p(0x1000)  # never dereferenced: the call returns first
    for n1, n2, kmax in ((1 << 31, 1 << 31, 4), (100, 100, 1 << 20), (3000, 3000, 500)):
        rc = L.ahx_aca_block_noalloc(fake, fake, fake, 0, n1, 0, n2, 0, 0.1, 1e-6, kmax, fake, fake, fake, None)
        assert rc == _capi.AHX_ERR_ARG
        assert b"scratch" in L.ahx_last_error()


@pytest.mark.parametrize("case", ["sphere65536-leaf32", "cube1048576-leaf64"])
def test_trees_at_benchmark_sizes_match_oracle(case):
    """The block-cluster trees of the benchmarked workloads (Fibonacci sphere N =
    65,536 with leaf 32; uniform cube surface N = 2^20, seed 4, with leaf 64;
    bounding-box bisection, eta 0.8) equal the oracle's bit for bit: both
    permutations and the DFS leaf list (Include/cluster_bbx.h:100-128,
    cluster/blcluster.cpp:40-66).  The oracle's trees are pinned to the
    reference's own on the golden cases."""
    import oracle as O

    if case.startswith("sphere"):
        P, leaf = A.geometry.fibonacci_sphere(65536), 32
    else:
        P, leaf = A.geometry.cube_surface(1 << 20, 4), 64
    H = A.HMatrix(P, "bbx", bmin=leaf, eta=0.8)
    Ho = O.OracleH(P, O.TREE_BBX, leaf, 0.8, 1.0)
    op, po = H.perm()
    oo, opo = Ho.perm()
    assert np.array_equal(op, oo) and np.array_equal(po, opo)
    assert np.array_equal(H.leaves(), Ho.leaves())
    if case.startswith("sphere"):
        Hp = A.HMatrix(P, "pca", bmin=leaf, eta=0.8)
        Hpo = O.OracleH(P, O.TREE_PCA, leaf, 0.8, 1.0)
        assert np.array_equal(Hp.perm()[0], Hpo.perm()[0])
        assert np.array_equal(Hp.leaves(), Hpo.leaves())
