"""ahx_aca_block_noalloc: ACA of one block with no device allocation.

The entry point serves callers that cannot call cudaMalloc themselves -- for
example code running while a framework's caching allocator holds the device
memory, or hosts that own every device allocation and only lend buffers.  It
runs the same ACA + recompression kernel code as ahx_assemble with its
scratch in a fixed array inside the library.  This test calls it through the
C ABI twice in a row (a CTA-sized block, then a warp-sized block, then the
first block again) and checks each result against the regular assembly's
leaf: same ranks, product U V^T within 1e-12.  The file is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

pytestmark = pytest.mark.gpu

KMAX = 64


def _scratch_bytes(n1, n2, kmax):
    c = kmax + 1  # ACA column capacity: the reference allocates kmax + 1 columns
    return 256 + 8 * (2 * (n1 + n2) * c + 2 * c * c + 3 * c) + 4 * (n1 + n2)


def _noalloc(torch, pts_dev, leaf, h, eps):
    b1, n1, b2, n2, _, _, i0 = (int(v) for v in leaf)
    dev = pts_dev[0].device
    U = torch.full((n1 * KMAX,), float("nan"), dtype=torch.float64, device=dev)
    V = torch.full((n2 * KMAX,), float("nan"), dtype=torch.float64, device=dev)
    info = torch.full((3,), -7, dtype=torch.int32, device=dev)
    rc = _capi.lib().ahx_aca_block_noalloc(
        C.c_void_p(pts_dev[0].data_ptr()), C.c_void_p(pts_dev[1].data_ptr()),
        C.c_void_p(pts_dev[2].data_ptr()), b1, n1, b2, n2, i0, h, eps, KMAX,
        C.c_void_p(U.data_ptr()), C.c_void_p(V.data_ptr()), C.c_void_p(info.data_ptr()), None)
    assert rc == _capi.AHX_OK, _capi.lib().ahx_last_error()
    torch.cuda.synchronize()
    st, kaca, kt = (int(v) for v in info.cpu())
    return st, kaca, kt, U[: n1 * kt].cpu().numpy(), V[: n2 * kt].cpu().numpy()


def _product(U, V, n1, n2, k):
    return U.reshape(k, n1).T @ V.reshape(k, n2)


def test_noalloc_matches_assembly_two_calls_in_a_row(golden):
    torch = pytest.importorskip("torch")
    g = golden("fib4096")
    h, eps = float(g["h"]), float(g["eps"])
    H = A.HMatrix(g["points"], "pca", bmin=int(g["bmin"]), eta=float(g["eta"]))
    H.matgenGeH_omp(h, eps)
    lv, ranks, aranks = H.leaves(), H.ranks(), H.aca_ranks()
    op, _ = H.perm()
    P = g["points"][op]
    pts = [torch.from_numpy(np.ascontiguousarray(P[:, j])).cuda() for j in range(3)]
    size = np.maximum(lv[:, 1], lv[:, 3]).astype(np.int64)
    fits = np.array([_scratch_bytes(int(a), int(b), KMAX) <= (8 << 20) for a, b in lv[:, [1, 3]]])
    ok = (lv[:, 4] == 1) & (ranks > 0) & (aranks < KMAX) & fits
    large = [l for l in np.nonzero(ok & (size > 256))[0]]
    small = [l for l in np.nonzero(ok & (size <= 256))[0]]
    assert large and small
    big = large[int(np.argmax(size[large]))]
    little = small[len(small) // 2]
    first = None
    for l in (big, little, big):
        st, kaca, kt, U, V = _noalloc(torch, pts, lv[l], h, eps)
        n1, n2 = int(lv[l, 1]), int(lv[l, 3])
        assert st == 1
        assert kaca == aranks[l] and kt == ranks[l]
        ref = H.leaf_data(l)
        k = int(ranks[l])
        Aref = _product(ref[: n1 * k], ref[n1 * k:], n1, n2, k)
        Anew = _product(U, V, n1, n2, kt)
        assert np.linalg.norm(Anew - Aref) <= 1e-12 * np.linalg.norm(Aref)
        if l == big:
            if first is None:
                first = (U.copy(), V.copy())
            else:
                assert np.array_equal(U, first[0]) and np.array_equal(V, first[1])


def test_noalloc_rejects_blocks_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    info = torch.zeros(3, dtype=torch.int32, device="cuda")
    p = C.c_void_p(x.data_ptr())
    rc = _capi.lib().ahx_aca_block_noalloc(p, p, p, 0, 200000, 0, 200000, 0, 0.1, 1e-6, 1000,
                                           C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()),
                                           C.c_void_p(info.data_ptr()), None)
    assert rc == _capi.AHX_ERR_ARG
    assert b"scratch" in _capi.lib().ahx_last_error()
    # sizes whose n1 + n2 wraps 32 bits are refused too, before any size arithmetic
    for n1, n2, kmax in ((1 << 31, 1 << 31, 4), (100, 100, 1 << 20)):
        rc = _capi.lib().ahx_aca_block_noalloc(p, p, p, 0, n1, 0, n2, 0, 0.1, 1e-6, kmax,
                                               C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()),
                                               C.c_void_p(info.data_ptr()), None)
        assert rc == _capi.AHX_ERR_ARG
        assert b"scratch" in _capi.lib().ahx_last_error()
