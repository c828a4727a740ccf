"""savembls / loadmbls of the Helmholtz leaves (mblock<dcomp>: Include/H.h:47-103,
Include/mblock.h:737-806 with T = dcomp).

The fixture (tests/golden/make_golden.py zmbls) holds the reference's own files
for a 200-point sphere on PCA trees, general and symmetric (status-5 SyM
diagonal blocks).  CPU: the files parse into the leaves of this library's
trees and their blocks are the Helmholtz matrix's.  GPU: loading a file gives
its leaves bit for bit and the matrix's product, saving them again gives the
reference's file byte for byte, and assemble -> save -> load round trips."""
import hashlib
import os

import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

import mbls_format as F

TAGS = ["gen", "sym"]


def _file(golden, tag, tmp_path):
    g = golden("zmbls_sph200")
    path = str(tmp_path / f"ref_{tag}.mbls")
    g[f"{tag}_file"].tofile(path)
    return g, path


def _dense(g, perm):
    P = g["points"][perm]
    D = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, float(g["h"]))
    return np.exp(1j * float(g["k"]) * D) / (4.0 * np.pi * D)


def _hmat(g, tag):
    return A.HMatrix(g["points"], "pca", bmin=int(g["bmin"]), eta=float(g["eta"]), symmetric=tag == "sym")


@pytest.mark.parametrize("tag", TAGS)
def test_reference_file_parses_into_the_tree(golden, tag, tmp_path):
    g, path = _file(golden, tag, tmp_path)
    eta, bmin, recs = F.read(path, np.complex128)
    assert eta == float(g["eta"]) and bmin == int(g["bmin"])
    H = _hmat(g, tag)
    L = H.leaves()
    np.testing.assert_array_equal(L, g[f"{tag}_leaves"])
    np.testing.assert_array_equal(H.perm()[0], g[f"{tag}_op_perm"])
    M = _dense(g, g[f"{tag}_op_perm"])
    ranks = g[f"{tag}_ranks"]
    assert len(recs) == len(L)
    for l, (n1, n2, status, rank, d) in enumerate(recs):
        b1, b2 = int(L[l, 0]), int(L[l, 2])
        assert (n1, n2) == (int(L[l, 1]), int(L[l, 3]))
        blk = M[b1:b1 + n1, b2:b2 + n2]
        if status == F.LOWRANK:
            assert rank == ranks[l]
            U = d[:n1 * rank].reshape(rank, n1).T
            V = d[n1 * rank:].reshape(rank, n2).T
            assert np.linalg.norm(U @ V.conj().T - blk) <= 2e-5 * np.linalg.norm(blk)
        elif status == F.SYM:
            assert tag == "sym" and b1 == b2 and ranks[l] == -1
            want = np.concatenate([blk[:j + 1, j] for j in range(n1)])
            assert np.abs(d - want).max() <= 1e-14 * np.abs(want).max()
        else:
            assert status == F.DENSE and ranks[l] == -1
            assert np.abs(d.reshape(n2, n1).T - blk).max() <= 1e-14 * np.abs(blk).max()
    assert any(r[2] == F.SYM for r in recs) == (tag == "sym")
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
def test_load_reference_file_and_save_it_back(golden, tag, tmp_path):
    g, path = _file(golden, tag, tmp_path)
    H = _hmat(g, tag)
    eta, bmin = H.helm_load(path)
    assert eta == float(g["eta"]) and bmin == int(g["bmin"])
    np.testing.assert_array_equal(H.helm_ranks(), g[f"{tag}_ranks"])
    _, _, recs = F.read(path, np.complex128)
    for l, rec in enumerate(recs):
        np.testing.assert_array_equal(H.helm_leaf_data(l), rec[4])  # bit for bit
    M = _dense(g, g[f"{tag}_op_perm"])
    x = np.random.default_rng(4).standard_normal(H.n) + 1j * np.random.default_rng(5).standard_normal(H.n)
    y = np.zeros(H.n, np.complex128)
    H.mltaGeHVec(1.0, x, y)
    assert np.linalg.norm(y - M @ x) <= 5e-6 * np.linalg.norm(M @ x)
    out = str(tmp_path / "again.mbls")
    H.helm_save(out, eta, bmin)
    assert hashlib.sha256(open(out, "rb").read()).digest() == hashlib.sha256(open(path, "rb").read()).digest()
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("chunk", [None, "7"])
def test_assemble_save_load_round_trip(golden, tag, chunk, tmp_path, monkeypatch):
    g = golden("zmbls_sph200")
    if chunk:
        monkeypatch.setenv("AHX_IO_CHUNK", chunk)  # doubles per staging chunk
    H = _hmat(g, tag).helmholtz_assemble(float(g["k"]), float(g["h"]), float(g["eps"]))
    path = str(tmp_path / "mine.mbls")
    H.helm_save(path)
    G = _hmat(g, tag)
    G.helm_load(path)
    np.testing.assert_array_equal(G.helm_ranks(), H.helm_ranks())
    for l in range(H.nleaves):
        np.testing.assert_array_equal(G.helm_leaf_data(l), H.helm_leaf_data(l))
    X = np.random.default_rng(6).standard_normal((3, H.n)) + 1j * np.random.default_rng(7).standard_normal((3, H.n))
    Y1 = np.zeros_like(X)
    Y2 = np.zeros_like(X)
    H.mltaGeHVec(0.3 - 1j, X, Y1)
    G.mltaGeHVec(0.3 - 1j, X, Y2)
    assert np.linalg.norm(Y1 - Y2) <= 1e-14 * np.linalg.norm(Y1)
    H.close()
    G.close()


@pytest.mark.parametrize("tag", TAGS)
def test_header_of_complex_file(golden, tag, tmp_path):
    """ahx_mbls_header reads the common header of a complex file (host only), so the
    tree can be built before the leaves are loaded."""
    g, path = _file(golden, tag, tmp_path)
    eta, bmin, n = A.mbls_header(path)
    assert eta == float(g["eta"]) and bmin == int(g["bmin"]) and n == len(g[f"{tag}_leaves"])
    # a tree with another leaf count is refused before any device work
    H = A.HMatrix(g["points"], "bbx", bmin=int(g["bmin"]), eta=float(g["eta"]))
    if H.nleaves != n:
        with pytest.raises(_capi.AhxError, match="leaves"):
            H.helm_load(path)
    H.close()
