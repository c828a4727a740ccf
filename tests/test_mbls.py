"""savembls / loadmbls (Include/H.h:47-103, Include/mblock.h:737-806).

CPU: the test-side writer reproduces the reference's own file byte for byte
(SHA-256 pinned from the compiled reference on sph360), the header reader of
the C ABI, and the leaf-count check that runs before any device work.
GPU: the library's save of the reference's leaves is the reference's file,
bit for bit; loading it gives the reference's product; assemble -> save ->
load round trips exactly (also through small staging chunks); packed,
absent, corrupt and truncated records.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import ahmed_gb300 as A
from ahmed_gb300 import _capi

import mbls_format as F

HERE = os.path.dirname(os.path.abspath(__file__))
# identical leaves: the products differ only by the order of the FP64 atomic sums
TOL_SAME = 1e-14
PIN = json.load(open(os.path.join(HERE, "golden", "mbls_sph360.json")))


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def _ref_file(golden, kind, path):
    g = golden("sph360")
    F.write(path, PIN["eta"], PIN["bmin"], g[f"{kind}_leaves"], g[f"{kind}_ranks"],
            g[f"{kind}_data"], g[f"{kind}_offsets"])
    return g


@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_writer_reproduces_reference_file(golden, kind, tmp_path):
    path = str(tmp_path / "A.mbls")
    _ref_file(golden, kind, path)
    assert os.path.getsize(path) == PIN[kind]["bytes"]
    assert _sha(path) == PIN[kind]["sha256"]
    eta, bmin, recs = F.read(path)
    g = golden("sph360")
    assert (eta, bmin, len(recs)) == (PIN["eta"], PIN["bmin"], len(g[f"{kind}_ranks"]))
    offs = g[f"{kind}_offsets"]
    for l, rec in enumerate(recs):
        assert rec[3] == g[f"{kind}_ranks"][l]
        assert np.array_equal(rec[4], g[f"{kind}_data"][offs[l]:offs[l + 1]])


def test_header_reader(golden, tmp_path):
    path = str(tmp_path / "A.mbls")
    g = _ref_file(golden, "bbx", path)
    assert A.mbls_header(path) == (PIN["eta"], PIN["bmin"], len(g["bbx_ranks"]))
    with pytest.raises(_capi.AhxError):
        A.mbls_header(str(tmp_path / "missing.mbls"))
    open(tmp_path / "short.mbls", "wb").write(b"\x00" * 10)
    with pytest.raises(_capi.AhxError, match="truncated"):
        A.mbls_header(str(tmp_path / "short.mbls"))


def test_load_rejects_another_tree_before_device_work(golden, tmp_path):
    path = str(tmp_path / "A.mbls")
    g = _ref_file(golden, "bbx", path)
    H = A.HMatrix(g["points"], "bbx", bmin=24, eta=PIN["eta"])
    assert H.nleaves != len(g["bbx_ranks"])
    with pytest.raises(_capi.AhxError, match="leaves"):
        H.load(path)


# ---------------------------------------------------------------- GPU ----

def _tree(g, kind):
    return A.HMatrix(g["points"], kind, bmin=PIN["bmin"], eta=PIN["eta"])


def _relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_save_of_reference_leaves_is_reference_file(golden, kind, tmp_path):
    g = golden("sph360")
    H = _tree(g, kind)
    H.set_leaves(g[f"{kind}_ranks"], g[f"{kind}_data"], g[f"{kind}_offsets"])
    path = str(tmp_path / "ours.mbls")
    H.save(path)
    assert _sha(path) == PIN[kind]["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["bbx", "pca"])
def test_load_reference_file_gives_reference_product(golden, kind, tmp_path):
    path = str(tmp_path / "ref.mbls")
    g = _ref_file(golden, kind, path)
    H = _tree(g, kind)
    assert A.loadmbls(path, H) == (PIN["eta"], PIN["bmin"])
    assert np.array_equal(H.ranks(), g[f"{kind}_ranks"])
    offs = g[f"{kind}_offsets"]
    for l in range(0, H.nleaves, 7):
        assert np.array_equal(H.leaf_data(l), g[f"{kind}_data"][offs[l]:offs[l + 1]])
    y = H.mltaGeHVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(y, g[f"{kind}_y"]) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [None, "1000"])
def test_assemble_save_load_round_trip(golden, tmp_path, monkeypatch, chunk):
    if chunk:
        monkeypatch.setenv("AHX_IO_CHUNK", chunk)   # many staging chunks both ways
    g = golden("fib4096")
    H = A.HMatrix(g["points"], "bbx", bmin=32, eta=0.8)
    A.matgenGeH_omp(H, float(g["h"]), 1e-6)
    path = str(tmp_path / "A.mbls")
    A.savembls(0.8, 32, H, path)
    eta, bmin, recs = F.read(path)
    ranks = H.ranks()
    assert (eta, bmin) == (0.8, 32)
    assert [r[3] for r in recs] == list(ranks)
    H2 = A.HMatrix(g["points"], "bbx", bmin=32, eta=0.8)
    H2.load(path)
    assert np.array_equal(H2.ranks(), ranks)
    for l in range(H.nleaves):
        assert np.array_equal(H2.leaf_data(l), H.leaf_data(l))
    x = g["X4"]
    Y1 = H.mltaGeHVec(1.0, x, np.zeros((4, H.n)))
    Y2 = H2.mltaGeHVec(1.0, x, np.zeros((4, H.n)))
    assert _relerr(Y2, Y1) <= TOL_SAME   # same leaves; FP64 atomics order the sums
    # the reloaded arena (leaf order) saves to the same bytes
    path2 = str(tmp_path / "B.mbls")
    H2.save(path2)
    assert _sha(path2) == _sha(path)


@pytest.mark.gpu
def test_packed_and_absent_blocks(golden, tmp_path):
    g = golden("sph360")
    kind = "pca"   # sph360's PCA tree has low-rank and dense leaves (its bbx tree only dense)
    leaves, ranks = g[f"{kind}_leaves"], g[f"{kind}_ranks"]
    data, offs = g[f"{kind}_data"], g[f"{kind}_offsets"]
    diag = [l for l in range(len(ranks)) if ranks[l] < 0 and leaves[l][0] == leaves[l][2]
            and leaves[l][1] == leaves[l][3]]
    lowr = [l for l in range(len(ranks)) if ranks[l] > 0]
    assert diag and lowr
    base = _tree(g, kind)
    base.set_leaves(ranks, data, offs)
    # diagonal dense blocks of the Laplace matrix are exactly symmetric: packed loads equal
    path = str(tmp_path / "packed.mbls")
    F.write(path, 0.8, 12, leaves, ranks, data, offs, packed=diag)
    H = _tree(g, kind)
    H.load(path)
    for l in diag:
        assert np.array_equal(H.leaf_data(l), base.leaf_data(l))
    x = g["x"]
    assert _relerr(H.mltaGeHVec(1.0, x, np.zeros(H.n)), base.mltaGeHVec(1.0, x, np.zeros(H.n))) <= TOL_SAME
    # an absent block is a zero block (rank 0)
    path = str(tmp_path / "absent.mbls")
    F.write(path, 0.8, 12, leaves, ranks, data, offs, absent=[lowr[0]])
    H.load(path)
    assert H.ranks()[lowr[0]] == 0 and H.leaf_data(lowr[0]).size == 0
    zr = ranks.copy()
    zr[lowr[0]] = 0
    keep = [data[offs[l]:offs[l + 1]] if l != lowr[0] else np.zeros(0) for l in range(len(ranks))]
    zo = np.zeros(len(ranks) + 1, np.uint64)
    zo[1:] = np.cumsum([k.size for k in keep])
    ref = _tree(g, kind)
    ref.set_leaves(zr, np.concatenate(keep), zo)
    assert _relerr(H.mltaGeHVec(1.0, x, np.zeros(H.n)), ref.mltaGeHVec(1.0, x, np.zeros(H.n))) <= TOL_SAME


@pytest.mark.gpu
def test_corrupt_and_truncated_files(golden, tmp_path):
    path = str(tmp_path / "ref.mbls")
    g = _ref_file(golden, "bbx", path)
    raw = bytearray(open(path, "rb").read())
    H = _tree(g, "bbx")
    # first record's n1 (bytes 17..20) changed: the tree disagrees
    bad = bytearray(raw)
    bad[17:21] = (int.from_bytes(raw[17:21], "little") + 1).to_bytes(4, "little")
    open(tmp_path / "bad.mbls", "wb").write(bad)
    with pytest.raises(_capi.AhxError, match="block-cluster tree"):
        H.load(str(tmp_path / "bad.mbls"))
    with pytest.raises(_capi.AhxError):   # the handle is left unassembled
        H.mltaGeHVec(1.0, g["x"], np.zeros(H.n))
    open(tmp_path / "cut.mbls", "wb").write(raw[: len(raw) // 2])
    with pytest.raises(_capi.AhxError, match="truncated"):
        H.load(str(tmp_path / "cut.mbls"))
    tri = bytearray(raw)
    tri[25:29] = (2).to_bytes(4, "little")   # first record's status -> lower triangular
    open(tmp_path / "tri.mbls", "wb").write(tri)
    with pytest.raises(_capi.AhxError, match="triangular"):
        H.load(str(tmp_path / "tri.mbls"))
    H.load(path)                          # a good file after failures
    y = H.mltaGeHVec(1.0, g["x"], np.zeros(H.n))
    assert _relerr(y, g["bbx_y"]) <= 1e-12
