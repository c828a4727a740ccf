"""Host checks of the tensor-core product's layout (no GPU): the tiles of the
V sweep and the rows sweep, their entries and Z-row indices, evaluated on the
host exactly as the sweeps combine them, reproduce the oracle's product
(H/mltaGeHVec.cpp:38-59 via mltaLrMGeM_ / mltaGeMGeM, H/mblock.cpp:141-154).
A small piece length forces V tiles split along K (their pieces add into
zeroed T rows)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ahmed_gb300 import _capi


def _leafset(Ho):
    lv = Ho.leaves()
    ranks = Ho.ranks()
    offs, parts, words = [], [], []
    off = 0
    for l in range(len(lv)):
        d = Ho.leaf_data(l)
        offs.append(off)
        parts.append(d)
        off += d.size
        words.append([lv[l, 0], lv[l, 1], lv[l, 2], lv[l, 3], np.uint32(np.int32(ranks[l]).view(np.uint32))])
    arena = np.concatenate(parts) if parts else np.zeros(1)
    return (np.ascontiguousarray(np.array(words, dtype=np.uint32)), np.array(offs, dtype=np.uint64),
            np.ascontiguousarray(arena))


@pytest.mark.parametrize("case,kpiece", [("fib4096", 4096), ("fib4096", 32), ("cube3000", 64), ("sph360", 0)])
def test_um_layout_reproduces_oracle_product(golden, case, kpiece):
    g = golden(case)
    Ho = O.OracleH(g["points"], O.TREE_BBX, 32, 0.8, float(g["h"]))
    Ho.assemble(1e-6, nthreads=4)
    words, offs, arena = _leafset(Ho)
    n = Ho.n
    p = 5
    X = np.random.default_rng(3).uniform(-1, 1, (p, n))
    Yo = Ho.matvec(X, np.zeros_like(X))
    Y = np.zeros((p, n))
    info = np.zeros(4, np.uint64)
    f = _capi.lib().ahx_um_host_product
    f.restype = C.c_int
    f.argtypes = [C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_uint32]
    rc = f(n, len(words), words.ctypes.data, offs.ctypes.data, arena.ctypes.data, p, X.ctypes.data, Y.ctypes.data,
           info.ctypes.data, kpiece)
    assert rc == 0
    err = np.linalg.norm(Y - Yo) / np.linalg.norm(Yo)
    assert err < 1e-13, err
    assert info[1] > 0 and info[3] > 0
