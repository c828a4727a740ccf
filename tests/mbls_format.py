"""Test-side restatement of the reference's savembls / loadmbls byte layout.

Follows Include/H.h:47-103 (savembls / loadmbls) and Include/mblock.h:737-806
(mblock::save / load): double eta, uint32 bmin, uint32 nleaves, then per leaf
uint8 present; if present uint32 n1, n2, status and
  status 0: uint32 rank, rank*(n1+n2) doubles;  status 4: n1*n2 doubles;
  status 1 / 5: n1*(n1+1)/2 doubles (packed upper triangle by columns).
Pinned by tests/golden/mbls_sph360.json (SHA-256 of the reference's own file).
Only the tests use it, to write reference-layout files and their variants.
"""
import struct

import numpy as np

LOWRANK, HERM, LOWER, UPPER, DENSE, SYM = 0, 1, 2, 3, 4, 5


def write(path, eta, bmin, leaves, ranks, data, offsets, packed=(), absent=()):
    """leaves: (nleaves, 7) [b1, n1, b2, n2, adm, idx, i0]; ranks[l] (-1 dense);
    packed: leaves written as status-5 packed blocks; absent: leaves written as absent."""
    packed, absent = set(packed), set(absent)
    with open(path, "wb") as f:
        f.write(struct.pack("<dII", eta, bmin, len(ranks)))
        for l, r in enumerate(ranks):
            if l in absent:
                f.write(b"\x00")
                continue
            n1, n2 = int(leaves[l][1]), int(leaves[l][3])
            d = np.asarray(data[int(offsets[l]):int(offsets[l + 1])], np.float64)
            f.write(b"\x01" + struct.pack("<II", n1, n2))
            if r >= 0:
                f.write(struct.pack("<II", LOWRANK, int(r)))
                f.write(d.tobytes())
            elif l in packed:
                assert n1 == n2
                D = d.reshape(n2, n1).T
                col = [D[:j + 1, j] for j in range(n1)]
                f.write(struct.pack("<I", SYM))
                f.write(np.concatenate(col).tobytes())
            else:
                f.write(struct.pack("<I", DENSE))
                f.write(d.tobytes())


def read(path, dtype=np.float64):
    """Returns (eta, bmin, records); record = None (absent) or (n1, n2, status, rank, data).
    dtype: the leaves' element type (np.complex128 for mblock<dcomp>)."""
    raw = open(path, "rb").read()
    esz = np.dtype(dtype).itemsize
    eta, bmin, n = struct.unpack_from("<dII", raw, 0)
    pos = 16
    recs = []
    for _ in range(n):
        present = raw[pos]
        pos += 1
        if not present:
            recs.append(None)
            continue
        n1, n2, status = struct.unpack_from("<III", raw, pos)
        pos += 12
        rank = -1
        if status == LOWRANK:
            (rank,) = struct.unpack_from("<I", raw, pos)
            pos += 4
            cnt = rank * (n1 + n2)
        elif status == DENSE:
            cnt = n1 * n2
        else:
            cnt = n1 * (n1 + 1) // 2
        d = np.frombuffer(raw, dtype, cnt, pos)
        pos += esz * cnt
        recs.append((n1, n2, status, rank, d))
    return eta, bmin, recs
