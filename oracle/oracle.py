"""ctypes wrapper of the CPU oracle (oracle/oracle.c) -- test infrastructure.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module, always as the checker.  It also wraps the reference build
(``oracle/_ref/libahmed_ref.so``) where that exists (x86 container only).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libahmed_ref.so")

TREE_BBX = 0
TREE_PCA = 1

_lib = None
_ref = None


def build():
    subprocess.check_call(["bash", os.path.join(HERE, "build_oracle.sh")])


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, u32, i32, dbl = C.c_void_p, C.c_uint32, C.c_int, C.c_double
        L.or_build.restype = vp
        L.or_build.argtypes = [vp, u32, i32, u32, dbl]
        L.or_free.argtypes = [vp]
        L.or_nleaves.restype = u32
        L.or_nleaves.argtypes = [vp]
        L.or_perm.argtypes = [vp, vp, vp]
        L.or_leaves.argtypes = [vp, vp]
        L.or_mean_nn.restype = dbl
        L.or_mean_nn.argtypes = [vp, u32]
        L.or_entry.restype = dbl
        L.or_entry.argtypes = [vp, dbl, u32, u32]
        L.or_assemble.argtypes = [vp, dbl, dbl, u32, i32]
        L.or_assemble_range.argtypes = [vp, dbl, dbl, u32, i32, u32, u32]
        L.or_ranks.argtypes = [vp, vp]
        L.or_aca_ranks.argtypes = [vp, vp]
        L.or_leaf_data.restype = C.c_uint64
        L.or_leaf_data.argtypes = [vp, u32, vp]
        L.or_set_leaf.argtypes = [vp, u32, C.c_int32, vp]
        L.or_matvec.argtypes = [vp, dbl, u32, vp, vp, i32]
        L.or_gmres.restype = u32
        L.or_gmres.argtypes = [vp, vp, vp, vp, u32, vp, i32]
        L.or_cg.restype = u32
        L.or_cg.argtypes = [vp, vp, vp, vp, vp, i32]
        L.or_aca_block.restype = i32
        L.or_aca_block.argtypes = [vp, dbl, u32, u32, u32, u32, dbl, u32, u32, vp, vp, vp]
        L.or_recompress.restype = u32
        L.or_recompress.argtypes = [u32, u32, u32, vp, vp, dbl, u32]
        _lib = L
    return _lib


def mean_nn(pts):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    return lib().or_mean_nn(_p(pts), pts.shape[0])


class OracleH:
    """H-matrix of the Laplace collocation generator, built and assembled on the CPU."""

    def __init__(self, pts, kind=TREE_BBX, bmin=32, eta=0.8, h=None):
        self.pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.n = self.pts.shape[0]
        self.kind = kind
        self.h = mean_nn(self.pts) if h is None else float(h)
        self._H = lib().or_build(_p(self.pts), self.n, kind, bmin, eta * eta)

    def __del__(self):
        if getattr(self, "_H", None) and _lib is not None:
            _lib.or_free(self._H)
            self._H = None

    @property
    def nleaves(self):
        return lib().or_nleaves(self._H)

    def perm(self):
        op = np.zeros(self.n, np.uint32)
        po = np.zeros(self.n, np.uint32)
        lib().or_perm(self._H, _p(op), _p(po))
        return op, po

    def leaves(self):
        out = np.zeros((self.nleaves, 7), np.uint32)
        lib().or_leaves(self._H, _p(out))
        return out

    def assemble(self, eps=1e-6, rankmax=2**31, nthreads=0, leaf_range=None):
        if leaf_range is None:
            lib().or_assemble(self._H, self.h, eps, min(rankmax, 2**32 - 1), nthreads)
        else:
            lib().or_assemble_range(self._H, self.h, eps, min(rankmax, 2**32 - 1), nthreads,
                                    leaf_range[0], leaf_range[1])

    def ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        lib().or_ranks(self._H, _p(out))
        return out

    def aca_ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        lib().or_aca_ranks(self._H, _p(out))
        return out

    def leaf_data(self, l):
        cnt = lib().or_leaf_data(self._H, l, None)
        out = np.zeros(cnt, np.float64)
        lib().or_leaf_data(self._H, l, _p(out))
        return out

    def set_leaf(self, l, rank, data):
        data = np.ascontiguousarray(data, dtype=np.float64)
        lib().or_set_leaf(self._H, l, int(rank), _p(data))

    def entry(self, i, j):
        return lib().or_entry(self._H, self.h, i, j)

    def matvec(self, X, Y, d=1.0, nthreads=0):
        """Y += d A X for X, Y of shape (n,) or (p, n) (rows are right-hand sides)."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        assert Y.flags.c_contiguous and Y.dtype == np.float64
        p = 1 if X.ndim == 1 else X.shape[0]
        lib().or_matvec(self._H, d, p, _p(X), _p(Y), nthreads)
        return Y

    def gmres(self, b, x, eps, m, nsteps, nthreads=0):
        b = np.ascontiguousarray(b, dtype=np.float64)
        e = C.c_double(eps)
        ns = C.c_uint32(nsteps)
        r = lib().or_gmres(self._H, _p(b), _p(x), C.byref(e), m, C.byref(ns), nthreads)
        return r, e.value, ns.value

    def cg(self, b, x, eps, nsteps, nthreads=0):
        b = np.ascontiguousarray(b, dtype=np.float64)
        e = C.c_double(eps)
        ns = C.c_uint32(nsteps)
        r = lib().or_cg(self._H, _p(b), _p(x), C.byref(e), C.byref(ns), nthreads)
        return r, e.value, ns.value

    def dense(self):
        """Full matrix in permuted order (small n only)."""
        op, _ = self.perm()
        P = self.pts[op]
        dx = P[:, None, 0] - P[None, :, 0]
        dy = P[:, None, 1] - P[None, :, 1]
        dz = P[:, None, 2] - P[None, :, 2]
        D = np.sqrt((dx * dx + dy * dy) + dz * dz)  # same rounding as or_entry
        np.fill_diagonal(D, self.h)
        return 1.0 / ((4.0 * np.pi) * D)


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    """The reference library compiled from its own sources (oracle/ref/build_ref.sh)."""
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        vp, u32, i32, dbl = C.c_void_p, C.c_uint, C.c_int, C.c_double
        L.ref_build.restype = vp
        L.ref_build.argtypes = [vp, u32, i32, u32, dbl, dbl]
        L.ref_build_sym.restype = vp
        L.ref_build_sym.argtypes = [vp, u32, i32, u32, dbl, dbl]
        L.ref_nleaves.restype = u32
        L.ref_nleaves.argtypes = [vp]
        L.ref_perm.argtypes = [vp, vp, vp]
        L.ref_leaves.argtypes = [vp, vp]
        L.ref_assemble.argtypes = [vp, dbl, u32, i32]
        L.ref_ranks.argtypes = [vp, vp]
        L.ref_leaf_data.restype = C.c_ulong
        L.ref_leaf_data.argtypes = [vp, u32, vp]
        L.ref_matvec.argtypes = [vp, dbl, u32, vp, vp]
        L.ref_gmres.restype = u32
        L.ref_gmres.argtypes = [vp, vp, vp, vp, u32, vp]
        L.ref_cg.restype = u32
        L.ref_cg.argtypes = [vp, vp, vp, vp, vp]
        L.ref_entry.restype = dbl
        L.ref_entry.argtypes = [vp, u32, u32]
        L.ref_free.argtypes = [vp]
        L.ref_helm_ranks.argtypes = [vp, dbl, dbl, dbl, u32, vp]
        L.ref_agglomerate.argtypes = [vp, dbl, u32]
        L.ref_save.restype = i32
        L.ref_save.argtypes = [vp, dbl, u32, C.c_char_p]
        L.ref_helm_assemble.argtypes = [vp, dbl, dbl, dbl, u32, i32]
        L.ref_helm_ranks_assembled.argtypes = [vp, vp]
        L.ref_helm_leaf_data.restype = C.c_ulong
        L.ref_helm_leaf_data.argtypes = [vp, u32, vp]
        L.ref_helm_matvec.argtypes = [vp, i32, dbl, dbl, u32, vp, vp]
        L.ref_helm_agglomerate.argtypes = [vp, dbl, u32]
        L.ref_helm_save.restype = i32
        L.ref_helm_save.argtypes = [vp, dbl, u32, C.c_char_p]
        L.ref_helm_gmres.restype = u32
        L.ref_helm_gmres.argtypes = [vp, vp, vp, vp, u32, vp]
        _ref = L
    return _ref


class RefH:
    """The reference library's own H-matrix (x86 container only)."""

    def __init__(self, pts, kind, bmin, eta, h, sym=False):
        """sym: the symmetric block tree (subdivide_sym), HeH assembly and product."""
        self.pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.n = self.pts.shape[0]
        build = ref().ref_build_sym if sym else ref().ref_build
        self._H = build(_p(self.pts), self.n, kind, bmin, eta * eta, h)

    def __del__(self):
        if getattr(self, "_H", None) and _ref is not None:
            _ref.ref_free(self._H)
            self._H = None

    @property
    def nleaves(self):
        return ref().ref_nleaves(self._H)

    def perm(self):
        op = np.zeros(self.n, np.uint32)
        po = np.zeros(self.n, np.uint32)
        ref().ref_perm(self._H, _p(op), _p(po))
        return op, po

    def leaves(self):
        out = np.zeros((self.nleaves, 7), np.uint32)
        ref().ref_leaves(self._H, _p(out))
        return out

    def assemble(self, eps, rankmax=2**32 - 1, nthreads=0):
        ref().ref_assemble(self._H, eps, rankmax, nthreads)

    def helmholtz_aca_ranks(self, wavenumber, h, eps, rankmax=2**32 - 1):
        """Complex ACA ranks of the Helmholtz matrix per leaf (-1 inadmissible, -2 failed)."""
        out = np.zeros(self.nleaves, np.int32)
        ref().ref_helm_ranks(self._H, wavenumber, h, eps, rankmax, _p(out))
        return out

    def ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        ref().ref_ranks(self._H, _p(out))
        return out

    def leaf_data(self, l):
        cnt = ref().ref_leaf_data(self._H, l, None)
        out = np.zeros(cnt, np.float64)
        ref().ref_leaf_data(self._H, l, _p(out))
        return out

    def agglomerate(self, eps, rankmax=2**32 - 1):
        """The reference's agglH of the assembled leaves."""
        ref().ref_agglomerate(self._H, eps, rankmax)

    def savembls(self, eta, bmin, path):
        """The reference's own savembls of the assembled leaves."""
        if ref().ref_save(self._H, eta, bmin, os.fsencode(path)) != 0:
            raise RuntimeError("ref_save failed")

    def matvec(self, X, Y, d=1.0):
        X = np.ascontiguousarray(X, dtype=np.float64)
        p = 1 if X.ndim == 1 else X.shape[0]
        ref().ref_matvec(self._H, d, p, _p(X), _p(Y))
        return Y

    def gmres(self, b, x, eps, m, nsteps):
        b = np.ascontiguousarray(b, dtype=np.float64)
        e = C.c_double(eps)
        ns = C.c_uint(nsteps)
        r = ref().ref_gmres(self._H, _p(b), _p(x), C.byref(e), m, C.byref(ns))
        return r, e.value, ns.value

    def cg(self, b, x, eps, nsteps):
        b = np.ascontiguousarray(b, dtype=np.float64)
        e = C.c_double(eps)
        ns = C.c_uint(nsteps)
        r = ref().ref_cg(self._H, _p(b), _p(x), C.byref(e), C.byref(ns))
        return r, e.value, ns.value

    # --- Helmholtz (complex) H-matrix: mblock<dcomp> leaves of the same tree ---
    def helm_assemble(self, wavenumber, h, eps, rankmax=2**32 - 1, nthreads=0):
        ref().ref_helm_assemble(self._H, wavenumber, h, eps, rankmax, nthreads)

    def helm_ranks(self):
        """per leaf: rank after recompression, -1 dense"""
        out = np.zeros(self.nleaves, np.int32)
        ref().ref_helm_ranks_assembled(self._H, _p(out))
        return out

    def helm_leaf_data(self, l):
        cnt = ref().ref_helm_leaf_data(self._H, l, None)
        out = np.zeros(cnt, np.complex128)
        ref().ref_helm_leaf_data(self._H, l, _p(out))
        return out

    def helm_matvec(self, X, Y, d=1.0, op=0):
        """Y += d op(A) X; X, Y complex (p x n rows = columns of the n x p array); op 0 A, 1 A^H, 2 A^T."""
        X = np.ascontiguousarray(X, dtype=np.complex128)
        assert Y.dtype == np.complex128 and Y.flags.c_contiguous
        p = 1 if X.ndim == 1 else X.shape[0]
        d = complex(d)
        ref().ref_helm_matvec(self._H, op, d.real, d.imag, p, _p(X), _p(Y))
        return Y

    def helm_gmres(self, b, x, eps, m, nsteps):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        e = C.c_double(eps)
        ns = C.c_uint(nsteps)
        r = ref().ref_helm_gmres(self._H, _p(b), _p(x), C.byref(e), m, C.byref(ns))
        return r, e.value, ns.value

    def helm_savembls(self, eta, bmin, path):
        """The reference's own savembls of the Helmholtz (mblock<dcomp>) leaves."""
        if ref().ref_helm_save(self._H, eta, bmin, os.fsencode(path)) != 0:
            raise RuntimeError("ref_helm_save failed")

    def helm_agglomerate(self, eps, rankmax=2**32 - 1):
        """The reference's agglH of the Helmholtz (mblock<dcomp>) leaves."""
        ref().ref_helm_agglomerate(self._H, eps, rankmax)
