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
        L.or_set_blas.argtypes = [vp, vp]
        L.or_assemble_list.argtypes = [vp, dbl, dbl, u32, i32, vp, u32]
        L.or_matvec_layers.argtypes = [vp, dbl, u32, vp, C.c_uint64, vp, C.c_uint64, i32, vp, vp, u32, vp, u32]
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

    def assemble_list(self, leaves, eps=1e-6, rankmax=2**31, nthreads=0):
        """Assemble only the listed leaves (a bounded sample of the matrix)."""
        sel = np.ascontiguousarray(leaves, dtype=np.uint32)
        lib().or_assemble_list(self._H, self.h, eps, min(rankmax, 2**32 - 1), nthreads, _p(sel), len(sel))

    def matvec_layers(self, plan, X, Y, d=1.0, nthreads=0):
        """Y += d A_S X over the leaves of `plan` (layered_groups), X and Y of shape
        (p, n) (rows are right-hand sides, i.e. n x p column-major, ld n)."""
        order, gs, ls = plan
        assert X.flags.c_contiguous and Y.flags.c_contiguous
        p = 1 if X.ndim == 1 else X.shape[0]
        lib().or_matvec_layers(self._H, d, p, _p(X), self.n, _p(Y), self.n, nthreads, _p(order), _p(gs),
                               len(gs) - 1, _p(ls), len(ls) - 1)
        return Y

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


def layered_groups(leaves, sel):
    """Groups the selected leaves by row cluster (b1, n1) and the groups into
    layers of pairwise disjoint row clusters (nesting depth in the cluster tree:
    two clusters either nest or are disjoint).  Returns (order, group_start,
    layer_start) as uint32 arrays for OracleH.matvec_layers."""
    sel = np.asarray(sel, dtype=np.int64)
    key = {}
    for l in sel:
        key.setdefault((int(leaves[l, 0]), int(leaves[l, 1])), []).append(int(l))
    clusters = sorted(key, key=lambda c: (c[0], -c[1]))
    depth, stack = {}, []
    for b1, n1 in clusters:
        while stack and stack[-1] <= b1:
            stack.pop()
        depth[(b1, n1)] = len(stack)
        stack.append(b1 + n1)
    layers = sorted(set(depth.values()))
    order, gs, ls = [], [0], [0]
    for q in layers:
        for c in clusters:
            if depth[c] == q:
                order.extend(key[c])
                gs.append(len(order))
        ls.append(len(gs) - 1)
    u = lambda a: np.asarray(a, dtype=np.uint32)
    return u(order), u(gs), u(ls)


def use_host_blas():
    """Routes the sampled products through the OpenBLAS that scipy bundles
    (dgemm_/dgemv_, one thread per caller; the reference calls BLAS in the same
    places).  Returns a description, or None when no such library is found."""
    import glob
    try:
        import scipy
    except ImportError:
        return None
    d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cand = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    for path in cand:
        try:
            B = C.CDLL(path)
            gemm = C.cast(B.scipy_dgemm_, C.c_void_p).value
            gemv = C.cast(B.scipy_dgemv_, C.c_void_p).value
            B.scipy_openblas_set_num_threads(1)
        except (OSError, AttributeError):
            continue
        lib().or_set_blas(gemm, gemv)
        use_host_blas._keep = B
        return os.path.basename(path) + " dgemm_/dgemv_, 1 thread per OpenMP thread"
    return None


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
