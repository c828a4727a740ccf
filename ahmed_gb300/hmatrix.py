"""Host-side mirror of the reference's H-matrix interface over libahx.

Names and argument meanings follow AHMED: ``matgenGeH_omp`` (assembly,
Include/matgen_omp.h:197), ``mltaGeHVec`` / ``mltaGeHGeM`` (y += d A x,
H/mltaGeHVec.cpp:567-577), ``GMRes`` (solvers/GMRES.cpp:80) and ``CG``
(solvers/CG.cpp:31).  Vectors are in the permuted (cluster) ordering.
"""
import atexit
import ctypes as C
import os
import weakref

import numpy as np

from . import _capi
from ._capi import BF16_FP32, DF64, FP32, FP64, TREE_BBX, TREE_PCA, check, lib, ptr

PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16": BF16_FP32, "df64": DF64}
TREES = {"bbx": TREE_BBX, "pca": TREE_PCA}


# Live handles are released in a fixed order (batches, then matrices) before
# the interpreter tears modules down; finalizers after that point do nothing.
_live = weakref.WeakSet()
_shutdown = False


@atexit.register
def _release_all():
    global _shutdown
    objs = list(_live)
    for o in objs:
        if isinstance(o, HBatch):
            o.close()
    for o in objs:
        if isinstance(o, HMatrix):
            o.close()
    _shutdown = True


def mean_nn(points):
    pts = np.ascontiguousarray(points, dtype=np.float64)
    return lib().ahx_mean_nn(ptr(pts), pts.shape[0])


def min_nn(points):
    """Smallest nearest-neighbour distance of the points (n x 3)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    return lib().ahx_min_nn(ptr(pts), pts.shape[0])


def _prec(p):
    return PRECISIONS[p] if isinstance(p, str) else int(p)


def _is_complex(a):
    """complex numpy array or torch tensor"""
    dt = getattr(a, "dtype", None)
    if dt is None:
        return False
    if isinstance(dt, np.dtype):
        return dt.kind == "c"
    return bool(getattr(dt, "is_complex", False))


def _ncols(a, n):
    if a.ndim == 1:
        return 1, n
    # numpy (p, n) C-contiguous rows == column-major n x p
    return a.shape[0], a.shape[1]


class HMatrix:
    """Cluster tree, block-cluster tree and (after assembly) device leaves."""

    def __init__(self, points, tree="bbx", bmin=32, eta=0.8, device=0, stream=None, symmetric=False):
        """symmetric: the symmetric block tree (subdivide_sym) with the HeH assembly
        (matgenHeH_omp) and products (mltaHeHVec): upper blocks stored once."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError("points must have shape (n, 3)")
        self.n = pts.shape[0]
        self.points = pts
        self.eta, self.bmin = float(eta), int(bmin)
        kind = TREES[tree] if isinstance(tree, str) else int(tree)
        h = C.c_void_p()
        create = lib().ahx_hmat_create_sym if symmetric else lib().ahx_hmat_create
        check(create(ptr(pts), self.n, kind, bmin, float(eta) ** 2, device,
                     C.c_void_p(stream) if stream else None, C.byref(h)))
        self.symmetric = bool(symmetric)
        self._h = h
        self.h = None
        self.eps = None
        self._batches = []
        self._stream_explicit = stream is not None
        _live.add(self)

    def close(self):
        for b in list(getattr(self, "_batches", [])):
            bb = b()
            if bb is not None:
                bb.close()
        if getattr(self, "_h", None):
            lib().ahx_hmat_destroy(self._h)
            self._h = None

    def __del__(self):
        if _shutdown:
            return
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def nleaves(self):
        return lib().ahx_hmat_nleaves(self._h)

    @property
    def stream(self):
        return lib().ahx_hmat_stream(self._h)

    def set_stream(self, stream):
        """Run this matrix's work on `stream` (a cudaStream_t value; None: a private stream)."""
        check(lib().ahx_hmat_set_stream(self._h, C.c_void_p(stream) if stream else None))
        self._stream_explicit = stream is not None

    def _follow_torch(self, *arrays):
        """Without an explicit stream, CUDA torch tensors are used on torch's current
        stream: the library is moved there so that it is ordered after their producers."""
        if self._stream_explicit:
            return
        for a in arrays:
            if getattr(a, "is_cuda", False):
                import torch

                # torch's legacy default stream is handle 0, which the library reads
                # as "private stream": pass cudaStreamLegacy (1) for it
                cur = torch.cuda.current_stream(a.device).cuda_stream or 1
                if cur != (self.stream or 0):
                    check(lib().ahx_hmat_set_stream(self._h, C.c_void_p(cur)))
                return

    def perm(self):
        op = np.zeros(self.n, np.uint32)
        po = np.zeros(self.n, np.uint32)
        check(lib().ahx_hmat_perm(self._h, ptr(op), ptr(po)))
        return op, po

    def leaves(self):
        out = np.zeros((self.nleaves, 7), np.uint32)
        check(lib().ahx_hmat_leaves(self._h, ptr(out)))
        return out

    # -- assembly ---------------------------------------------------------
    def matgenGeH_omp(self, h=None, eps=1e-6, rankmax=2**32 - 1):
        """ACA assembly of every leaf on the GPU (h: diagonal 1/(4 pi h); default mean NN)."""
        self.h = mean_nn(self.points) if h is None else float(h)
        self.eps = float(eps)
        check(lib().ahx_assemble(self._h, self.h, self.eps, min(int(rankmax), 2**32 - 1)))
        return self

    assemble = matgenGeH_omp
    # symmetric handles assemble with the HeH rules (Include/matgen_omp.h:96-101)
    matgenHeH_omp = matgenGeH_omp

    def assemble_hinted(self, h, eps, rank_hint, rankmax=2**32 - 1):
        """Assembly whose ACA workspace is sized by per-leaf rank hints (negative: none)."""
        self.h = float(h)
        self.eps = float(eps)
        hint = np.ascontiguousarray(rank_hint, dtype=np.float32)
        check(lib().ahx_assemble_hinted(self._h, self.h, self.eps, min(int(rankmax), 2**32 - 1),
                                        ptr(hint)))
        return self

    def assembly_stats(self):
        """(largest workspace batch in bytes, capacity retries, batches) of the last assembly."""
        out = np.zeros(3, np.uint64)
        check(lib().ahx_hmat_assembly_stats(self._h, ptr(out)))
        return tuple(int(v) for v in out)

    def autotune(self, precision, p):
        """Choose the mixed product's stream bucketing for p right-hand sides by timing
        candidates; returns (width, unit_bytes, best_ns, candidates)."""
        out = np.zeros(4, np.uint32)
        check(lib().ahx_hmat_autotune(self._h, _prec(precision), int(p), ptr(out)))
        return tuple(int(v) for v in out)

    def helmholtz_aca_ranks(self, wavenumber, h, eps, rankmax=2**32 - 1, rank_hint=None):
        """Complex ACA ranks of the Helmholtz matrix exp(ikr)/(4 pi r) per leaf
        (-1 inadmissible, -2 ACA failed); bounding-box trees."""
        out = np.zeros(self.nleaves, np.int32)
        hint = None if rank_hint is None else np.ascontiguousarray(rank_hint, dtype=np.float32)
        check(lib().ahx_helm_aca_ranks(self._h, float(wavenumber), float(h), float(eps),
                                       min(int(rankmax), 2**32 - 1), ptr(hint), ptr(out)))
        return out

    def features(self, eps, wavenumber=0.0):
        out = np.zeros((self.nleaves, 8), np.float32)
        check(lib().ahx_hmat_features(self._h, float(wavenumber), float(eps), ptr(out)))
        return out

    def ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        check(lib().ahx_hmat_ranks(self._h, ptr(out)))
        return out

    def aca_ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        check(lib().ahx_hmat_aca_ranks(self._h, ptr(out)))
        return out

    def leaf_data(self, l):
        cnt = lib().ahx_hmat_leaf_size(self._h, l)
        out = np.zeros(cnt, np.float64)
        if cnt:
            check(lib().ahx_hmat_get_leaf(self._h, l, ptr(out)))
        return out

    def set_leaves(self, ranks, data, offsets):
        ranks = np.ascontiguousarray(ranks, dtype=np.int32)
        data = np.ascontiguousarray(data, dtype=np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        check(lib().ahx_hmat_set_leaves(self._h, ptr(ranks), ptr(data), ptr(offsets)))
        self.eps = self.eps or 0.0

    # -- persistent leaves (savembls / loadmbls, Include/H.h:47-103) ---------
    def save(self, path, eta=None, bmin=None):
        """Writes the leaves in the reference's savembls layout; eta and bmin
        default to the ones this tree was built with."""
        eta = self.eta if eta is None else float(eta)
        bmin = self.bmin if bmin is None else int(bmin)
        check(lib().ahx_hmat_save(self._h, eta, bmin, os.fsencode(path)))

    def load(self, path):
        """Reads leaves written by savembls (the reference's or save()) into
        this tree; returns the file's (eta, bmin)."""
        eta, bmin = C.c_double(), C.c_uint32()
        check(lib().ahx_hmat_load(self._h, os.fsencode(path), C.byref(eta), C.byref(bmin)))
        self.eps = self.eps or 0.0
        return eta.value, bmin.value

    def storage_bytes(self, precision="fp64"):
        return lib().ahx_hmat_storage_bytes(self._h, _prec(precision))

    def prepare(self, precision="fp64"):
        check(lib().ahx_hmat_prepare(self._h, _prec(precision)))

    def release(self, precision):
        """Frees the product copy of a precision (not the FP64 leaves)."""
        check(lib().ahx_hmat_release(self._h, _prec(precision)))

    # -- Helmholtz leaves (mblock<dcomp>) ---------------------------------
    def helmholtz_assemble(self, wavenumber, h=None, eps=1e-6, rankmax=2**32 - 1):
        """The Helmholtz H-matrix exp(ikr)/(4 pi r) (diagonal exp(ikh)/(4 pi h)) on this
        tree, as the reference's apprx_unsym with T = dcomp (ACA<dcomp> + addtrll); on a
        symmetric handle the complex symmetric form of matgenSyH_omp (ACAr<dcomp>).
        Complex products and GMRes take complex128 arrays (see mltaGeHVec)."""
        self.zh = mean_nn(self.points) if h is None else float(h)
        self.zk = float(wavenumber)
        check(lib().ahx_helm_assemble(self._h, self.zk, self.zh, float(eps), min(int(rankmax), 2**32 - 1)))
        return self

    matgenSyH_omp = helmholtz_assemble

    def helm_ranks(self):
        out = np.zeros(self.nleaves, np.int32)
        check(lib().ahx_helm_ranks(self._h, ptr(out)))
        return out

    def helm_leaf_data(self, l):
        cnt = lib().ahx_helm_leaf_size(self._h, l)
        out = np.zeros(cnt, np.complex128)
        if cnt:
            check(lib().ahx_helm_get_leaf(self._h, l, ptr(out)))
        return out

    def helm_save(self, path, eta=None, bmin=None):
        """savembls of the Helmholtz (mblock<dcomp>) leaves in the reference's layout."""
        eta = self.eta if eta is None else float(eta)
        bmin = self.bmin if bmin is None else int(bmin)
        check(lib().ahx_helm_save(self._h, eta, bmin, os.fsencode(path)))

    def helm_load(self, path):
        """loadmbls of mblock<dcomp> leaves into this tree; returns the file's (eta, bmin)."""
        eta, bmin = C.c_double(), C.c_uint32()
        check(lib().ahx_helm_load(self._h, os.fsencode(path), C.byref(eta), C.byref(bmin)))
        return eta.value, bmin.value

    def helm_agglH(self, eps=1e-6, max_rank=2**32 - 1):
        """agglH with T = dcomp (H/agglH.cpp:291-305) on the Helmholtz leaves; returns the
        number of merged blocks.  The block tree changes: real leaves must be assembled again."""
        n = C.c_uint32()
        check(lib().ahx_helm_agglomerate(self._h, float(eps), min(int(max_rank), 2**32 - 1), C.byref(n)))
        return n.value

    def helm_storage_bytes(self, precision="fp64"):
        return lib().ahx_helm_storage_bytes(self._h, _prec(precision))

    def _helm_product(self, op, d, p, X, ldX, Y, ldY, precision):
        self._follow_torch(X, Y)
        d = complex(d)
        check(lib().ahx_helm_matvec(self._h, _prec(precision), int(op), d.real, d.imag, int(p), ptr(X),
                                    int(ldX), ptr(Y), int(ldY)))
        return Y

    # -- product ----------------------------------------------------------
    def mltaGeHGeM(self, d, p, X, ldX, Y, ldY, precision="fp64"):
        """Y += d A X with X, Y column-major (numpy / torch, host or CUDA).  Complex
        arrays use the Helmholtz leaves (the reference's dcomp instantiation;
        precision "fp32": complex64 leaves)."""
        if _is_complex(X):
            return self._helm_product(0, d, p, X, ldX, Y, ldY, precision)
        self._follow_torch(X, Y)
        check(lib().ahx_matvec(self._h, _prec(precision), float(d), int(p), ptr(X), int(ldX),
                               ptr(Y), int(ldY)))
        return Y

    def mltaGeHVec(self, d, x, y, precision="fp64"):
        """y += d A x; x, y of shape (n,) or (p, n) (rows are right-hand sides)."""
        p, ld = _ncols(x, self.n)
        return self.mltaGeHGeM(d, p, x, ld, y, ld, precision)

    def mltaGeHtGeM(self, d, p, X, ldX, Y, ldY, precision="fp64"):
        """Y += d A^T X (FP64 leaves; complex arrays: the Helmholtz leaves)."""
        if _is_complex(X):
            return self._helm_product(2, d, p, X, ldX, Y, ldY, precision)
        self._follow_torch(X, Y)
        check(lib().ahx_matvec_transposed(self._h, float(d), int(p), ptr(X), int(ldX), ptr(Y), int(ldY)))
        return Y

    def mltaGeHhGeM(self, d, p, X, ldX, Y, ldY, precision="fp64"):
        """Y += d A^H X (real leaves: A^T)."""
        if _is_complex(X):
            return self._helm_product(1, d, p, X, ldX, Y, ldY, precision)
        return self.mltaGeHtGeM(d, p, X, ldX, Y, ldY)

    # symmetric handles: the same products (H/mltaGeHVec.cpp:421-475)
    def mltaHeHVec(self, d, x, y, precision="fp64"):
        return self.mltaGeHVec(d, x, y, precision)

    def mltaHeHGeM(self, d, p, X, ldX, Y, ldY, precision="fp64"):
        return self.mltaGeHGeM(d, p, X, ldX, Y, ldY, precision)

    # complex symmetric (Helmholtz leaves of a symmetric handle, H/mltaGeHVec.cpp:885-895)
    mltaSyHVec = mltaHeHVec
    mltaSyHGeM = mltaHeHGeM

    def mltaGeHtVec(self, d, x, y, precision="fp64"):
        p, ld = _ncols(x, self.n)
        return self.mltaGeHtGeM(d, p, x, ld, y, ld, precision)

    def mltaGeHhVec(self, d, x, y, precision="fp64"):
        p, ld = _ncols(x, self.n)
        return self.mltaGeHhGeM(d, p, x, ld, y, ld, precision)

    # -- solvers ----------------------------------------------------------
    def GMRes(self, b, x, eps, m, nsteps, precision="fp64"):
        """Restarted GMRES(m); b, x of shape (n,) or (p, n).  Returns (status, eps[], nsteps[])."""
        p, ld = _ncols(b, self.n)
        self._follow_torch(b, x)
        iters = np.zeros(p, np.uint32)
        res = np.zeros(p, np.float64)
        fn = lib().ahx_helm_gmres if _is_complex(b) else lib().ahx_gmres
        code = check(fn(self._h, _prec(precision), p, ptr(b), ld, ptr(x), ld, float(eps), int(m), int(nsteps),
                        ptr(iters), ptr(res)))
        return (0 if code == _capi.AHX_OK else 1), res, iters

    def agglH(self, eps=None, max_rank=2**32 - 1):
        """Agglomeration (H/agglH.cpp:111-272): merges sibling low-rank leaves whose
        recompressed union stores no more; returns the number of merged blocks."""
        eps = self.eps if eps is None else float(eps)
        n = C.c_uint32()
        check(lib().ahx_agglomerate(self._h, eps, min(int(max_rank), 2**32 - 1), C.byref(n)))
        return n.value

    def matgenGeH_sqntl(self, h=None, recmpr=False, eps=1e-6, rankmax=2**32 - 1):
        """Include/matgen_sqntl.h:88-102: the assembly, then (recmpr) agglomeration."""
        self.matgenGeH_omp(h, eps, rankmax)
        if recmpr:
            self.agglH(eps, rankmax)
        return self

    def spctrlnrm(self, it_num=10):
        """Include/matrix.h:50-75: sqrt of the largest eigenvalue of A^T A by it_num
        power steps from x = 1 (FP64 leaves)."""
        out = C.c_double()
        check(lib().ahx_spctrlnrm(self._h, int(it_num), C.byref(out)))
        return out.value

    def CG(self, b, x, eps, nsteps):
        p, ld = _ncols(b, self.n)
        self._follow_torch(b, x)
        iters = np.zeros(p, np.uint32)
        res = np.zeros(p, np.float64)
        code = check(lib().ahx_cg(self._h, p, ptr(b), ld, ptr(x), ld, float(eps), int(nsteps),
                                  ptr(iters), ptr(res)))
        return (0 if code == _capi.AHX_OK else 1), res, iters


class HBatch:
    """Many assembled H-matrices as one product / one batched GMRES."""

    def __init__(self, mats, precision="fp64"):
        self.mats = list(mats)
        arr = (C.c_void_p * len(self.mats))(*[m.handle.value for m in self.mats])
        h = C.c_void_p()
        check(lib().ahx_batch_create(arr, len(self.mats), _prec(precision), C.byref(h)))
        self._h = h
        self.n = lib().ahx_batch_n(h)
        self.offsets = np.concatenate([[0], np.cumsum([m.n for m in self.mats])]).astype(np.int64)
        for m in self.mats:
            m._batches.append(weakref.ref(self))
        _live.add(self)

    def close(self):
        if getattr(self, "_h", None):
            lib().ahx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        if _shutdown:
            return
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _torch_sync(*arrays):
        # the batch runs on its own stream: CUDA torch tensors are synchronized around calls
        if any(getattr(a, "is_cuda", False) for a in arrays):
            import torch

            torch.cuda.synchronize()

    def prepare(self, precision):
        """Builds the product copy of a precision ahead of use ("df64": the
        refinement's outer residual)."""
        check(lib().ahx_batch_prepare(self._h, _prec(precision)))

    def matvec(self, d, X, Y, p=1):
        self._torch_sync(X, Y)
        check(lib().ahx_batch_matvec(self._h, float(d), int(p), ptr(X), ptr(Y)))
        self._torch_sync(X, Y)
        return Y

    def gmres(self, b, x, eps, m, nsteps):
        k = len(self.mats)
        self._torch_sync(b, x)
        iters = np.zeros(k, np.uint32)
        res = np.zeros(k, np.float64)
        code = check(lib().ahx_batch_gmres(self._h, ptr(b), ptr(x), float(eps), int(m),
                                           int(nsteps), ptr(iters), ptr(res)))
        return (0 if code == _capi.AHX_OK else 1), res, iters


# functional forms with the reference's argument order
def matgenGeH_omp(H, h=None, eps=1e-6, rankmax=2**32 - 1):
    return H.matgenGeH_omp(h, eps, rankmax)


def mltaGeHVec(d, H, x, y, precision="fp64"):
    return H.mltaGeHVec(d, x, y, precision)


def mltaGeHGeM(d, H, p, X, ldX, Y, ldY, precision="fp64"):
    return H.mltaGeHGeM(d, p, X, ldX, Y, ldY, precision)


def GMRes(H, b, x, eps, m, nsteps, precision="fp64"):
    return H.GMRes(b, x, eps, m, nsteps, precision)


def CG(H, b, x, eps, nsteps):
    return H.CG(b, x, eps, nsteps)


def mbls_header(path):
    """(eta, bmin, nleaves) of a savembls file (host only)."""
    eta, bmin, n = C.c_double(), C.c_uint32(), C.c_uint32()
    check(lib().ahx_mbls_header(os.fsencode(path), C.byref(eta), C.byref(bmin), C.byref(n)))
    return eta.value, bmin.value, n.value


def savembls(eta, bmin, H, path):
    """Include/H.h:89-103: the leaves of H with the caller's eta and bmin."""
    H.save(path, eta, bmin)


def loadmbls(path, H):
    """Include/H.h:60-73 into the tree H (built with the file's eta and bmin,
    see mbls_header); returns (eta, bmin)."""
    return H.load(path)
