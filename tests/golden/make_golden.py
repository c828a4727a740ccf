"""Generate golden vectors from the reference library itself.

Runs only where the AHMED sources are available and oracle/ref/build_ref.sh
has produced oracle/_ref/libahmed_ref.so.  The outputs (small .npz files next
to this script) are committed; the tests read them on any host.

Usage:  python tests/golden/make_golden.py            (Laplace cases)
        python tests/golden/make_golden.py helmholtz  (complex ACA ranks)
        python tests/golden/make_golden.py mbls       (savembls file hashes)
        python tests/golden/make_golden.py sym        (symmetric trees, HeH assembly/product)
        python tests/golden/make_golden.py aggl       (agglomeration, agglH)
        python tests/golden/make_golden.py zhmat      (Helmholtz H-matrix: complex assembly,
                                                       products, GMRes)
        python tests/golden/make_golden.py zmbls      (savembls files of mblock<dcomp> leaves)
        python tests/golden/make_golden.py zaggl      (agglH of mblock<dcomp> leaves)
        python tests/golden/make_golden.py cg         (the reference's CG, solvers/CG.cpp:31-113)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from ahmed_gb300 import geometry as G  # noqa: E402

EPS = 1e-6
ETA = 0.8

# name -> (points, bmin)
CASES = {
    "fib4096": (lambda: G.fibonacci_sphere(4096), 32),
    "cube3000": (lambda: G.cube_surface(3000, 5), 32),
    "ell2500": (lambda: G.ellipsoid_surface(2500, 7), 32),
    "sph360": (lambda: G.sphere_surface(360, 11), 12),
    "fib50": (lambda: G.fibonacci_sphere(50), 32),   # single-leaf tree edge case
}
FULL_DATA = {"sph360"}          # complete leaf arena committed for these
GMRES = {"fib4096", "cube3000"}


def main():
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    for name, (gen, bmin) in CASES.items():
        P = gen()
        h = O.mean_nn(P)
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin),
               "eta": np.float64(ETA), "eps": np.float64(EPS)}
        n = P.shape[0]
        rng = np.random.default_rng(0)
        x = rng.uniform(-1.0, 1.0, n)
        X = rng.uniform(-1.0, 1.0, (4, n))
        for kind, kname in ((O.TREE_BBX, "bbx"), (O.TREE_PCA, "pca")):
            R = O.RefH(P, kind, bmin, ETA, h)
            op, po = R.perm()
            out[f"{kname}_op_perm"] = op
            out[f"{kname}_po_perm"] = po
            out[f"{kname}_leaves"] = R.leaves()
            R.assemble(EPS, nthreads=1)
            out[f"{kname}_ranks"] = R.ranks()
            out[f"{kname}_y"] = R.matvec(x, np.zeros(n))
            Y = np.zeros((4, n))
            R.matvec(X, Y, d=-0.5)
            out[f"{kname}_Y4"] = Y
            if name in FULL_DATA:
                chunks = [R.leaf_data(l) for l in range(R.nleaves)]
                offs = np.zeros(R.nleaves + 1, np.uint64)
                offs[1:] = np.cumsum([c.size for c in chunks])
                out[f"{kname}_data"] = np.concatenate(chunks) if chunks else np.zeros(0)
                out[f"{kname}_offsets"] = offs
            if name in GMRES and kind == O.TREE_BBX:
                b = np.random.default_rng(3).standard_normal(n)
                for tag, hh in (("spec", h), ("spd", h / 2.0)):
                    R2 = O.RefH(P, kind, bmin, ETA, hh)
                    R2.assemble(EPS, nthreads=1)
                    xg = np.zeros(n)
                    ret, e, ns = R2.gmres(b, xg, 1e-8, 30, 150)
                    out[f"gmres_{tag}"] = np.array([ret, e, ns], np.float64)
                    out[f"gmres_{tag}_x"] = xg
                    out[f"gmres_{tag}_h"] = np.float64(hh)
                out["gmres_b"] = b
        out["x"] = x
        out["X4"] = X
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


# Helmholtz exp(ikr)/(4 pi r): ranks of the reference's complex ACA per leaf
HELM_CASES = {
    "helm_fib4096": (lambda: G.fibonacci_sphere(4096), 32),
    "helm_ell3000": (lambda: G.ellipsoid_surface(3000, 9), 32),
}
HELM_K = (1.0, 5.0, 15.0)


def helmholtz():
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    for name, (gen, bmin) in HELM_CASES.items():
        P = gen()
        h = O.mean_nn(P)
        R = O.RefH(P, O.TREE_BBX, bmin, ETA, h)
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
               "eps": np.float64(EPS), "leaves": R.leaves(), "wavenumbers": np.array(HELM_K)}
        for k in HELM_K:
            out[f"ranks_k{k:g}"] = R.helmholtz_aca_ranks(k, h, EPS)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


def mbls():
    """SHA-256 of the reference's own savembls file for sph360 (both trees):
    pins the byte layout without committing the file (the leaf data it holds
    are sph360.npz's *_data)."""
    import hashlib
    import json
    import tempfile
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    P = G.sphere_surface(360, 11)
    bmin = 12
    h = O.mean_nn(P)
    out = {"case": "sph360", "eta": ETA, "bmin": bmin}
    gold = np.load(os.path.join(HERE, "sph360.npz"))
    for kind, kname in ((O.TREE_BBX, "bbx"), (O.TREE_PCA, "pca")):
        R = O.RefH(P, kind, bmin, ETA, h)
        R.assemble(EPS, nthreads=1)
        chunks = [R.leaf_data(l) for l in range(R.nleaves)]
        if not np.array_equal(np.concatenate(chunks), gold[f"{kname}_data"]):
            sys.exit("reference leaves differ from sph360.npz")
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "A.mbls")
            R.savembls(ETA, bmin, path)
            raw = open(path, "rb").read()
        out[kname] = {"sha256": hashlib.sha256(raw).hexdigest(), "bytes": len(raw)}
    path = os.path.join(HERE, "mbls_sph360.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {path}")


# symmetric block trees (subdivide_sym) with the HeH assembly (ACAr, Hermitian
# diagonal blocks) and product (mltaHeHVec / mltaHeHGeM)
SYM_CASES = {"sym_fib4096": ("fib4096", False), "sym_sph360": ("sph360", True)}


def sym():
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    for name, (base, full) in SYM_CASES.items():
        gen, bmin = CASES[base]
        P = gen()
        h = O.mean_nn(P)
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
               "eps": np.float64(EPS)}
        n = P.shape[0]
        rng = np.random.default_rng(0)
        x = rng.uniform(-1.0, 1.0, n)
        X = rng.uniform(-1.0, 1.0, (4, n))
        for kind, kname in ((O.TREE_BBX, "bbx"), (O.TREE_PCA, "pca")):
            R = O.RefH(P, kind, bmin, ETA, h, sym=True)
            out[f"{kname}_leaves"] = R.leaves()
            R.assemble(EPS, nthreads=1)
            out[f"{kname}_ranks"] = R.ranks()
            out[f"{kname}_y"] = R.matvec(x, np.zeros(n))
            Y = np.zeros((4, n))
            R.matvec(X, Y, d=-0.5)
            out[f"{kname}_Y4"] = Y
            if full and kind == O.TREE_PCA:  # (sph360's bbx tree has dense leaves only)
                chunks = [R.leaf_data(l) for l in range(R.nleaves)]
                offs = np.zeros(R.nleaves + 1, np.uint64)
                offs[1:] = np.cumsum([c.size for c in chunks])
                out[f"{kname}_data"] = np.concatenate(chunks) if chunks else np.zeros(0)
                out[f"{kname}_offsets"] = offs
        out["x"] = x
        out["X4"] = X
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


def aggl():
    """The reference's agglomeration (agglH) after its assembly: leaves in index
    order, their ranks, the stored doubles and y = A x."""
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    for base in ("fib4096", "cube3000"):
        gen, bmin = CASES[base]
        P = gen()
        h = O.mean_nn(P)
        n = P.shape[0]
        x = np.random.default_rng(0).uniform(-1.0, 1.0, n)
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
               "eps": np.float64(EPS), "x": x}
        for kind, kname in ((O.TREE_BBX, "bbx"), (O.TREE_PCA, "pca")):
            R = O.RefH(P, kind, bmin, ETA, h)
            R.assemble(EPS, nthreads=1)
            R.agglomerate(EPS)
            L = R.leaves()
            r = R.ranks()
            order = np.argsort(L[:, 5])
            out[f"{kname}_leaves"] = L[order]
            out[f"{kname}_ranks"] = r[order]
            out[f"{kname}_stored"] = np.int64(sum(R.leaf_data(l).size for l in range(R.nleaves)))
            out[f"{kname}_y"] = R.matvec(x, np.zeros(n))
        path = os.path.join(HERE, f"aggl_{base}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


# Helmholtz H-matrices: the reference's mblock<dcomp> assembly (ACA<dcomp> +
# addtrll of H/mblock_Z.cpp), its complex products A, A^H, A^T and its complex
# GMRes; zhs_*: the complex symmetric form on the symmetric block tree
# (matgenSyH_omp: ACAr<dcomp>, packed symmetric diagonal blocks; mltaSyHVec /
# mltaSyHGeM; A^H X = conj(A conj(X)) from the same product).  GMRES cases use
# h = (smallest point distance) / gm_div: with the mean spacing the collocation
# matrix is indefinite and GMRES stagnates.
ZH_CASES = {"zh_fib4096": ("fib4096", O.TREE_BBX, 1, False, 8.0, False),
            "zh_ell2500": ("ell2500", O.TREE_PCA, 2, True, 4.0, False),
            "zhs_fib4096": ("fib4096", O.TREE_BBX, 2, True, 8.0, True),
            "zhs_ell2500": ("ell2500", O.TREE_PCA, 1, True, 4.0, True)}
ZH_K = 5.0
ZH_D = complex(0.7, -0.3)


def zhmat():
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    from scipy.spatial import cKDTree
    for name, (base, kind, p, full, gm_div, sym) in ZH_CASES.items():
        gen, bmin = CASES[base]
        P = gen()
        n = P.shape[0]
        h = O.mean_nn(P)
        rng = np.random.default_rng(3)
        X = rng.standard_normal((p, n)) + 1j * rng.standard_normal((p, n))
        Y0 = rng.standard_normal((p, n)) + 1j * rng.standard_normal((p, n))
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
               "eps": np.float64(EPS), "kind": np.int32(kind), "k": np.float64(ZH_K), "d": np.complex128(ZH_D),
               "X": X, "Y0": Y0, "sym": np.bool_(sym)}
        R = O.RefH(P, kind, bmin, ETA, h, sym=sym)
        out["leaves"] = R.leaves()
        out["op_perm"] = R.perm()[0]
        R.helm_assemble(ZH_K, h, EPS, nthreads=1)
        out["ranks"] = R.helm_ranks()
        for op in (0, 1, 2):
            Y = Y0.copy()
            if sym and op == 1:
                T = np.zeros_like(Y0)
                R.helm_matvec(np.ascontiguousarray(X.conj()), T, d=1.0, op=0)
                Y += ZH_D * T.conj()
            else:
                R.helm_matvec(X, Y, d=ZH_D, op=op)
            out[f"Y_op{op}"] = Y
        L = out["leaves"]
        if full:  # factors (U then V) of 40 low-rank leaves spread over the leaf list
            size = (L[:, 1].astype(np.int64) + L[:, 3]) * out["ranks"]
            lr = np.flatnonzero((out["ranks"] >= 0) & (size <= 2048))
            pick = lr[np.linspace(0, lr.size - 1, min(40, lr.size)).astype(int)]
            chunks = [R.helm_leaf_data(int(l)) for l in pick]
            offs = np.zeros(pick.size + 1, np.uint64)
            offs[1:] = np.cumsum([c.size for c in chunks])
            out["data_leaves"] = pick.astype(np.uint32)
            out["data"] = np.concatenate(chunks)
            out["offsets"] = offs
        if sym:  # packed symmetric diagonal blocks (mblock SyM data) of three dense leaves
            dd = np.flatnonzero((out["ranks"] < 0) & (L[:, 0] == L[:, 2]))[:3]
            out["sym_leaves"] = dd.astype(np.uint32)
            for q, l in enumerate(dd):
                out[f"sym_data{q}"] = R.helm_leaf_data(int(l))
        dd, _ = cKDTree(P).query(P, 2)
        gh = float(dd[:, 1].min()) / gm_div
        G2 = O.RefH(P, kind, bmin, ETA, gh, sym=sym)
        G2.helm_assemble(ZH_K, gh, EPS, nthreads=1)
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        x = np.zeros(n, np.complex128)
        r, e, ns = G2.helm_gmres(b, x, 1e-8, 100, 100)
        if r != 0:
            sys.exit(f"{name}: the reference GMRes did not converge in one cycle")
        out.update({"gm_h": np.float64(gh), "gm_b": b, "gm_x": x, "gm_iters": np.uint32(ns),
                    "gm_resid": np.float64(e), "gm_m": np.uint32(100)})
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB) ranks>=0: {(out['ranks'] >= 0).sum()}"
              f" gmres {ns} steps {e:.2e}")


def zmbls():
    """The reference's own savembls files of mblock<dcomp> leaves (Helmholtz, k = 5) on a
    200-point sphere (PCA trees, leaf 6), general and symmetric (status 5 SyM blocks)."""
    import tempfile
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    P = G.sphere_surface(200, 11)
    bmin, h = 6, O.mean_nn(P)
    out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
           "eps": np.float64(EPS), "k": np.float64(ZH_K)}
    for sym, tag in ((False, "gen"), (True, "sym")):
        R = O.RefH(P, O.TREE_PCA, bmin, ETA, h, sym=sym)
        R.helm_assemble(ZH_K, h, EPS, nthreads=1)
        out[f"{tag}_leaves"] = R.leaves()
        out[f"{tag}_op_perm"] = R.perm()[0]
        out[f"{tag}_ranks"] = R.helm_ranks()
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "A.mbls")
            R.helm_savembls(ETA, bmin, path)
            out[f"{tag}_file"] = np.frombuffer(open(path, "rb").read(), np.uint8)
    path = os.path.join(HERE, "zmbls_sph200.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


def zaggl():
    """The reference's agglH of mblock<dcomp> leaves (Helmholtz, k = 5): leaves in index
    order, their ranks, the stored elements and y = A x after agglomeration."""
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    for base, kind, kname in (("fib4096", O.TREE_BBX, "bbx"), ("ell2500", O.TREE_PCA, "pca")):
        gen, bmin = CASES[base]
        P = gen()
        h = O.mean_nn(P)
        n = P.shape[0]
        rng = np.random.default_rng(8)
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        out = {"points": P, "h": np.float64(h), "bmin": np.uint32(bmin), "eta": np.float64(ETA),
               "eps": np.float64(EPS), "k": np.float64(ZH_K), "kind": np.int32(kind), "x": x}
        R = O.RefH(P, kind, bmin, ETA, h)
        out["op_perm"] = R.perm()[0]
        R.helm_assemble(ZH_K, h, EPS, nthreads=1)
        out["nleaves_before"] = np.uint32(R.nleaves)
        R.helm_agglomerate(EPS)
        L = R.leaves()
        r = R.helm_ranks()
        order = np.argsort(L[:, 5])
        out["leaves"] = L[order]
        out["ranks"] = r[order]
        out["stored"] = np.int64(sum(R.helm_leaf_data(l).size for l in range(R.nleaves)))
        y = np.zeros(n, np.complex128)
        out["y"] = R.helm_matvec(x, y)
        path = os.path.join(HERE, f"zaggl_{base}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB) leaves {out['nleaves_before']} -> {R.nleaves}")


# CG (solvers/CG.cpp:31-113) on positive definite diagonal variants: h = mean
# spacing / 2 on the Fibonacci sphere, h = smallest spacing / 2 on the random
# cube surface (with the mean spacing a random cloud's matrix is indefinite);
# a converging solve and one stopped by its step limit.
CG_CASES = {"fib4096": "mean", "cube3000": "min"}


def _min_nn(P):
    from scipy.spatial import cKDTree

    d, _ = cKDTree(P).query(P, k=2)
    return float(d[:, 1].min())


def cg():
    if not O.ref_available():
        sys.exit("reference build missing: run oracle/ref/build_ref.sh first")
    out = {}
    for name, diag in CG_CASES.items():
        gen, bmin = CASES[name]
        P = gen()
        h = (O.mean_nn(P) if diag == "mean" else _min_nn(P)) / 2.0
        n = P.shape[0]
        b = np.random.default_rng(3).standard_normal(n)
        R = O.RefH(P, O.TREE_BBX, bmin, ETA, h)
        R.assemble(EPS, nthreads=1)
        for tag, steps in (("conv", 300), ("cap", 8)):
            x = np.zeros(n)
            ret, e, ns = R.cg(b, x, 1e-8, steps)
            out[f"{name}_{tag}"] = np.array([ret, e, ns], np.float64)
            out[f"{name}_{tag}_x"] = x
            print(f"{name} {tag}: ret {ret} eps {e:.3e} steps {ns}")
        out[f"{name}_b"] = b
        out[f"{name}_h"] = np.float64(h)
    path = os.path.join(HERE, "cg.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "cg":
        cg()
    elif len(sys.argv) > 1 and sys.argv[1] == "helmholtz":
        helmholtz()
    elif len(sys.argv) > 1 and sys.argv[1] == "mbls":
        mbls()
    elif len(sys.argv) > 1 and sys.argv[1] == "sym":
        sym()
    elif len(sys.argv) > 1 and sys.argv[1] == "aggl":
        aggl()
    elif len(sys.argv) > 1 and sys.argv[1] == "zhmat":
        zhmat()
    elif len(sys.argv) > 1 and sys.argv[1] == "zmbls":
        zmbls()
    elif len(sys.argv) > 1 and sys.argv[1] == "zaggl":
        zaggl()
    else:
        main()
