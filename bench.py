"""Benchmark: H-matvec and GMRES on one GB300 (and the CPU reference path beside it).

Default workload (--workload headline): N = 1,048,576 uniform random points on
the unit-cube surface (seed 4), Laplace kernel with diagonal 1/(4 pi h), h = half
the smallest nearest-neighbour distance, bounding-box tree, leaf 64, eta 0.8, ACA
eps 1e-6; 64 right-hand sides.  A step is one product Y += A X with all 64
right-hand sides, FP32 leaves on the tensor cores (error per right-hand side
against the FP64 product <= 1e-6); `value` counts vector products per second.
The same line carries the BF16-factor product with its error, the plain FP64
product, and GMRES(50) to a 1e-8 FP64 residual (mixed and plain, median of 3
solves).  The leaf streams (tens of GB) are larger than L2: no flush.

The --workload sphere case below is the N = 65,536 sphere benchmark:

Workload (Laplace single-layer collocation on the unit sphere):
  N = 65,536 Fibonacci-sphere points, K(x,y) = 1/(4 pi |x-y|), diagonal
  1/(4 pi h) with h the mean nearest-neighbour distance; bounding-box cluster
  tree, leaf size 32, eta = 0.8, ACA eps = 1e-6; 16 right-hand sides
  X ~ U[-1, 1] (numpy PCG64 seed 1).
A step is one product Y += A X of the assembled H-matrix with all 16
right-hand sides; `value` counts vector products (16 per step) per second.
The leaf arena (>= 0.5 GB) is larger than L2, so no flush is needed between
steps.  `value` uses FP32 leaf storage (the mixed form); the plain FP64 form
is timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_POINTS = 65536
NRHS = 16
BMIN = 32
ETA = 0.8
EPS = 1e-6
METRIC = "H-matvec/s"
UNIT = "vector products/s"
WORKLOAD = {
    "workload": "laplace-sphere-65536-16rhs",
    "points": "fibonacci sphere", "n": N_POINTS, "rhs": NRHS, "tree": "bbx", "leaf": BMIN,
    "eta": ETA, "eps": EPS, "kernel": "1/(4 pi r), diag 1/(4 pi h)",
    "l2": "inputs larger than L2 (no flush)",
}


def set_size(n):
    """Smaller point counts are used only for profiling captures."""
    global N_POINTS
    N_POINTS = n
    WORKLOAD["n"] = n
    WORKLOAD["workload"] = f"laplace-sphere-{n}-16rhs"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_max_ms(ms, ws, dev):
    """Time of a step over all replicas (N > 1: every rank runs the whole workload
    on its own GPU, no data-path collective): the slowest rank's, by one MAX
    all-reduce of a one-element tensor on `dev` (the rank's GPU under NCCL; the
    CPU under gloo in the tests)."""
    if ws <= 1:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            sm = [float(r[0]) for r in rows]
            out["sm_mhz"] = statistics.median(sm) if sm else None
            out["sm_max_mhz"] = float(rows[0][1]) if rows else None
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for k, nm in enumerate(names):
                if any(r[3 + k].strip() in ("Active", "1") for r in rows):
                    out["reasons"].append(nm)
            out["samples"] = len(rows)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        return out


def algorithmic_bytes(H, prec, p):
    """Leaf bytes read once per product + X read once + Y read and written once."""
    arena = H.storage_bytes(prec)
    return arena + p * H.n * (8 + 2 * 8)


def cpu_reference_run(steps, warmup, threads):
    """The reference path on the host cores (oracle restatement; full product per step)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from ahmed_gb300 import geometry as G

    P = G.fibonacci_sphere(N_POINTS)
    h = O.mean_nn(P)
    Ho = O.OracleH(P, O.TREE_BBX, BMIN, ETA, h)
    Ho.assemble(EPS, nthreads=threads)
    X = np.random.default_rng(1).uniform(-1.0, 1.0, (NRHS, N_POINTS))
    Y = np.zeros_like(X)
    for _ in range(warmup):
        Ho.matvec(X, Y, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        Ho.matvec(X, Y, nthreads=threads)
    dt = time.perf_counter() - t0
    return NRHS * steps / dt, dt / steps


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    val, sec = cpu_reference_run(args.steps, args.warmup, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": WORKLOAD,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full 16-RHS products of the N=65536 H-matrix "
                                   "(oracle C restatement, OpenMP over right-hand sides)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch
    import ahmed_gb300 as A

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P = A.geometry.fibonacci_sphere(N_POINTS)
    h = A.mean_nn(P)
    H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA, device=local)
    # a dedicated (non-default) stream shared by the library and the CUDA events
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    H.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    H.matgenGeH_omp(h, EPS)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    ranks = H.ranks()
    X = torch.from_numpy(np.random.default_rng(1).uniform(-1.0, 1.0, (NRHS, N_POINTS))).to(dev)
    Y = torch.zeros_like(X)

    launches = {}

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = A.lib().ahx_kernel_launches()
        e0.record(stream)
        for _ in range(steps):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        e1.record(stream)
        torch.cuda.synchronize()
        launches[prec] = A.lib().ahx_kernel_launches() - l0
        ms = replica_max_ms(e0.elapsed_time(e1), ws, dev)
        return ms / steps

    H.prepare("fp64")
    H.prepare("fp32")
    tuned = H.autotune("fp32", NRHS) if args.autotune else None
    ms64 = timed("fp64", max(2, args.steps // 4), args.warmup)
    with ClockSampler(local) as cs:
        ms32 = timed("fp32", args.steps, args.warmup)
    clocks = cs.summary()

    # end to end through the public API with pinned host buffers
    Xh = torch.from_numpy(np.random.default_rng(1).uniform(-1.0, 1.0, (NRHS, N_POINTS))).pin_memory()
    Yh = torch.zeros_like(Xh).pin_memory()
    for _ in range(args.warmup):
        H.mltaGeHVec(1.0, Xh.numpy(), Yh.numpy(), precision="fp32")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        H.mltaGeHVec(1.0, Xh.numpy(), Yh.numpy(), precision="fp32")
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps

    # accuracy of the measured forms against the FP64 product (per right-hand side)
    Y64 = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Y64, precision="fp64")
    Y32 = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Y32, precision="fp32")
    torch.cuda.synchronize()
    err32 = float(((Y32 - Y64).norm(dim=1) / Y64.norm(dim=1)).max())

    peak, peak_kind = _peaks()
    bytes32 = algorithmic_bytes(H, "fp32", NRHS)
    bytes64 = algorithmic_bytes(H, "fp64", NRHS)
    achieved = bytes32 / (ms32 * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("tc_product_fp32_16rhs_sphere65536")
        except Exception:
            traffic = None
    value = ws * NRHS / (ms32 * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(WORKLOAD, parallelism=("replicas%d" % ws),
                       leaves=int(H.nleaves), lowrank_leaves=int((ranks >= 0).sum()),
                       avg_rank=float(ranks[ranks >= 0].mean()),
                       fp32_arena_bytes=int(H.storage_bytes("fp32")),
                       fp64_arena_bytes=int(H.storage_bytes("fp64")),
                       plain_fp64_value=ws * NRHS / (ms64 * 1e-3), plain_fp64_ms=ms64,
                       mixed_over_plain=ms64 / ms32, fp32_max_rel_err_per_rhs=err32,
                       assembly_s=t_asm,
                       autotuned=(None if tuned is None else
                                  {"rhs_width": tuned[0], "unit_bytes": tuned[1], "candidates": tuned[3]})),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind, "algorithmic_bytes": bytes32,
                     "fp64_algorithmic_bytes": bytes64},
        "e2e": {"value": ws * NRHS / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": 2 * NRHS * N_POINTS * 8,
                "d2h_bytes_per_step": NRHS * N_POINTS * 8},
        "gpu_launches": launches.get("fp32"),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cval, _ = cpu_reference_run(max(2, min(args.steps, 8)), 1, threads)
        line["cpu_baseline"] = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "full 16-RHS products of the same N=65536 H-matrix "
                                          "assembled by the oracle (C restatement)"}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def _sample_rows_exact(P, perm, x, rows, h):
    """Exact FP64 rows of A x (Laplace, permuted order) by direct summation on the host."""
    Pp = P[perm]
    out = np.zeros((len(rows), x.shape[0]))
    for q, i in enumerate(rows):
        d = Pp - Pp[i]
        r = np.sqrt((d * d).sum(axis=1))
        r[i] = 1.0
        k = 1.0 / (4.0 * np.pi * r)
        k[i] = 1.0 / (4.0 * np.pi * h)
        out[q] = x @ k
    return out


def run_large(args):
    """N = 1,048,576 uniform random points on the unit-cube surface (seed 4), leaf 64,
    eta 0.8, ACA eps 1e-6; BF16 low-rank factors + FP32 dense leaves; 64 right-hand sides;
    GMRES(50) to a 1e-8 FP64 residual (FP64 refinement) against the plain FP64 form."""
    import torch
    import ahmed_gb300 as A

    n, p, bmin = args.n_large, 64, 64
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    P = A.geometry.cube_surface(n, 4)
    t0 = time.perf_counter()
    h = (A.min_nn(P) if args.diag == "min" else A.mean_nn(P)) / args.diag_scale
    H = A.HMatrix(P, "bbx", bmin=bmin, eta=ETA, device=0)
    t_tree = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    H.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    H.matgenGeH_omp(h, EPS)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    ranks = H.ranks()
    op, _ = H.perm()
    out = {"workload": f"laplace-cube-{n}-64rhs", "n": n, "rhs": p, "leaf": bmin,
           "diag": f"1/(4 pi h), h = {args.diag} nearest-neighbour distance / {args.diag_scale:g}",
           "tree_s": t_tree, "assembly_s": t_asm, "leaves": int(H.nleaves),
           "lowrank_leaves": int((ranks >= 0).sum()), "avg_rank": float(ranks[ranks >= 0].mean()),
           "fp64_arena_bytes": int(H.storage_bytes("fp64"))}
    # assembly error on sampled rows against the exact FP64 kernel sums
    rng = np.random.default_rng(4)
    x1 = rng.uniform(-1.0, 1.0, n)
    y1 = torch.zeros(n, dtype=torch.float64, device=dev)
    H.mltaGeHVec(1.0, torch.from_numpy(x1).to(dev), y1, precision="fp64")
    rows = rng.choice(n, 32, replace=False)
    ex = _sample_rows_exact(P, op, x1[None, :], rows, h)[:, 0]
    out["assembly_rel_err_sampled_rows"] = float(np.linalg.norm(y1.cpu().numpy()[rows] - ex) / np.linalg.norm(ex))
    H.prepare("bf16")
    if args.autotune:
        out["autotuned"] = dict(zip(("rhs_width", "unit_bytes", "best_ns", "candidates"), H.autotune("bf16", p)))
    out["bf16_arena_bytes"] = int(H.storage_bytes("bf16"))
    X = torch.from_numpy(np.random.default_rng(5).uniform(-1.0, 1.0, (p, n))).to(dev)
    Y = torch.zeros_like(X)

    def timed(prec, steps):
        for _ in range(3):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    with ClockSampler(0) as cs:
        ms_bf16 = timed("bf16", args.steps)
    out["clocks"] = cs.summary()
    ms_64 = timed("fp64", 2)
    ms_df = timed("df64", 2)   # the refinement's outer residual product (double-float)
    Y64 = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Y64, precision="fp64")
    Yb = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Yb, precision="bf16")
    torch.cuda.synchronize()
    peak, peak_kind = _peaks()
    bytes_b = algorithmic_bytes(H, "bf16", p)
    out["product"] = {"bf16_ms": ms_bf16, "fp64_ms": ms_64, "df64_ms": ms_df, "speedup": ms_64 / ms_bf16,
                      "bf16_max_rel_err_per_rhs": float(((Yb - Y64).norm(dim=1) / Y64.norm(dim=1)).max()),
                      "algorithmic_bytes": bytes_b,
                      "achieved_gbs": bytes_b / (ms_bf16 * 1e-3) / 1e9, "peak_gbs": peak,
                      "frac": bytes_b / (ms_bf16 * 1e-3) / 1e9 / peak, "peak_kind": peak_kind}
    del Y, Y64, Yb
    # GMRES(50) to 1e-8 with 64 right-hand sides b ~ N(0, 1)
    B = torch.from_numpy(np.random.default_rng(6).standard_normal((p, n))).to(dev)
    res = {}
    for prec, cap in (("bf16", args.gmres_cap), ("fp64", args.gmres_cap_fp64)):
        Xs = torch.zeros_like(B)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, rr, its = H.GMRes(B, Xs, 1e-8, 50, cap, precision=prec)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # true FP64 residual of the returned solution
        R = B.clone()
        H.mltaGeHVec(-1.0, Xs, R, precision="fp64")
        true = float((R.norm(dim=1) / B.norm(dim=1)).max())
        res[prec] = {"s": dt, "converged": st == 0, "max_iters": int(its.max()),
                     "mean_iters": float(its.mean()), "max_resid": float(rr.max()),
                     "true_max_resid": true, "iters_per_s": float(its.max()) / dt,
                     "solves_per_s": (p / dt) if st == 0 else None}
        del Xs, R
    if res["bf16"]["solves_per_s"] and res["fp64"]["solves_per_s"]:
        res["mixed_over_plain"] = res["bf16"]["solves_per_s"] / res["fp64"]["solves_per_s"]
    out["gmres"] = res
    print(json.dumps(out))


def run_product(args):
    """Products only (profiling cases): `--geometry` sphere (Fibonacci) or cube (random
    surface, seed 4), `--n` points, `--leaf`, `--rhs`, `--precision`; assembly with the
    mean nearest-neighbour diagonal, then `--warmup` + `--steps` products Y += A X."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    n = args.n
    P = A.geometry.cube_surface(n, 4) if args.geometry == "cube" else A.geometry.fibonacci_sphere(n)
    H = A.HMatrix(P, "bbx", bmin=args.leaf, eta=ETA, device=0, symmetric=args.symmetric)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    H.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    H.matgenGeH_omp(A.mean_nn(P), EPS)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    H.prepare(args.precision)
    X = torch.from_numpy(np.random.default_rng(1).uniform(-1.0, 1.0, (args.rhs, n))).to(dev)
    Y = torch.zeros_like(X)
    for _ in range(args.warmup):
        H.mltaGeHVec(1.0, X, Y, precision=args.precision)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        H.mltaGeHVec(1.0, X, Y, precision=args.precision)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    b = algorithmic_bytes(H, args.precision, args.rhs)
    sym = "-sym" if args.symmetric else ""
    out = {"workload": f"laplace-{args.geometry}-{n}-{args.rhs}rhs-{args.precision}{sym}", "ms": ms,
           "algorithmic_bytes": b, "achieved_gbs": b / (ms * 1e-3) / 1e9, "assembly_s": t_asm,
           "fp64_leaf_bytes": int(H.storage_bytes("fp64"))}
    if args.precision == "fp32" and not args.symmetric:
        out["sweep_bytes"] = _kernel_bytes(H, args.rhs)
    print(json.dumps(out))


def run_predictor(args):
    """Learned rank predictor: trains the 8-64-64-1 network on the GPU on (feature, ACA rank)
    pairs of five assembled H-matrices (spheres, an ellipsoid, a cube surface; leaf 32, eta 0.8,
    eps 1e-6), then assembles two held-out N = 65,536 matrices with and without rank hints."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    G = A.geometry
    train = []
    for n, geo in [(3000, "s"), (5000, "e"), (8000, "s"), (16384, "c"), (32768, "s")]:
        P = G.fibonacci_sphere(n) if geo == "s" else (G.ellipsoid_surface(n, n) if geo == "e" else G.cube_surface(n, n))
        train.append(A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA).matgenGeH_omp(A.mean_nn(P), EPS))
    X, r = A.training_set(train, EPS)
    M = A.RankPredictor(seed=0)
    t0 = time.perf_counter()
    losses = M.fit(X, r, epochs=60, batch=512, lr=3e-3)
    t_train = time.perf_counter() - t0
    out = {"workload": "rank-predictor", "train_pairs": int(len(r)), "train_s": t_train,
           "loss_first_epoch": float(losses[0]), "loss_last_epoch": float(losses[-1])}
    for name, P in [("ellipsoid-65536", G.ellipsoid_surface(65536, 5, (1.0, 0.7, 0.4))),
                    ("sphere-65536", G.fibonacci_sphere(65536))]:
        h = A.mean_nn(P)
        H0 = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
        H0.matgenGeH_omp(h, EPS)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H0.matgenGeH_omp(h, EPS)
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        a0, st0, lv = H0.aca_ranks(), H0.assembly_stats(), H0.leaves()
        t0 = time.perf_counter()
        pred = M.predict(H0.features(EPS))
        t_pred = time.perf_counter() - t0
        adm = (lv[:, 4] == 1) & (a0 >= 0)
        rel = np.abs(pred[adm] - a0[adm]) / np.maximum(a0[adm], 1)
        H1 = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
        hint = np.where(lv[:, 4] == 1, pred, -1.0)
        H1.assemble_hinted(h, EPS, hint)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H1.assemble_hinted(h, EPS, hint)
        torch.cuda.synchronize()
        t_hint = time.perf_counter() - t0
        st1 = H1.assembly_stats()
        out[name] = {"identical_ranks": bool((H1.aca_ranks() == a0).all() and (H1.ranks() == H0.ranks()).all()),
                     "median_rel_rank_err": float(np.median(rel)), "p90_rel_rank_err": float(np.percentile(rel, 90)),
                     "plain": {"assembly_s": t_plain, "workspace_bytes": st0[0], "retries": st0[1], "batches": st0[2]},
                     "hinted": {"assembly_s": t_hint, "workspace_bytes": st1[0], "retries": st1[1], "batches": st1[2],
                                "predict_s": t_pred}}
        H0.close()
        H1.close()
    print(json.dumps(out))


def run_helmholtz(args):
    """Rank predictor on the Helmholtz kernel exp(ikr)/(4 pi r) (diagonal exp(ikh)/(4 pi h)):
    (feature, complex-ACA rank) pairs from Fibonacci spheres at N = 16,384 / 65,536 / 131,072
    with wavenumbers k ~ U[1, 20] (numpy PCG64 seed 7), eps 1e-6, leaf 32, eta 0.8; the MLP is
    trained on the GPU; then complex ACA with and without predicted ranks on held-out
    matrices (random sphere points, N = 65,536, k = 3.7 and 16.2), and the complex
    H-matrix of the k = 16.2 one: assembly and products with complex128 / complex64 leaves."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    G = A.geometry
    rng = np.random.default_rng(7)
    Xs, ys = [], []
    t0 = time.perf_counter()
    for n, nk in [(16384, 12), (65536, 5), (131072, 3)]:
        P = G.fibonacci_sphere(n)
        h = A.mean_nn(P)
        H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
        lv = H.leaves()
        for k in rng.uniform(1.0, 20.0, nk):
            r = H.helmholtz_aca_ranks(k, h, EPS)
            sel = (lv[:, 4] == 1) & (r >= 0)
            Xs.append(H.features(EPS, wavenumber=k)[sel])
            ys.append(r[sel])
        H.close()
    t_data = time.perf_counter() - t0
    X, y = np.concatenate(Xs), np.concatenate(ys)
    M = A.RankPredictor(seed=0)
    t0 = time.perf_counter()
    losses = M.fit(X, y, epochs=30, batch=1024, lr=2e-3)
    t_train = time.perf_counter() - t0
    out = {"workload": "helmholtz-rank-predictor", "train_pairs": int(len(y)), "pairs_s": t_data,
           "train_s": t_train, "loss_first_epoch": float(losses[0]), "loss_last_epoch": float(losses[-1])}
    P = G.sphere_surface(65536, 17)
    h = A.mean_nn(P)
    H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
    lv = H.leaves()
    for k in (3.7, 16.2):
        H.helmholtz_aca_ranks(k, h, EPS)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r0 = H.helmholtz_aca_ranks(k, h, EPS)
        t_plain = time.perf_counter() - t0
        st0 = H.assembly_stats()
        t0 = time.perf_counter()
        pred = M.predict(H.features(EPS, wavenumber=k))
        t_pred = time.perf_counter() - t0
        hint = np.where(lv[:, 4] == 1, pred, -1.0)
        t0 = time.perf_counter()
        r1 = H.helmholtz_aca_ranks(k, h, EPS, rank_hint=hint)
        t_hint = time.perf_counter() - t0
        st1 = H.assembly_stats()
        adm = (lv[:, 4] == 1) & (r0 >= 0)
        rel = np.abs(pred[adm] - r0[adm]) / np.maximum(r0[adm], 1)
        out[f"k{k:g}"] = {"identical_ranks": bool((r0 == r1).all()), "mean_rank": float(r0[adm].mean()),
                          "median_rel_rank_err": float(np.median(rel)), "p90_rel_rank_err": float(np.percentile(rel, 90)),
                          "plain": {"aca_s": t_plain, "workspace_bytes": st0[0], "retries": st0[1], "batches": st0[2]},
                          "hinted": {"aca_s": t_hint, "predict_s": t_pred, "workspace_bytes": st1[0],
                                     "retries": st1[1], "batches": st1[2]}}
    # the complex H-matrix itself (mblock<dcomp> leaves) at k = 16.2: assembly and
    # products with complex128 and complex64 leaves (CUDA events, 16 and 1 RHS)
    dev = torch.device("cuda", 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    H.helmholtz_assemble(16.2, h, EPS)
    torch.cuda.synchronize()
    zr = H.helm_ranks()
    zout = {"k": 16.2, "assembly_s": time.perf_counter() - t0, "low_rank_leaves": int((zr >= 0).sum()),
            "mean_rank": float(zr[zr >= 0].mean()), "complex128_bytes": int(H.helm_storage_bytes("fp64")),
            "complex64_bytes": int(H.helm_storage_bytes("fp32"))}
    rng2 = np.random.default_rng(11)
    for p in (16, 1):
        X = torch.from_numpy(rng2.standard_normal((p, H.n)) + 1j * rng2.standard_normal((p, H.n))).to(dev)
        ys = {}
        for prec in ("fp64", "fp32"):
            Y = torch.zeros_like(X)
            H.mltaGeHVec(1.0, X, Y, precision=prec)  # warm-up (builds the complex64 copy)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(5):
                H.mltaGeHVec(1.0, X, Y, precision=prec)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 5
            Y.zero_()
            H.mltaGeHVec(1.0, X, Y, precision=prec)
            ys[prec] = Y.cpu().numpy()
            leaf = H.helm_storage_bytes(prec)
            byts = leaf + p * H.n * 16 * 3
            zout[f"{prec}_{p}rhs"] = {"ms": ms, "algorithmic_bytes": int(byts), "achieved_gbs": byts / (ms * 1e-3) / 1e9}
        err = np.linalg.norm(ys["fp32"] - ys["fp64"], axis=1) / np.linalg.norm(ys["fp64"], axis=1)
        zout[f"fp32_err_{p}rhs"] = float(err.max())
    out["complex_hmatrix"] = zout
    H.close()
    print(json.dumps(out))


def run_zhmat(args):
    """The Helmholtz H-matrix (mblock<dcomp> leaves) on `--n` random sphere points (seed 17),
    k = 16.2, leaf 32, eta 0.8, eps 1e-6 (`--symmetric`: the complex symmetric form on the
    symmetric tree): complex assembly; products with complex128 and complex64 leaves at 16
    and 1 RHS (`--warmup` + `--steps`, CUDA events); complex GMRES(50) to 1e-8 with
    h = smallest nearest-neighbour distance / 8, one RHS b ~ N(0,1) + i N(0,1) (seed 12),
    complex128 leaves and complex64 leaves with FP64 refinement."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    P = A.geometry.sphere_surface(args.n, 17)
    k = 16.2
    H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA, symmetric=args.symmetric)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    H.helmholtz_assemble(k, A.mean_nn(P), EPS)
    torch.cuda.synchronize()
    zr = H.helm_ranks()
    out = {"workload": f"helmholtz-sphere-{args.n}" + ("-sym" if args.symmetric else ""), "k": k,
           "assembly_s": time.perf_counter() - t0, "low_rank_leaves": int((zr >= 0).sum()),
           "mean_rank": float(zr[zr >= 0].mean()) if (zr >= 0).any() else 0.0,
           "complex128_bytes": int(H.helm_storage_bytes("fp64")), "complex64_bytes": int(H.helm_storage_bytes("fp32"))}
    peak, _ = _peaks()
    rng = np.random.default_rng(11)
    for p in (16, 1):
        X = torch.from_numpy(rng.standard_normal((p, H.n)) + 1j * rng.standard_normal((p, H.n))).to(dev)
        ys = {}
        for prec in ("fp64", "fp32"):
            Y = torch.zeros_like(X)
            for _ in range(args.warmup):
                H.mltaGeHVec(1.0, X, Y, precision=prec)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                H.mltaGeHVec(1.0, X, Y, precision=prec)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            Y.zero_()
            H.mltaGeHVec(1.0, X, Y, precision=prec)
            ys[prec] = Y.cpu().numpy()
            byts = H.helm_storage_bytes(prec) + p * H.n * 16 * 3
            out[f"{prec}_{p}rhs"] = {"ms": ms, "algorithmic_bytes": int(byts), "achieved_gbs": byts / (ms * 1e-3) / 1e9,
                                     "frac_of_hbm": byts / (ms * 1e-3) / 1e9 / peak}
        err = np.linalg.norm(ys["fp32"] - ys["fp64"], axis=1) / np.linalg.norm(ys["fp64"], axis=1)
        out[f"fp32_err_{p}rhs"] = float(err.max())
    H.close()
    # GMRES on the well-conditioned variant
    gh = A.min_nn(P) / 8.0
    G = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA, symmetric=args.symmetric)
    G.helmholtz_assemble(k, gh, EPS)
    b = np.random.default_rng(12).standard_normal(G.n) + 1j * np.random.default_rng(13).standard_normal(G.n)
    for prec in ("fp64", "fp32"):
        x = np.zeros_like(b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, res, its = G.GMRes(b, x, 1e-8, 50, 2000, precision=prec)
        t_s = time.perf_counter() - t0
        r = b.copy()
        G.mltaGeHVec(-1.0, x, r)  # r = b - A x with the complex128 leaves
        out[f"gmres_{prec}"] = {"s": t_s, "converged": st == 0, "iters": int(its[0]),
                                "true_resid": float(np.linalg.norm(r) / np.linalg.norm(b))}
    G.close()
    print(json.dumps(out))


def run_aggl(args):
    """Agglomeration (agglH) after the assembly: Fibonacci sphere `--n` points, leaf 32,
    eta 0.8, eps 1e-6, bounding-box tree (`--symmetric`: the symmetric one); wall clock of
    the agglomeration, leaves and FP64 storage before / after, and the change of y = A x."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    P = A.geometry.fibonacci_sphere(args.n)
    H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA, symmetric=args.symmetric)
    H.matgenGeH_omp(A.mean_nn(P), EPS)
    x = np.random.default_rng(0).uniform(-1.0, 1.0, H.n)
    y0 = H.mltaGeHVec(1.0, x, np.zeros(H.n))
    n0, s0 = H.nleaves, H.storage_bytes("fp64")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    merged = H.agglH(EPS)
    torch.cuda.synchronize()
    t_aggl = time.perf_counter() - t0
    y = H.mltaGeHVec(1.0, x, np.zeros(H.n))
    print(json.dumps({"workload": f"agglomeration-sphere-{args.n}" + ("-sym" if args.symmetric else ""),
                      "agglomeration_s": t_aggl, "merged": int(merged), "leaves_before": int(n0),
                      "leaves_after": int(H.nleaves), "fp64_bytes_before": int(s0),
                      "fp64_bytes_after": int(H.storage_bytes("fp64")),
                      "product_change": float(np.linalg.norm(y - y0) / np.linalg.norm(y0))}))
    H.close()


def run_batch(args):
    """Many uneven H-matrices in one launch: `--instances` instances (256), N log-uniform
    in [2048, 32768] (numpy PCG64 seed 2), geometry uniform among the unit sphere, the
    ellipsoid (1, 0.5, 0.25) and the unit-cube surface with uniform random surface points;
    leaf 32, eta 0.8, ACA eps 1e-6; one right-hand side per instance b ~ N(0, 1) (seed 3);
    GMRES(30) to 1e-8 with BF16 and with FP32-class leaves and FP64 refinement, against
    plain FP64."""
    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(2)
    k = args.instances
    ns = np.exp(rng.uniform(np.log(2048), np.log(32768), k)).astype(np.int64)
    geos = rng.integers(0, 3, k)
    names = ["sphere", "ellipsoid", "cube"]
    mats = []
    t_asm = 0.0
    for i in range(k):
        P = A.geometry.GEOMETRIES[names[geos[i]]](int(ns[i]), 1000 + i)
        h = (A.min_nn(P) if args.diag == "min" else A.mean_nn(P)) / args.diag_scale
        H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H.matgenGeH_omp(h, EPS)
        torch.cuda.synchronize()
        t_asm += time.perf_counter() - t0
        mats.append(H)
    ntot = int(ns.sum())
    out = {"workload": f"laplace-batch{k}", "instances": k, "points": ntot,
           "n_min": int(ns.min()), "n_max": int(ns.max()),
           "diag": f"1/(4 pi h), h = {args.diag} nearest-neighbour distance / {args.diag_scale:g}",
           "assembly_s_sum": t_asm,
           "fp64_arena_bytes": int(sum(H.storage_bytes("fp64") for H in mats))}
    b = np.random.default_rng(3).standard_normal(ntot)
    peak, _ = _peaks()
    for prec in ("bf16", "fp32", "fp64"):
        Bt = A.HBatch(mats, precision=prec)
        if prec != "fp64":
            Bt.prepare("df64")   # refinement residual copy, built with the streams (setup)
        x = torch.from_numpy(np.random.default_rng(4).uniform(-1, 1, ntot)).to(dev)
        y = torch.zeros_like(x)
        for _ in range(3):
            Bt.matvec(1.0, x, y)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            Bt.matvec(1.0, x, y)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        X = np.zeros(ntot)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, rr, its = Bt.gmres(b, X, 1e-8, 30, args.gmres_cap)
        dt = time.perf_counter() - t0
        out[prec] = {"product_ms": ms, "gmres_s": dt, "converged": st == 0,
                     "max_iters": int(its.max()), "mean_iters": float(its.mean()),
                     "max_resid": float(rr.max()), "solves_per_s": k / dt}
        Bt.close()
    out["bf16"]["product_over_fp64"] = out["fp64"]["product_ms"] / out["bf16"]["product_ms"]
    out["fp32"]["product_over_fp64"] = out["fp64"]["product_ms"] / out["fp32"]["product_ms"]
    out["gmres_mixed_over_plain"] = out["fp64"]["gmres_s"] / out["bf16"]["gmres_s"]
    out["gmres_mixed_fp32_over_plain"] = out["fp64"]["gmres_s"] / out["fp32"]["gmres_s"]
    print(json.dumps(out))


def run_kernels(args):
    """One small case of every kernel family, for per-kernel profiling captures (ncu
    launch lists with DRAM bytes): the Laplace sphere at `--n` points (leaf 32, eta 0.8,
    eps 1e-6): assembly (ACA, recompression, dense leaves), products with FP64 / FP32 /
    BF16 / double-float leaves at 16 and 1 right-hand sides, the transposed product;
    save and load of the leaves; the rank predictor (features, training, prediction,
    hinted assembly); the symmetric tree; agglomeration (N = 4096, real and complex);
    the Helmholtz H-matrix (complex ACA and products); a batch of four instances; the
    solvers last (GMRES, CG, spectral norm, batched GMRES), with short step limits."""
    import tempfile as _tf

    import torch
    import ahmed_gb300 as A

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    G = A.geometry
    n = args.n
    P = G.fibonacci_sphere(n)
    h = A.mean_nn(P)
    H = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
    H.matgenGeH_omp(h, EPS)
    rng = np.random.default_rng(1)
    for p in (16, 1):
        X = torch.from_numpy(rng.uniform(-1.0, 1.0, (p, n))).to(dev)
        for prec in ("fp64", "fp32", "bf16", "df64"):
            Y = torch.zeros_like(X)
            for _ in range(2):
                H.mltaGeHVec(1.0, X, Y, precision=prec)
        H.mltaGeHhGeM(1.0, p, X, n, torch.zeros_like(X), n)
    with _tf.TemporaryDirectory() as d:
        f = os.path.join(d, "leaves.mbls")
        H.save(f)
        H2 = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
        H2.load(f)
        H2.close()
    feats = H.features(EPS)
    r = H.aca_ranks()
    lv = H.leaves()
    sel = np.nonzero((lv[:, 4] == 1) & (r >= 0))[0][:8192]
    M = A.RankPredictor(seed=0)
    M.fit(feats[sel], r[sel], epochs=2, batch=1024, lr=2e-3)
    pred = M.predict(feats)
    Hh = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
    Hh.assemble_hinted(h, EPS, np.where(lv[:, 4] == 1, pred, -1.0))
    Hh.close()
    # the allocation-free ACA of one admissible block (points in cluster order on the device)
    import ctypes as _C
    from ahmed_gb300 import _capi
    op, _ = H.perm()
    pts = [torch.from_numpy(np.ascontiguousarray(P[op][:, i])).to(dev) for i in range(3)]
    adm = np.nonzero((lv[:, 4] == 1) & (lv[:, 1].astype(np.int64) + lv[:, 3] <= 2048))[0]  # fits its 8 MiB scratch
    b1, n1, b2, n2, _, _, i0 = (int(v) for v in lv[adm[len(adm) // 2]][:7])
    Ub = torch.zeros(n1 * 32, dtype=torch.float64, device=dev)
    Vb = torch.zeros(n2 * 32, dtype=torch.float64, device=dev)
    info = torch.zeros(3, dtype=torch.int32, device=dev)
    _capi.check(_capi.lib().ahx_aca_block_noalloc(
        _C.c_void_p(pts[0].data_ptr()), _C.c_void_p(pts[1].data_ptr()), _C.c_void_p(pts[2].data_ptr()),
        b1, n1, b2, n2, i0, h, EPS, 32, _C.c_void_p(Ub.data_ptr()), _C.c_void_p(Vb.data_ptr()),
        _C.c_void_p(info.data_ptr()), None))
    Psym = G.fibonacci_sphere(16384)
    Hy = A.HMatrix(Psym, "bbx", bmin=BMIN, eta=ETA, symmetric=True)
    Hy.matgenGeH_omp(A.mean_nn(Psym), EPS)
    Xs = torch.from_numpy(rng.uniform(-1.0, 1.0, (16, Hy.n))).to(dev)
    Hy.mltaGeHVec(1.0, Xs, torch.zeros_like(Xs))
    Hy.mltaGeHVec(1.0, Xs, torch.zeros_like(Xs), precision="fp32")  # mirror images for the streams
    Hy.close()
    Pa = G.fibonacci_sphere(4096)
    Ha = A.HMatrix(Pa, "bbx", bmin=BMIN, eta=ETA)
    Ha.matgenGeH_omp(A.mean_nn(Pa), EPS)
    Ha.agglH(EPS)
    Ha.close()
    Ha2 = A.HMatrix(Pa, "bbx", bmin=BMIN, eta=ETA)
    Ha2.helmholtz_assemble(5.0, A.mean_nn(Pa), EPS)
    Ha2.helm_agglH(EPS)
    Ha2.close()
    Pz = G.sphere_surface(16384, 17)
    Hz = A.HMatrix(Pz, "bbx", bmin=BMIN, eta=ETA)
    Hz.helmholtz_aca_ranks(16.2, A.mean_nn(Pz), EPS)
    Hz.helmholtz_assemble(16.2, A.mean_nn(Pz), EPS)
    for p in (16, 1):
        Xz = torch.from_numpy(rng.standard_normal((p, Hz.n)) + 1j * rng.standard_normal((p, Hz.n))).to(dev)
        for prec in ("fp64", "fp32"):
            Hz.mltaGeHVec(1.0, Xz, torch.zeros_like(Xz), precision=prec)
    xz1 = rng.standard_normal(Hz.n) + 1j * rng.standard_normal(Hz.n)
    Hz.mltaGeHhVec(1.0, xz1, np.zeros_like(xz1))  # the adjoint
    mats = []
    for i, m in enumerate((2048, 3000, 5000, 8000)):
        Pm = G.sphere_surface(m, 100 + i)
        Hm = A.HMatrix(Pm, "bbx", bmin=BMIN, eta=ETA)
        Hm.matgenGeH_omp(A.min_nn(Pm) / 2.0, EPS)
        mats.append(Hm)
    Bt = A.HBatch(mats, precision="bf16")
    xb = np.random.default_rng(4).standard_normal(Bt.n)
    Bt.matvec(1.0, xb, np.zeros(Bt.n))
    # solvers last: their graphs launch many small kernels
    H.close()
    b = np.random.default_rng(3).standard_normal(n)
    Hs = A.HMatrix(P, "bbx", bmin=BMIN, eta=ETA)
    Hs.matgenGeH_omp(h / 2.0, EPS)
    Hs.GMRes(b, np.zeros(n), 1e-8, 30, 30)
    Hs.GMRes(b, np.zeros(n), 1e-8, 30, 60, precision="fp32")
    Hs.CG(b, np.zeros(n), 1e-8, 30)
    Hs.spctrlnrm(3)
    Hs.close()
    zb = np.random.default_rng(12).standard_normal(Hz.n) + 1j * np.random.default_rng(13).standard_normal(Hz.n)
    Hz.GMRes(zb, np.zeros_like(zb), 1e-8, 30, 20)
    Hz.GMRes(zb, np.zeros_like(zb), 1e-8, 30, 20, precision="fp32")  # complex refinement
    Hz.close()
    Bt.gmres(xb, np.zeros(Bt.n), 1e-8, 30, 60)
    Bt.close()
    torch.cuda.synchronize()
    print(json.dumps({"workload": f"kernels-sphere-{n}", "ok": True}))


# ---------------------------------------------------------------------------
# Headline workload: N = 1,048,576 uniform random points on the unit-cube surface
# (seed 4), Laplace kernel, bounding-box tree, leaf 64, eta 0.8, ACA eps 1e-6,
# 64 right-hand sides; products, and GMRES(50) to a 1e-8 FP64 residual.
HL_N, HL_P, HL_LEAF = 1 << 20, 64, 64
HEADLINE = {
    "workload": "laplace-cube-1048576-64rhs",
    "points": "uniform random points on the unit-cube surface (numpy PCG64 seed 4)",
    "n": HL_N, "rhs": HL_P, "tree": "bbx", "leaf": HL_LEAF, "eta": ETA, "eps": EPS,
    "kernel": "1/(4 pi r)",
    "diag": "1/(4 pi h), h = smallest nearest-neighbour distance / 2 (with the mean spacing the "
            "matrix of a random cloud is indefinite and GMRES stagnates)",
    "x": "X ~ U[-1, 1] (seed 5)",
    "gmres": "GMRES(50) to a 1e-8 relative FP64 residual, b ~ N(0, 1) (seed 6)",
    "l2": "inputs larger than L2 (no flush)",
}
METRIC_HL = "H-matvec/s & GMRES solves/s"


def _min_nn_host(P):
    """Smallest nearest-neighbour distance (host, scipy k-d tree): the CPU arm sets
    h without the library."""
    from scipy.spatial import cKDTree

    d, _ = cKDTree(P).query(P, k=2)
    return float(d[:, 1].min())


def cpu_sample(n, p, leaf, steps, warmup, threads, frac=8, seed=9):
    """The reference path on the host cores, on a bounded sample of the headline
    matrix: 1/frac of its leaves (uniform random, seeded) assembled by the oracle
    (apprx_unsym per leaf), multiplied with the reference's BLAS calls per leaf
    (mltaGeM_, H/mblock.cpp:141-154) by OpenMP threads sharing row-disjoint leaf
    groups.  The product cost is a sum over leaves, so the full product's time is
    the sample's times frac.  GMRES per right-hand side (solvers/GMRES.cpp:80-181)
    costs per step one single-vector product and the Gram-Schmidt work of the
    step (timed on full-length vectors, averaged over a 50-step cycle)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from ahmed_gb300 import geometry as G

    P = G.cube_surface(n, 4)
    h = _min_nn_host(P) / 2
    Ho = O.OracleH(P, O.TREE_BBX, leaf, ETA, h)
    lv = Ho.leaves()
    nl = len(lv)
    sel = np.sort(np.random.default_rng(seed).choice(nl, nl // frac, replace=False))
    blas = O.use_host_blas()
    t0 = time.perf_counter()
    Ho.assemble_list(sel, EPS, nthreads=threads)
    t_asm = time.perf_counter() - t0
    plan = O.layered_groups(lv, sel)
    scale = nl / len(sel)
    X = np.random.default_rng(5).uniform(-1.0, 1.0, (p, n))
    Y = np.zeros_like(X)
    for _ in range(max(1, warmup)):
        Ho.matvec_layers(plan, X, Y, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        Ho.matvec_layers(plan, X, Y, nthreads=threads)
    t_prod = (time.perf_counter() - t0) / steps
    x1 = X[0].copy()
    y1 = np.zeros(n)
    Ho.matvec_layers(plan, x1, y1, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(3):
        Ho.matvec_layers(plan, x1, y1, nthreads=threads)
    t_prod1 = (time.perf_counter() - t0) / 3
    # Gram-Schmidt of a 50-step cycle: step i takes i + 1 dots and axpys over n
    V = np.random.default_rng(1).standard_normal((26, n))
    w = np.random.default_rng(2).standard_normal(n)
    t0 = time.perf_counter()
    for i in range(25):
        w -= (V[i] @ w) * V[i]
    np.linalg.norm(w)
    t_orth = (time.perf_counter() - t0) / 25 * 25.5  # mean step of the cycle: 25.5 vectors
    return {"products_per_s": p / (t_prod * scale), "product_s_full": t_prod * scale,
            "product1_s_full": t_prod1 * scale, "gmres_step_s": t_prod1 * scale + t_orth,
            "assembly_s_sample": t_asm, "assembly_s_full_estimate": t_asm * scale,
            "sample_leaves": int(len(sel)), "leaves": int(nl), "scale": scale, "blas": blas,
            "cores": threads}


def _cpu_desc(c, steps):
    return (f"{c['sample_leaves']} of the {c['leaves']} leaves of the same matrix (1/{c['scale']:.0f}, uniform "
            f"random, seed 9) assembled by the oracle and multiplied {steps} times with 64 right-hand "
            f"sides (reference BLAS calls per leaf: {c['blas'] or 'C loops'}); the full product's time is "
            f"the sample's x {c['scale']:.2f}")


def run_reference_headline(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    c = cpu_sample(HL_N, HL_P, HL_LEAF, max(1, args.steps), max(1, args.warmup // 3), threads)
    val = c["products_per_s"]
    line = {
        "impl": "reference", "metric": METRIC_HL, "value": val, "unit": "vector products/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": c["product_s_full"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": dict(HEADLINE),
        "cpu_baseline": {"value": val, "unit": "vector products/s", "cores": threads, "kind": "port",
                         "sample": _cpu_desc(c, args.steps)},
        "e2e": {"value": val, "unit": "vector products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "details": {"cpu": c},
    }
    print(json.dumps(line))


def _kernel_bytes(H, p):
    """Algorithmic bytes of the two FP32 sweeps of one product: V sweep = V factors
    + X read; rows sweep = U factors + dense leaves + Y read and written (FP64)."""
    lv = H.leaves()
    r = H.ranks()
    n1, n2 = lv[:, 1].astype(np.int64), lv[:, 3].astype(np.int64)
    lr = r > 0
    v = 4 * int((n2[lr] * r[lr]).sum())
    u = 4 * int((n1[lr] * r[lr]).sum())
    d = 4 * int((n1[r < 0] * n2[r < 0]).sum())
    return {"v_sweep": v + 8 * p * H.n, "rows_sweep": u + d + 16 * p * H.n}


def run_headline(args):
    import torch
    import ahmed_gb300 as A
    from ahmed_gb300 import _capi

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, p = HL_N, HL_P
    P = A.geometry.cube_surface(n, 4)
    t0 = time.perf_counter()
    h = A.min_nn(P) / 2
    H = A.HMatrix(P, "bbx", bmin=HL_LEAF, eta=ETA, device=local)
    t_tree = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    H.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    H.matgenGeH_omp(h, EPS)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    ranks = H.ranks()
    L = _capi.lib()
    X = torch.from_numpy(np.random.default_rng(5).uniform(-1.0, 1.0, (p, n))).to(dev)
    Y = torch.zeros_like(X)
    t0 = time.perf_counter()
    H.prepare("fp32")
    torch.cuda.synchronize()
    t_prep32 = time.perf_counter() - t0
    H.prepare("fp64")
    launches = {}

    def timed(prec, steps, warmup, kernel_times=False):
        for _ in range(warmup):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ms2, cnt2 = np.zeros(2), np.zeros(2, np.uint64)
        if kernel_times:
            L.ahx_timing_read(ms2.ctypes.data, cnt2.ctypes.data, 1)
            L.ahx_timing(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = L.ahx_kernel_launches()
        e0.record(stream)
        for _ in range(steps):
            H.mltaGeHVec(1.0, X, Y, precision=prec)
        e1.record(stream)
        torch.cuda.synchronize()
        launches[prec] = int(L.ahx_kernel_launches() - l0)
        ms = e0.elapsed_time(e1)
        if kernel_times:
            L.ahx_timing_read(ms2.ctypes.data, cnt2.ctypes.data, 1)
            L.ahx_timing(0)
        ms = replica_max_ms(ms, ws, dev)
        return ms / steps, (ms2 / np.maximum(cnt2, 1), cnt2)

    with ClockSampler(local) as cs:
        ms32, (kms, kcnt) = timed("fp32", args.steps, args.warmup, kernel_times=True)
    clocks = cs.summary()
    ms64, _ = timed("fp64", 2, 1)
    Y64 = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Y64, precision="fp64")
    Y32 = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Y32, precision="fp32")
    torch.cuda.synchronize()
    err32 = float(((Y32 - Y64).norm(dim=1) / Y64.norm(dim=1)).max())
    del Y32
    # end to end through the public API: pinned host X and Y, copies inside the timed region
    Xh = torch.from_numpy(np.random.default_rng(5).uniform(-1.0, 1.0, (p, n))).pin_memory()
    Yh = torch.zeros_like(Xh).pin_memory()
    for _ in range(2):
        H.mltaGeHVec(1.0, Xh.numpy(), Yh.numpy(), precision="fp32")
    torch.cuda.synchronize()
    ne2e = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(ne2e):
        H.mltaGeHVec(1.0, Xh.numpy(), Yh.numpy(), precision="fp32")
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / ne2e
    # BF16 factors beside it (the C5 storage of the task), with its error per right-hand side
    H.release("fp32")
    t0 = time.perf_counter()
    H.prepare("bf16")
    torch.cuda.synchronize()
    t_prepb = time.perf_counter() - t0
    msb, _ = timed("bf16", max(3, args.steps // 2), 2)
    Yb = torch.zeros_like(X)
    H.mltaGeHVec(1.0, X, Yb, precision="bf16")
    torch.cuda.synchronize()
    errb = float(((Yb - Y64).norm(dim=1) / Y64.norm(dim=1)).max())
    del Yb, Y64, Y
    # GMRES(50) to 1e-8: mixed (inner solves on the FP32-class tcgen05 product or on
    # BF16 factors, FP64 refinement) and plain FP64, 3 solves each
    B = torch.from_numpy(np.random.default_rng(6).standard_normal((p, n))).to(dev)
    gm = {}
    H.prepare("fp32")
    for prec in ("fp32", "bf16", "fp64"):
        runs = []
        for _ in range(args.gmres_solves):
            Xs = torch.zeros_like(B)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st, rr, its = H.GMRes(B, Xs, 1e-8, 50, args.gmres_cap, precision=prec)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            R = B.clone()
            H.mltaGeHVec(-1.0, Xs, R, precision="fp64")
            true = float((R.norm(dim=1) / B.norm(dim=1)).max())
            runs.append({"s": dt, "converged": st == 0, "max_iters": int(its.max()),
                         "true_max_resid": true})
            del Xs, R
        secs = sorted(r["s"] for r in runs)
        med = secs[len(secs) // 2]
        ok = all(r["converged"] and r["true_max_resid"] <= 1e-8 for r in runs)
        gm[prec] = {"median_s": med, "solves_per_s": (p / med) if ok else None, "runs": runs}
    if gm["fp32"]["solves_per_s"] and gm["fp64"]["solves_per_s"]:
        gm["mixed_over_plain"] = gm["fp32"]["solves_per_s"] / gm["fp64"]["solves_per_s"]
    if gm["bf16"]["solves_per_s"] and gm["fp64"]["solves_per_s"]:
        gm["mixed_bf16_over_plain"] = gm["bf16"]["solves_per_s"] / gm["fp64"]["solves_per_s"]
    peak, peak_kind = _peaks()
    kb = _kernel_bytes(H, p)
    total_alg = H.storage_bytes("fp64") // 2 + p * n * 24  # FP32 payload + X read + Y read and written
    dom = 1 if kms[1] >= kms[0] else 0
    dom_bytes = kb["rows_sweep"] if dom == 1 else kb["v_sweep"]
    achieved = dom_bytes / (kms[dom] * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("umma_rows_sweep_fp32_64rhs_cube1048576")
        except Exception:
            traffic = None
    value = ws * p / (ms32 * 1e-3)
    line = {
        "metric": METRIC_HL, "value": value, "unit": "vector products/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": dict(HEADLINE),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": ("um_sweep_kernel rows sweep" if dom == 1 else "um_sweep_kernel V sweep"),
                     "kernel_ms": float(kms[dom]), "kernel_algorithmic_bytes": dom_bytes,
                     "step": {"algorithmic_bytes": total_alg, "achieved": total_alg / (ms32 * 1e-3) / 1e9,
                              "frac": total_alg / (ms32 * 1e-3) / 1e9 / peak}},
        "e2e": {"value": ws * p / e2e_s, "unit": "vector products/s", "h2d_bytes_per_step": p * n * 16,
                "d2h_bytes_per_step": p * n * 8},
        "gpu_launches": launches.get("fp32"),
        "clocks": clocks,
        "gmres": {"mixed_fp32_solves_per_s": gm["fp32"]["solves_per_s"],
                  "mixed_bf16_solves_per_s": gm["bf16"]["solves_per_s"], "plain_fp64_solves_per_s":
                  gm["fp64"]["solves_per_s"], "mixed_over_plain": gm.get("mixed_over_plain"),
                  "mixed_bf16_over_plain": gm.get("mixed_bf16_over_plain"),
                  "restart": 50, "tol": 1e-8, "diag": "h = smallest nearest-neighbour distance / 2",
                  "detail": gm},
        "details": {"tree_s": t_tree, "assembly_s": t_asm, "leaves": int(H.nleaves),
                    "lowrank_leaves": int((ranks >= 0).sum()), "avg_rank": float(ranks[ranks >= 0].mean()),
                    "fp64_leaf_bytes": int(H.storage_bytes("fp64")), "fp32_prepare_s": t_prep32,
                    "bf16_prepare_s": t_prepb, "fp32_max_rel_err_per_rhs": err32,
                    "plain_fp64_ms": ms64, "fp32_over_fp64_product": ms64 / ms32,
                    "bf16_ms": msb, "bf16_max_rel_err_per_rhs": errb,
                    "sweep_ms": {"v": float(kms[0]), "rows": float(kms[1])}, "sweep_bytes": kb},
    }
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        c = cpu_sample(n, p, HL_LEAF, 3, 1, threads)
        line["cpu_baseline"] = {"value": c["products_per_s"], "unit": "vector products/s", "cores": threads,
                                "kind": "port", "sample": _cpu_desc(c, 3),
                                "gmres_solves_per_s_estimate": 1.0 / (c["gmres_step_s"] * gm["fp64"]["runs"][0]["max_iters"]),
                                "gmres_step_s": c["gmres_step_s"]}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ahx", choices=["ahx", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--autotune", type=int, default=1, help="1: tune the stream bucketing before timing")
    ap.add_argument("--n", type=int, default=N_POINTS,
                    help="number of points (smaller cases are for profiling only)")
    ap.add_argument("--workload", default="headline",
                    choices=["headline", "sphere", "cube-large", "batch", "product", "predictor", "helmholtz",
                             "zhmat", "aggl", "kernels"],
                    help="headline (default): N = 2^20 cube surface, leaf 64, 64 right-hand sides, FP32 "
                         "products on the tensor cores and GMRES(50); sphere: N = 65,536 sphere, 16 "
                         "right-hand sides; cube-large: the same N = 2^20 workload with BF16 factors; "
                         "batch: 256 uneven instances, one launch per product, batched GMRES")
    ap.add_argument("--gmres-solves", type=int, default=3, help="headline: timed GMRES solves per form (median)")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--geometry", default="sphere", choices=["sphere", "cube"], help="product workload")
    ap.add_argument("--leaf", type=int, default=BMIN, help="product workload")
    ap.add_argument("--rhs", type=int, default=NRHS, help="product workload")
    ap.add_argument("--symmetric", action="store_true",
                    help="product / zhmat workloads: symmetric block tree (upper blocks once)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "bf16", "fp64", "df64"], help="product workload")
    ap.add_argument("--n-large", type=int, default=1 << 20)
    ap.add_argument("--diag", default="mean", choices=["mean", "min"],
                    help="cube-large / batch: h = mean (configured) or minimum nearest-neighbour "
                         "distance (random clouds: positive definite, GMRES converges)")
    ap.add_argument("--diag-scale", type=float, default=1.0,
                    help="cube-large / batch: diagonal 1/(4 pi h / s)")
    ap.add_argument("--gmres-cap", type=int, default=600)
    ap.add_argument("--gmres-cap-fp64", type=int, default=600)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.n != N_POINTS:
        set_size(args.n)
    if args.impl == "reference":
        if args.workload == "sphere":
            run_reference(args)
        else:
            run_reference_headline(args)
    elif args.workload == "headline":
        run_headline(args)
    elif args.workload == "cube-large":
        run_large(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "product":
        run_product(args)
    elif args.workload == "predictor":
        run_predictor(args)
    elif args.workload == "helmholtz":
        run_helmholtz(args)
    elif args.workload == "zhmat":
        run_zhmat(args)
    elif args.workload == "aggl":
        run_aggl(args)
    elif args.workload == "kernels":
        run_kernels(args)
    else:
        run_gpu(args)  # sphere


if __name__ == "__main__":
    main()
