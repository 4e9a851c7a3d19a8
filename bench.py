"""H-matrix-vector product benchmark (one JSON line on stdout).

Workload (the headline configuration): N = 2^20 cell centres of a 1024 x 1024 x 1
thin-film grid, spacing 1 (coordinates in nm), Gaussian jitter sigma = 0.05
spacing on every coordinate (seeded), Laplace kernel 1/(4 pi r) with G(x,x) = 0,
leaf size 64, admissibility eta = 2 (the reference's dist > eta (rX + rY)), ACA+
tolerance 1e-4 with SVD recompression, assembled on the device.  One step is one
product y = H x with x ~ N(0,1) (FP32 storage and arithmetic, 1 right-hand side).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`value` is products per second over the whole job with x already in HBM;
`e2e` is the same through the public API on pinned host buffers (x copied in,
y copied out every step).  The reference arm (--impl reference) times the
reference's CPU product (src/mult.jl:6-32) restated by the oracle, on all host
cores, over the same whole matrix assembled by the oracle.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "hmatrixgpu.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "H-matvec/s at N=2^20, 1 & 32 RHS: mixed vs plain FP32 at equal err; HBM GB/s"
WORKLOAD = "film-2^20 Laplace leaf64 eta2 tol1e-4, 1 RHS, FP32 storage"
GRID, LEAF, ETA, TOL = 1024, 64, 2.0, 1e-4
# DRAM traffic / algorithmic bytes of the near/U kernel, from an ncu capture on
# film 512 x 512 (1983.5 MB of dram__bytes_read + write for 1952.3 MB algorithmic)
TRAFFIC_RATIO = 1983.5 / 1952.3


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_samples(self, k, timeout_s):
        """Waits until k samples have arrived (or the timeout runs out)."""
        t0 = time.time()
        while self.proc is not None and len(self.lines) < k and time.time() - t0 < timeout_s:
            time.sleep(0.02)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def film_points():
    from tests import geometry
    return geometry.film(GRID, GRID, spacing=1.0, jitter=0.05, seed=1)


def set_grid(g):
    """A smaller film (g x g) for profiling captures; the headline is g = 1024."""
    global GRID, WORKLOAD
    GRID = g
    if g != 1024:
        WORKLOAD = WORKLOAD.replace("film-2^20", f"film-{g}x{g}")


def batch_measurement(dev, steps):
    """32 independent H-matrices (unit-sphere surfaces, N log-uniform in
    [8192, 131072], Yukawa exp(-r)/r, leaf 32, eta 1.5, tol 1e-5, FP32), one
    product each: one product per member in turn, the block-diagonal batch
    (one launch per kernel for all members) and the batch replayed from a CUDA
    graph. Returns the per-product figures."""
    import torch

    import hmgpu
    from tests import geometry
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(8192), np.log(131072), 32)).astype(int)
    t0 = time.time()
    members = []
    for i, N in enumerate(sizes):
        P = geometry.sphere(int(N), seed=100 + i)
        T = hmgpu.ClusterTree(P, max_points_per_leaf=32, gpu=True)
        members.append(hmgpu.HMatrix(hmgpu.Kernel("yukawa", P), T, T, eta=1.5, eps=1e-5, precision="f32"))
    B = hmgpu.batch(members)
    build = time.time() - t0
    tune = B.autotune()  # the batch's own unit sizes and V schedule
    m, n = B.shape
    x = torch.randn(n, device=dev, generator=torch.Generator(dev).manual_seed(5))
    y = torch.empty(m, device=dev)
    offs = np.concatenate([[0], np.cumsum([H.shape[1] for H in members])])
    xs = [x[offs[k]:offs[k + 1]] for k in range(len(members))]
    ys = [y[offs[k]:offs[k + 1]] for k in range(len(members))]
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        s.record(stream)
        for _ in range(reps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps

    reps = max(20, min(steps, 200))
    t_each = timed(lambda: [hmgpu.mul_(ys[k], members[k], xs[k]) for k in range(len(members))], reps)
    y_each = y.clone()
    t_batch = timed(lambda: hmgpu.mul_(y, B, x), reps)
    same = bool(torch.equal(y, y_each))
    G = hmgpu.Graph(B, x, y)
    t_graph = timed(lambda: G.launch(), reps)
    import ctypes as C
    L = hmgpu._lib.lib()
    hmgpu.check(L.hmgpu_hmatrix_set_profiling(B._h, 1))
    for _ in range(reps):
        hmgpu.mul_(y, B, x)
    ph = np.zeros(3)
    nl, npd = C.c_int64(), C.c_int64()
    hmgpu.check(L.hmgpu_hmatrix_phase_times(B._h, hmgpu.ptr(ph), C.byref(nl), C.byref(npd)))
    hmgpu.check(L.hmgpu_hmatrix_set_profiling(B._h, 0))
    ph = ph / max(npd.value, 1)
    inf = B.info()
    byts = 4 * (inf["dense_entries"] + inf["far_entries"]) + 4 * (2 * n + 2 * inf["total_rank"])
    _, a = B.blocks()
    u_entries = int(((a[:, 1] - a[:, 0] + 1) * a[:, 4]).sum()) if len(a) else 0
    du_b = 4 * (inf["dense_entries"] + u_entries) + 4 * (2 * n + inf["total_rank"])
    v_b = 4 * (inf["far_entries"] - u_entries) + 4 * inf["total_rank"]
    return {"workload": "32 sphere H-matrices, N log-uniform in [8192, 131072] (total %d), Yukawa, "
                        "leaf 32, eta 1.5, tol 1e-5, FP32, 1 RHS each" % int(sizes.sum()),
            "ms_members_one_by_one": t_each, "ms_batch": t_batch, "ms_batch_cuda_graph": t_graph,
            "products_per_s_batch_graph": 32e3 / t_graph,
            "speedup_batch_graph_vs_one_by_one": t_each / t_graph,
            "batch_equals_members_bitwise": same, "algorithmic_gbs_batch_graph": byts / (t_graph * 1e-3) / 1e9,
            "phases_ms": {"permute": ph[0], "v_pass": ph[1], "near_u_pass": ph[2]}, "autotuned": tune,
            "v_pass_gbs": v_b / (ph[1] * 1e-3) / 1e9, "near_u_gbs": du_b / (ph[2] * 1e-3) / 1e9,
            "dense_entries": inf["dense_entries"], "far_entries": inf["far_entries"],
            "build_seconds": build}


def cpu_product(runs):
    """The reference's CPU product (src/mult.jl:6-32) on the workload's whole
    H-matrix. The oracle assembles the matrix (FP64, ACA+ and recompression on
    all host cores; about 24 GB for the headline film); then, for each
    (threads, warm-up, steps) in `runs`, whole products y = H x run back to
    back, each with its own permutation of x, block gemvs and scatter
    (oracle/cpu_mul.c). Returns ({threads: figures}, description)."""
    from oracle import oracle as O
    P = film_points()
    t0 = time.time()
    T = O.Tree(P.T, LEAF)
    K = O.Kernel("laplace", P.T, P.T)
    cores = os.cpu_count() or 1
    H = O.HMatrix(K, T, T, eta=ETA, eps=TOL, nthreads=cores)
    build_s = time.time() - t0
    x = np.random.default_rng(0).standard_normal(H.n)
    entries = H.stored_entries()
    y_check = H.mul(x)  # the checker's sequential product on the same matrix
    out = {}
    for th, warm, steps in runs:
        cp = H.timed_product(th)
        if warm:
            cp.run(x, warm)
        dt, y = cp.run(x, steps)
        out[th] = {"value": steps / dt, "unit": "matvec/s", "cores": th, "steps": steps, "warmup": warm,
                   "seconds": dt, "ms_per_step": 1e3 * dt / steps, "gbs": 8.0 * entries * steps / dt / 1e9,
                   "rel_diff_vs_checker": float(np.linalg.norm(y - y_check) / np.linalg.norm(y_check))}
        del cp
    desc = (f"the whole matrix ({H.nD} dense + {H.nA} low-rank blocks, {entries:.3e} FP64 entries, "
            f"{8 * entries / 1e9:.1f} GB), assembled by the oracle on {cores} cores in {build_s:.0f} s; "
            f"every step one whole product (x permuted, one gemv per dense block, two per low-rank block, "
            f"y scattered)")
    del H
    return out, desc


def bench_config(n):
    """The workload as both arms name it."""
    return {"workload": WORKLOAD, "N": n, "leaf": LEAF, "eta": ETA, "tol": TOL, "nrhs": 1,
            "l2": "inputs larger than L2: the factors streamed per step are many times the 129 MB L2",
            "parallelism": "1 GPU"}


def film_tight_measurement(dev, steps, hbm, P, T, tol=1e-6):
    """The headline film at the tighter tolerance the precision case also names
    (tol 1e-6, same points, tree, leaf 64 and eta 2): the 1-RHS FP32 product
    (time, algorithmic GB/s, error against the FP64 H-matrix) and 32 RHS plain
    FP32 against mixed precision, errors against the FP64 product of the same
    32 vectors."""
    import torch

    import hmgpu
    n = P.shape[1]
    K = hmgpu.Kernel("laplace", P)
    t0 = time.time()
    H = hmgpu.HMatrix(K, T, T, eta=ETA, eps=tol, precision="f32")
    torch.cuda.synchronize()
    build = time.time() - t0
    tune = H.autotune()
    inf = H.info()
    g = torch.Generator(dev).manual_seed(21)
    x = torch.randn(n, device=dev, generator=g)
    X = torch.randn(32, n, device=dev, generator=g).t()
    H64 = hmgpu.HMatrix(K, T, T, eta=ETA, eps=tol, precision="f64")
    y64 = H64 * x.double()
    Y64 = torch.empty(32, n, dtype=torch.float64, device=dev).t()
    hmgpu.mul_(Y64, H64, X.double())
    del H64
    y = torch.empty(n, device=dev)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        hmgpu.mul_(y, H, x)
    reps = max(10, min(steps, 200))
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        hmgpu.mul_(y, H, x)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / reps
    err1 = float(torch.linalg.norm(y.double() - y64) / torch.linalg.norm(y64))
    alg = 4 * (inf["dense_entries"] + inf["far_entries"] + 2 * n + 2 * inf["total_rank"])
    out = {"workload": f"film-{GRID}x{GRID} Laplace leaf{LEAF} eta{ETA:g} tol{tol:g}",
           "build_seconds": build, "autotuned": tune, "dense_entries": inf["dense_entries"],
           "far_entries": inf["far_entries"], "max_rank": inf["max_rank"],
           "f32_1rhs": {"ms_per_product": ms, "matvec_per_s": 1e3 / ms, "hbm_gbs": alg / (ms * 1e-3) / 1e9,
                        "frac_of_measured": alg / (ms * 1e-3) / 1e9 / hbm, "rel_err_vs_fp64_hmatrix": err1}}
    Hm = hmgpu.HMatrix(K, T, T, eta=ETA, eps=tol, precision="mixed")
    Y = torch.empty(32, n, device=dev).t()
    rhs = {"errors": "max over the 32 columns of ||y - y64|| / ||y64||"}
    for name, HH in (("plain_f32", H), ("mixed_tensor_cores", Hm)):
        for _ in range(3):
            hmgpu.mul_(Y, HH, X)
        r32 = max(5, min(steps // 10, 30))
        torch.cuda.synchronize()
        s.record()
        for _ in range(r32):
            hmgpu.mul_(Y, HH, X)
        e.record()
        torch.cuda.synchronize()
        t32 = s.elapsed_time(e) / r32
        err = float(((Y.double() - Y64).norm(dim=0) / Y64.norm(dim=0)).max())
        rhs[name] = {"ms_per_32rhs_product": t32, "matvec_per_s": 32e3 / t32, "rel_err": err}
    rhs["mixed_speedup_vs_plain_f32"] = rhs["plain_f32"]["ms_per_32rhs_product"] / \
        rhs["mixed_tensor_cores"]["ms_per_32rhs_product"]
    out["rhs32"] = rhs
    del Hm, H
    torch.cuda.empty_cache()
    return out


def cube_measurement(dev, steps, hbm, npts=1 << 18):
    """The plain drop-in case: N = 2^18 points uniform in [0,1]^3, Laplace
    1/(4 pi r), leaf 64, eta 2, tol 1e-6, FP32 storage, one RHS. Device build
    (trees included), autotuned layout, product time with its phases, the
    passes' bandwidth against the measured peak, and the error of 256 rows of y
    against the exact kernel sums (FP64 on the host)."""
    import torch

    import hmgpu
    from tests import geometry
    P = geometry.cube(npts, seed=2)
    n = P.shape[1]
    t0 = time.time()
    T = hmgpu.ClusterTree(P, max_points_per_leaf=64, gpu=True)
    H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision="f32")
    torch.cuda.synchronize()
    build = time.time() - t0
    tune = H.autotune()
    x = torch.randn(n, device=dev, generator=torch.Generator(dev).manual_seed(11))
    y = torch.empty(n, device=dev)
    for _ in range(3):
        hmgpu.mul_(y, H, x)
    lib = hmgpu._lib.lib()
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H._h, 1))
    stream = torch.cuda.current_stream(dev)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(10, min(steps // 5, 100))
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(reps):
        hmgpu.mul_(y, H, x)
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / reps
    import ctypes as C
    ph = np.zeros(3)
    nl, npd = C.c_int64(), C.c_int64()
    hmgpu.check(lib.hmgpu_hmatrix_phase_times(H._h, hmgpu.ptr(ph), C.byref(nl), C.byref(npd)))
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H._h, 0))
    ph = ph / max(npd.value, 1)
    inf = H.info()
    R = inf["total_rank"]
    d, a = H.blocks()
    u_entries = int(((a[:, 1] - a[:, 0] + 1) * a[:, 4]).sum()) if len(a) else 0
    v_entries = inf["far_entries"] - u_entries
    alg = 4 * (inf["dense_entries"] + inf["far_entries"]) + 4 * (2 * n + 2 * R)
    du_b = 4 * (inf["dense_entries"] + u_entries) + 4 * (2 * n + R)
    v_b = 4 * v_entries + 4 * R
    rows = np.random.default_rng(12).choice(n, 256, replace=False)
    xs = x.double().cpu().numpy()
    ys = y.double().cpu().numpy()
    Pt = P.T
    exact = np.empty(len(rows))
    for k, i in enumerate(rows):  # K(x_i, x_j) = 1/(4 pi r), 0 at r = 0
        r = np.linalg.norm(Pt - Pt[i], axis=1)
        w = np.zeros(n)
        nz = r > 0
        w[nz] = 1.0 / (4.0 * np.pi * r[nz])
        exact[k] = w @ xs
    err = float(np.linalg.norm(ys[rows] - exact) / np.linalg.norm(exact))

    # 64 right-hand sides (the tensor-core batching case): plain FP32 passes
    # on the CUDA cores against a mixed-precision copy on the tensor cores,
    # both checked on the same 256 rows against exact kernel sums
    X = torch.randn(64, n, device=dev, generator=torch.Generator(dev).manual_seed(13)).t()
    Y = torch.empty(64, n, device=dev).t()
    Xh = X.double().cpu().numpy()
    exact64 = np.empty((len(rows), 64))
    for k, i in enumerate(rows):
        r = np.linalg.norm(Pt - Pt[i], axis=1)
        w = np.zeros(n)
        nz = r > 0
        w[nz] = 1.0 / (4.0 * np.pi * r[nz])
        exact64[k] = w @ Xh
    rhs64 = {}
    Hm = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision="mixed")
    Hm.autotune()
    for name, HH in (("plain_f32", H), ("mixed_tensor_cores", Hm)):
        for _ in range(2):
            hmgpu.mul_(Y, HH, X)
        reps64 = max(3, min(steps // 50, 20))
        torch.cuda.synchronize()
        s.record(stream)
        for _ in range(reps64):
            hmgpu.mul_(Y, HH, X)
        e.record(stream)
        torch.cuda.synchronize()
        t64 = s.elapsed_time(e) / reps64
        Ys = Y.double().cpu().numpy()[rows]
        e64 = float(np.max(np.linalg.norm(Ys - exact64, axis=0) / np.linalg.norm(exact64, axis=0)))
        rhs64[name] = {"ms_per_64rhs_product": t64, "matvec_per_s": 64e3 / t64, "rel_err_256_exact_rows": e64}
    rhs64["mixed_speedup_vs_plain_f32"] = rhs64["plain_f32"]["ms_per_64rhs_product"] / \
        rhs64["mixed_tensor_cores"]["ms_per_64rhs_product"]
    del Hm

    # the same matrix stored in FP64 (the drop-in's FP64 mode), one RHS
    H64 = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision="f64")
    H64.autotune()
    x64, y64 = x.double(), torch.empty(n, dtype=torch.float64, device=dev)
    for _ in range(3):
        hmgpu.mul_(y64, H64, x64)
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H64._h, 1))
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(reps):
        hmgpu.mul_(y64, H64, x64)
    e.record(stream)
    torch.cuda.synchronize()
    ms64 = s.elapsed_time(e) / reps
    ph64 = np.zeros(3)
    hmgpu.check(lib.hmgpu_hmatrix_phase_times(H64._h, hmgpu.ptr(ph64), C.byref(nl), C.byref(npd)))
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H64._h, 0))
    ph64 = ph64 / max(npd.value, 1)
    b64 = 2 * alg  # every stored entry and vector entry in 8 bytes
    y64h = y64.cpu().numpy()
    f64 = {"ms_per_product": ms64, "matvec_per_s": 1e3 / ms64, "hbm_gbs": b64 / (ms64 * 1e-3) / 1e9,
           "frac_of_measured": b64 / (ms64 * 1e-3) / 1e9 / hbm,
           "phases_ms": {"permute": ph64[0], "v_pass": ph64[1], "near_u_pass": ph64[2]},
           "near_u_gbs": 2 * du_b / (ph64[2] * 1e-3) / 1e9, "v_pass_gbs": 2 * v_b / (ph64[1] * 1e-3) / 1e9,
           "stored_gb": H64.info()["matrix_bytes"] / 1e9,
           "rel_err_256_exact_rows": float(np.linalg.norm(y64h[rows] - exact) / np.linalg.norm(exact)),
           "rel_diff_vs_f32": float(np.linalg.norm(y64h - ys) / np.linalg.norm(y64h))}
    del H64
    return {"workload": f"cube-{npts} Laplace leaf64 eta2 tol1e-6, 1 RHS, FP32 storage",
            "build_seconds": build, "build": H.build_profile(), "autotuned": tune,
            "dense_entries": inf["dense_entries"], "far_entries": inf["far_entries"],
            "lowrank_blocks": inf["admissible_leaves"], "dense_blocks": inf["full_leaves"],
            "max_rank": inf["max_rank"], "ms_per_product": ms, "matvec_per_s": 1e3 / ms,
            "hbm_gbs": alg / (ms * 1e-3) / 1e9,
            "phases_ms": {"permute": ph[0], "v_pass": ph[1], "near_u_pass": ph[2]},
            "v_pass_gbs": v_b / (ph[1] * 1e-3) / 1e9, "near_u_gbs": du_b / (ph[2] * 1e-3) / 1e9,
            "near_u_frac_of_measured": du_b / (ph[2] * 1e-3) / 1e9 / hbm,
            "v_pass_frac_of_measured": v_b / (ph[1] * 1e-3) / 1e9 / hbm,
            "rel_err_256_exact_rows": err, "rhs64": rhs64, "f64_storage": f64}


def learned_measurement(dev):
    """The learned rank predictor at scale: N = 2^20 points uniform in [0,1]^3,
    Laplace, leaf 64, eta 2, tol 1e-4, FP32 storage. The MLP is trained on
    (block features, ACA rank) pairs from plain device ACA runs on smaller
    cube, film and sphere geometries (6000 to 65536 points, leaves of 32 and
    64, tol 1e-4 and 1e-6); the matrix is then
    assembled without and with it. Reported: assembly time and phases, ACA
    workspace, batches, blocks rerun after outgrowing their predicted cap (the
    misprediction rate), bitwise equality of the two products, the product
    time and the error of 256 rows against exact kernel sums. At tol 1e-6 the
    same cube would hold about four times the low-rank entries (about 500 GB),
    more than one GPU has, so only tol 1e-4 is run."""
    import torch

    import hmgpu
    from tests import geometry
    t0 = time.time()
    feats, ranks = [], []
    for Pg, leaf in ((geometry.cube(6000, seed=1), 32), (geometry.film(80, 80), 32), (geometry.sphere(6000, seed=2), 32),
                     (geometry.cube(1 << 16, seed=3), 64), (geometry.film(256, 256, seed=4), 64),
                     (geometry.sphere(1 << 16, seed=6), 64)):
        Tg = hmgpu.ClusterTree(Pg, max_points_per_leaf=leaf, gpu=True)
        for eps in (1e-4, 1e-6):
            Hg = hmgpu.HMatrix(hmgpu.Kernel("laplace", Pg), Tg, Tg, eta=2.0, eps=eps, precision="f32")
            f = hmgpu.block_features(Tg, Tg, 2.0, eps)
            a, _ = Hg.aca_ranks(len(f))
            feats.append(f)
            ranks.append(a.astype(np.float32))
            del Hg
    X = np.concatenate(feats)
    y = np.concatenate(ranks)
    model = hmgpu.RankModel(seed=1)
    loss = model.train(X, y, epochs=60, batch=512, lr=2e-3, seed=1)
    train_s = time.time() - t0
    P = geometry.cube(1 << 20, seed=5)
    n = P.shape[1]
    T = hmgpu.ClusterTree(P, max_points_per_leaf=64, gpu=True)
    x = torch.randn(n, device=dev, generator=torch.Generator(dev).manual_seed(17))
    out = {"workload": "cube-2^20 Laplace leaf64 eta2 tol1e-4, FP32 storage, 1 RHS",
           "training": {"samples": int(len(y)), "final_loss": float(loss), "seconds": train_s}}
    y_first = None
    for name, rm in (("plain", None), ("learned", model)):
        t1 = time.time()
        H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-4, precision="f32", rank_model=rm)
        torch.cuda.synchronize()
        build = time.time() - t1
        inf = H.info()
        yv = torch.empty(n, device=dev)
        for _ in range(3):
            hmgpu.mul_(yv, H, x)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record()
        for _ in range(10):
            hmgpu.mul_(yv, H, x)
        e.record()
        torch.cuda.synchronize()
        rec = {"build_seconds": build, "build": H.build_profile(), "aca_batches": inf["aca_batches"],
               "aca_workspace_gb": inf["aca_workspace_bytes"] / 1e9, "aca_reruns": inf["aca_reruns"],
               "aca_continued": inf["aca_continued"],
               "misprediction_rate": (inf["aca_reruns"] + inf["aca_continued"]) / max(1, inf["admissible_leaves"]),
               "restart_rate": inf["aca_reruns"] / max(1, inf["admissible_leaves"]),
               "lowrank_blocks": inf["admissible_leaves"], "dense_blocks": inf["full_leaves"],
               "stored_gb": inf["matrix_bytes"] / 1e9, "ms_per_product": s.elapsed_time(e) / 10}
        if y_first is None:
            y_first = yv.clone()
            rows = np.random.default_rng(18).choice(n, 256, replace=False)
            xs, ys, Pt = x.double().cpu().numpy(), yv.double().cpu().numpy(), P.T
            exact = np.empty(len(rows))
            for k, i in enumerate(rows):
                r = np.linalg.norm(Pt - Pt[i], axis=1)
                w = np.zeros(n)
                nz = r > 0
                w[nz] = 1.0 / (4.0 * np.pi * r[nz])
                exact[k] = w @ xs
            rec["rel_err_256_exact_rows"] = float(np.linalg.norm(ys[rows] - exact) / np.linalg.norm(exact))
        else:
            rec["product_equals_plain_bitwise"] = bool(torch.equal(yv, y_first))
        out[name] = rec
        del H
    out["workspace_ratio_learned_vs_plain"] = out["learned"]["aca_workspace_gb"] / max(out["plain"]["aca_workspace_gb"], 1e-9)
    out["build_ratio_learned_vs_plain"] = out["learned"]["build_seconds"] / out["plain"]["build_seconds"]
    return out


def run_reference(args):
    """The reference arm: the reference's CPU product (src/mult.jl:6-32),
    restated by the oracle (Julia is absent here and on the GPU host), on the
    whole headline matrix with every host core; `warmup` and `steps` whole
    products. One more short run on one core is reported beside it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    runs = [(threads, args.warmup, args.steps)]
    if threads > 1:
        runs.append((1, 1, 2))
    res, desc = cpu_product(runs)
    r = res[threads]
    line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": "matvec/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded film points, x ~ N(0,1))",
            "config": bench_config(GRID * GRID),
            "cpu_baseline": {"value": r["value"], "unit": "matvec/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "host_gbs": r["gbs"], "rel_diff_vs_checker": r["rel_diff_vs_checker"],
            "one_core": res.get(1),
            "e2e": {"value": r["value"], "unit": "matvec/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def replica_layout():
    """(world size, rank, local rank) of a torchrun launch; (1, 0, 0) without one.
    Every rank runs the whole workload on its own GPU (independent replicas: the
    product needs no exchange between GPUs)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(v, dist, device):
    """The largest of every rank's v, on every rank (v itself without dist)."""
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, seconds_per_product):
    """Whole-job products per second of `world` replicas, each taking
    `seconds_per_product` (the slowest rank's time) per product."""
    return world / seconds_per_product


def run_gpu(args):
    import torch

    import hmgpu

    world, rank, local = replica_layout()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    P = film_points()
    t0 = time.time()
    T = hmgpu.ClusterTree(P, max_points_per_leaf=LEAF, gpu=True)
    tree_s = time.time() - t0
    H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=ETA, eps=TOL, precision="f32")
    torch.cuda.synchronize()
    build_s = time.time() - t0
    build = {"seconds": build_s, "cluster_tree_s": tree_s, **{k + "_s": v for k, v in H.build_profile().items()}}
    inf = H.info()
    if args.build_only:  # assembly of the workload alone (for launch lists of the build)
        if rank == 0:
            print(json.dumps({"metric": "assembly seconds", "value": build_s, "unit": "s", "n_gpus": world,
                              "higher_is_better": False, "config": {"workload": WORKLOAD, "N": P.shape[1]},
                              "build": build, "lowrank_blocks": inf["admissible_leaves"],
                              "dense_blocks": inf["full_leaves"]}), flush=True)
        if dist:
            dist.destroy_process_group()
        return
    n = P.shape[1]
    x = torch.randn(n, device=dev, generator=torch.Generator(dev).manual_seed(rank))
    y = torch.empty(n, device=dev)
    stream = torch.cuda.current_stream(dev)

    tune = H.autotune()  # unit sizes and the multi-RHS threshold, timed on this matrix
    for _ in range(max(args.warmup, 3)):
        hmgpu.mul_(y, H, x)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    lib = hmgpu._lib.lib()
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H._h, 1))
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # clocks: the sampler's first line arrives before the timed loop starts;
    # the timed loop is short (tens of ms), so the same products go on, untimed,
    # until a few more samples of the loaded GPU are in
    with Clocks(local) as clk:
        clk.wait_samples(1, 3.0)
        torch.cuda.synchronize()
        s.record(stream)
        for _ in range(args.steps):
            hmgpu.mul_(y, H, x)
        e.record(stream)
        torch.cuda.synchronize()
        t_end = time.time() + 2.0
        k0 = len(clk.lines)
        while len(clk.lines) < k0 + 4 and time.time() < t_end:
            for _ in range(20):
                hmgpu.mul_(y, H, x)
            torch.cuda.synchronize()
    ms = s.elapsed_time(e) / args.steps
    import ctypes as C
    ph = np.zeros(3)
    nl, npd = C.c_int64(), C.c_int64()
    hmgpu.check(lib.hmgpu_hmatrix_phase_times(H._h, hmgpu.ptr(ph), C.byref(nl), C.byref(npd)))
    hmgpu.check(lib.hmgpu_hmatrix_set_profiling(H._h, 0))
    ph = ph / max(npd.value, 1)
    ms = max_over_ranks(ms, dist, dev)

    # end to end: pinned host x in, host y out, every step
    xh = torch.randn(n, generator=torch.Generator().manual_seed(rank + 7)).pin_memory()
    yh = torch.empty(n).pin_memory()
    xn, yn = xh.numpy(), yh.numpy()
    for _ in range(3):
        hmgpu.mul_(yn, H, xn)
    ksteps = max(10, min(args.steps, 200))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(ksteps):
        hmgpu.mul_(yn, H, xn)
    e2e_s = max_over_ranks((time.perf_counter() - t1) / ksteps, dist, dev)

    # accuracy of this step against an FP64 H-matrix product on the device
    H64 = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=ETA, eps=TOL, precision="f64")
    y64 = H64 * x.double()
    hmgpu.mul_(y, H, x)
    rel_err = float(torch.linalg.norm(y.double() - y64) / torch.linalg.norm(y64))

    # 32 right-hand sides: plain FP32 (CUDA cores) against mixed precision
    # (scaled FP16 hi/lo pairs on the tensor cores), same matrix, errors against the
    # FP64 product of the same 32 vectors
    rhs32 = None
    if not args.skip_rhs32:
        X = torch.randn(32, n, device=dev, generator=torch.Generator(dev).manual_seed(rank + 3)).t()
        Y64 = torch.empty(32, n, dtype=torch.float64, device=dev).t()
        hmgpu.mul_(Y64, H64, X.double())
        del H64
        Hm = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=ETA, eps=TOL, precision="mixed")
        Y = torch.empty(32, n, device=dev).t()
        rhs32 = {"nrhs": 32, "errors": "max over the 32 columns of ||y - y64|| / ||y64||"}
        for name, HH in (("plain_f32", H), ("mixed_tensor_cores", Hm)):
            for _ in range(3):
                hmgpu.mul_(Y, HH, X)
            reps = max(5, min(args.steps // 10, 50))
            torch.cuda.synchronize()
            s.record(stream)
            for _ in range(reps):
                hmgpu.mul_(Y, HH, X)
            e.record(stream)
            torch.cuda.synchronize()
            t32 = s.elapsed_time(e) / reps
            err = float(((Y.double() - Y64).norm(dim=0) / Y64.norm(dim=0)).max())
            rhs32[name] = {"ms_per_32rhs_product": t32, "matvec_per_s": 32e3 / t32, "rel_err": err}
        rhs32["mixed_speedup_vs_plain_f32"] = rhs32["plain_f32"]["ms_per_32rhs_product"] / \
            rhs32["mixed_tensor_cores"]["ms_per_32rhs_product"]
        rhs32["mixed_device_gb"] = Hm.info()["device_bytes"] / 1e9
        del Hm
        # lean mixed: only the tensor-core copy on the device; 1 RHS runs on
        # the tensor cores as well (error of the first column against FP64)
        Hl = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=ETA, eps=TOL, precision="mixed", lean=True)
        lean = {"device_gb": Hl.info()["device_bytes"] / 1e9}
        x1, y1 = X[:, 0].contiguous(), torch.empty(n, device=dev)
        for name, xx, yy in (("1rhs", x1, y1), ("32rhs", X, Y)):
            for _ in range(3):
                hmgpu.mul_(yy, Hl, xx)
            reps = max(5, min(args.steps // 10, 50))
            torch.cuda.synchronize()
            s.record(stream)
            for _ in range(reps):
                hmgpu.mul_(yy, Hl, xx)
            e.record(stream)
            torch.cuda.synchronize()
            yv = yy.reshape(n, -1).double()
            lean["ms_" + name] = s.elapsed_time(e) / reps
            lean["rel_err_" + name] = float(((yv - Y64[:, :yv.shape[1]]).norm(dim=0) / Y64[:, :yv.shape[1]].norm(dim=0)).max())
        rhs32["mixed_lean"] = lean
        del Hl
    else:
        del H64

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    hbm, src = peaks()
    # algorithmic bytes (FP32): near field + low-rank factors + vectors
    es = 4
    dense_b = inf["dense_entries"] * es
    far_b = inf["far_entries"] * es
    R = inf["total_rank"]
    vec_b = es * (2 * n + 2 * R)
    alg_bytes = dense_b + far_b + vec_b
    # the near/U pass: dense entries + U entries + y + gathered x and t
    d, a = H.blocks()
    u_entries = int(((a[:, 1] - a[:, 0] + 1) * a[:, 4]).sum()) if len(a) else 0
    du_bytes = (inf["dense_entries"] + u_entries) * es + es * (2 * n + R)
    du_ms = ph[2]
    achieved = du_bytes / (du_ms * 1e-3) / 1e9
    batch32 = None if args.skip_batch else batch_measurement(dev, args.steps)
    cube18 = None if args.skip_cube else cube_measurement(dev, args.steps, hbm, args.cube_points)
    film_tight = None if args.skip_film_tight else film_tight_measurement(dev, args.steps, hbm, P, T)
    learned = learned_measurement(dev) if args.learned else None
    cores = os.cpu_count() or 1
    cpu_runs, cpu_desc = cpu_product([(1, 1, 4)] + ([(cores, 3, 10)] if cores > 1 else []))
    value = job_rate(world, ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "matvec/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded film points, x ~ N(0,1))",
        "config": dict(bench_config(n), parallelism=f"replicas x{world}" if world > 1 else "1 GPU"),
        "precision": "f32", "autotuned": tune,
        "streamed_gb_per_step": inf["matrix_bytes"] / 1e9,
        "hbm_gbs": alg_bytes / (ms * 1e-3) / 1e9,
        "rel_err_vs_fp64_hmatrix": rel_err,
        "structure": {"dense_blocks": inf["full_leaves"], "lowrank_blocks": inf["admissible_leaves"],
                      "dense_entries": inf["dense_entries"], "far_entries": inf["far_entries"],
                      "total_rank": R, "max_rank": inf["max_rank"], "algorithmic_bytes": alg_bytes,
                      "stored_bytes": inf["matrix_bytes"], "build_seconds": build_s, "build": build},
        "phases_ms": {"permute": ph[0], "v_pass": ph[1], "near_u_pass": ph[2]},
        "roofline": {"bound": "hbm", "kernel": "du_rows_kernel<float,0> (near field + U t)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "frac_of_nominal_7900": achieved / 7900.0,
                     "peak_source": src, "algorithmic_bytes_per_launch": du_bytes,
                     "traffic": du_bytes * TRAFFIC_RATIO,
                     "traffic_source": "ncu dram__bytes_read+write of du_rows_kernel on film 512x512 "
                                       "(1983.5 MB for 1952.3 MB algorithmic), scaled by algorithmic bytes "
                                       "(profiles/du_rows_v_pass_film512.md)"},
        "cpu_baseline": {"value": cpu_runs[1]["value"], "unit": "matvec/s", "cores": 1, "kind": "port",
                         "sample": cpu_desc + f"; {cpu_runs[1]['steps']} timed products on one core",
                         "one_core": cpu_runs[1], "all_cores": cpu_runs.get(cores)},
        "e2e": {"value": job_rate(world, e2e_s), "unit": "matvec/s", "h2d_bytes_per_step": n * es,
                "d2h_bytes_per_step": n * es},
        "gpu_launches": int(nl.value),
        "rhs32": rhs32,
        "batch32": batch32,
        "cube18": cube18,
        "film_tol1e-6": film_tight,
        "learned_cube20": learned,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--grid", type=int, default=1024, help="film side (1024 = the headline workload)")
    ap.add_argument("--skip-rhs32", action="store_true", help="leave out the 32-RHS plain / mixed lines")
    ap.add_argument("--skip-batch", action="store_true", help="leave out the 32-H-matrix batch lines")
    ap.add_argument("--build-only", action="store_true", help="assemble the workload, print its build line, exit")
    ap.add_argument("--skip-cube", action="store_true", help="leave out the 2^18-cube tol 1e-6 line")
    ap.add_argument("--skip-film-tight", action="store_true", help="leave out the film tol 1e-6 line")
    ap.add_argument("--cube-points", type=int, default=1 << 18,
                    help="points of the cube case (2^18 = the plain drop-in workload; smaller for profiling captures)")
    ap.add_argument("--learned", action="store_true",
                    help="also assemble the 2^20 cube (tol 1e-4) without and with the learned rank predictor")
    args = ap.parse_args()
    set_grid(args.grid)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
