"""Benchmark: H-matvec/s at n = 2^20 Cauchy points (KernelMatrix), GB300.

Workload: K_ij = 1/(x_i - y_j), x_i = (i-1)/n + 1/(2n), y_j = (j-1)/n on [0,1),
n = 2^20, both lists reversed to the descending order the reference needs
(a = c = 1, b = d = 0), BLOCKRANK 20, BLOCKSIZE 80, compression in FP64.
A step is one matrix-vector product with b ~ N(0,1) resident in HBM; the
headline `value` is the FP32-storage form (factors and leaves FP32, FP64
compression), single right-hand side.  The plain FP64 product and the FP32
32/256-column forms are reported under "variants".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "hierarchicalmatrices.jl_gb300"))
sys.path.insert(0, REPO)

METRIC = "H-matvec/s & HBM GB/s at n=2^20 (FP32 batched vs FP64 plain, rel err<=1e-6)"
UNIT = "matvec/s"
N_DEFAULT = 1 << 20
L2_BYTES = 129 * 1024 * 1024


def grid_points(n):
    x = (np.arange(n, dtype=np.float64) / n + 1.0 / (2 * n))[::-1].copy()
    y = (np.arange(n, dtype=np.float64) / n)[::-1].copy()
    return x, y


def beta_points(n, seed, min_gap=1e-9):
    """x, y i.i.d. Beta(1/2, 1/2) on [0, 1] (clustered at both ends), sorted,
    consecutive gaps raised to at least min_gap, returned descending."""
    rng = np.random.default_rng(seed)
    out = []
    steps = np.arange(n, dtype=np.float64) * min_gap
    for _ in range(2):
        p = np.sort(rng.beta(0.5, 0.5, n))
        # p'_i = max(p_i, p'_{i-1} + g)  <=>  p'_i - i g = running max of p_j - j g
        p = np.maximum.accumulate(p - steps) + steps
        out.append(p[::-1].copy())
    return out[0], out[1]


def profiled_traffic(n):
    """DRAM bytes (read + write) per launch of the near-field kernel from the
    committed ncu summary of the n = 2^20 workload, or None."""
    if n != N_DEFAULT:
        return None
    p = os.path.join(REPO, "profiles", "expand_near_kernelmatrix_cauchy_n2p20_fp32.md")
    try:
        with open(p) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch"):
                    return float(ln.split("=")[1]) / 1e9
    except OSError:
        pass
    return None


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.4)                     # let the sampler start before the timed region
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in getattr(self, "lines", []):
            f = [c.strip() for c in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_device(fn, steps, warmup, torch, barrier=None, after_warmup=None):
    for _ in range(warmup):
        fn()
    if after_warmup:
        after_warmup()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    if barrier:
        barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    if barrier:
        barrier()
    return e0.elapsed_time(e1) / steps


def serial_stages(H, fn, steps, torch):
    """Per-stage milliseconds per call with the tree passes run in order on
    the caller's stream (so stage times do not overlap)."""
    H.set_overlap(False)
    H.profile()
    time_device(fn, steps, 2, torch, after_warmup=lambda: H.stage_times(reset=True))
    st = H.stage_times(reset=True)
    H.profile([])
    H.set_overlap(True)
    n = max(1, max(v[1] for v in st.values()))
    return {k: v[0] / n for k, v in st.items()}


def rel_err_sampled(H, u, b64, rows, torch):
    ref = H.direct_rows(b64, rows)
    got = u.index_select(0, rows).to(torch.float64)
    return float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))


# ----------------------------------------------------------------- CPU baseline

def cpu_baseline(n, budget_s=25.0, threads=None, single_core=True):
    """The oracle (CPU restatement of the reference, reference layout and loop
    order) timed on this host: build once, then full matvecs on all host
    threads until ~budget_s, and (single_core) a few on one thread -- the
    reference itself is single-threaded Julia."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    avail = int(ln.split()[1]) * 1024
    except Exception:
        pass
    # The reference layout stores ~1750 values per point at n = 2^20 (14 GB).
    n_run = n
    while avail is not None and n_run > 4096 and n_run * 1750 * 8 * 1.3 > 0.6 * avail:
        n_run //= 2
    x, y = grid_points(n_run)
    t0 = time.perf_counter()
    H = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0, nthreads=threads)
    build_s = time.perf_counter() - t0
    b = np.random.default_rng(7).standard_normal(n_run)
    u = np.zeros(n_run)

    def timed(nthr, budget, least, most):
        H.mul(u, b, nthreads=nthr)          # warm-up
        times = []
        t_end = time.perf_counter() + budget
        while len(times) < least or (time.perf_counter() < t_end and len(times) < most):
            u[:] = 0
            t0 = time.perf_counter()
            H.mul(u, b, nthreads=nthr)
            times.append(time.perf_counter() - t0)
        return statistics.median(times), len(times)

    med, cnt = timed(threads, budget_s, 2, 20)
    st = H.stats()
    scale = 1.0
    if n_run != n:
        # scale by the reference-layout values streamed per matvec at full size
        from hierarchicalmatrices import Plan
        xf, yf = grid_points(n)
        scale = st["stored_values"] / Plan(xf, yf, 1.0, 0.0, 1.0, 0.0).sizes["reference_values"]
    sample = (f"oracle KernelMatrix n={n_run} grid, reference per-block layout "
              f"({st['stored_values']} values), {cnt} full matvecs on {threads} threads after 1 warm-up, "
              f"median {med * 1e3:.1f} ms; build {build_s:.1f} s")
    if n_run != n:
        sample += f"; scaled to n={n} by reference-layout values (host memory)"
    out = {"value": scale / med, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    if single_core:
        med1, cnt1 = timed(1, 0.0, 3, 3)
        out["single_core"] = {
            "value": scale / med1, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"the same matrix and vector, {cnt1} full matvecs on 1 thread after 1 warm-up, "
                      f"median {med1 * 1e3:.1f} ms (the reference is single-threaded)"}
    return out


def workload_config(n, world):
    """The headline workload as both arms report it (the same keys and values)."""
    return {
        "workload": "KernelMatrix Cauchy 1/(x-y), n=2^20 interleaved grid (descending, "
                    "a=c=1, b=d=0), rank 20, leaf 80, FP64 compression, FP32 factors/leaves, "
                    "1 RHS per step",
        "n": n, "rank": 20, "blocksize": 80, "nrhs": 1, "parallelism": f"replicas{world}",
        "l2": "inputs larger than L2 every step: the factors streamed per product (1.14 GB in FP32, "
              "14 GB in the reference's FP64 per-block layout at n=2^20) exceed the 129 MB L2; no flush",
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    cb = cpu_baseline(args.n, budget_s=max(5.0, min(60.0, 3.0 * (args.steps + args.warmup))),
                      threads=threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 / cb["value"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.n, args.gpus),
        "precision_note": "the reference computes in FP64 (its only CPU path); the GPU arm's headline is FP32 "
                          "storage from FP64 compression, and its FP64 product is under variants.fp64_k1",
        "reference_path": "the oracle's restatement of the reference's KernelMatrix product (reference "
                          "per-block layout and loop order, FP64) on the host cores; Julia is not installed",
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- batching

def batch_instances(count=512, lo=1024, hi=65536, seed=0):
    """count instances, n_k log-uniform in [lo, hi], points uniform on [0,1],
    sorted descending."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    xs = [np.sort(rng.random(int(n)))[::-1].copy() for n in ns]
    ys = [np.sort(rng.random(int(n)))[::-1].copy() for n in ns]
    return xs, ys, [(1.0, 0.0, 1.0, 0.0)] * count


def run_batch(hm, torch, dev, args, count=512, nrhs=8):
    """512 independent Cauchy KernelMatrices, 8 FP32 right-hand sides each,
    multiplied together by one captured CUDA graph; instances/s and the
    per-batch latency distribution over the replays."""
    xs, ys, boxes = batch_instances(count)
    t0 = time.perf_counter()
    Hb = hm.KernelMatrixBatch(hm.cauchykernel, xs, ys, boxes, dtype=np.float32)
    if getattr(args, "wide_tree", None):
        Hb.set_wide_tree({"off": False, "on": True, "all": "all"}[args.wide_tree])
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    st = Hb.stats()
    B = torch.randn(nrhs, Hb.shape[1], device=dev, dtype=torch.float32).t()
    U = torch.empty(nrhs, Hb.shape[0], device=dev, dtype=torch.float32).t()
    sched = Hb.autotune(nrhs, reps=5)            # schedule picked by the autotuner, then captured
    cs = torch.cuda.Stream()
    cs.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cs):
        for _ in range(3):                      # warm-up: per-stream scratch, side stream
            Hb.mul(U, B, accumulate=False, stream=cs)
    cs.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cs):
        Hb.mul(U, B, accumulate=False, stream=cs)
    reps = max(10, args.steps)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    cur = torch.cuda.current_stream()
    for a, b in evs:
        a.record(cur)
        g.replay()
        b.record(cur)
    torch.cuda.synchronize()
    lat = np.array([a.elapsed_time(b) for a, b in evs])
    # error of the last instance's last column against exact dense rows
    i = count - 1
    r0, c0 = int(Hb.row_offsets[i]), int(Hb.col_offsets[i])
    Hi = hm.KernelMatrix(hm.cauchykernel, xs[i], ys[i], *boxes[i])
    rows = torch.arange(0, len(xs[i]), 7, device=dev)
    ref = Hi.direct_rows(B[c0:c0 + len(ys[i]), nrhs - 1].double().contiguous(), rows)
    got = U[r0:r0 + len(xs[i]), nrhs - 1].double()[rows]
    err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
    return {
        "workload": f"{count} Cauchy KernelMatrices, n log-uniform in [1024, 65536] (sum {Hb.shape[0]}), "
                    f"uniform sorted points, {nrhs} FP32 RHS each, one captured CUDA graph per batch",
        "instances_per_s": count / (lat.mean() * 1e-3), "matvec_per_s": count * nrhs / (lat.mean() * 1e-3),
        "batch_ms_mean": float(lat.mean()), "batch_ms_p50": float(np.percentile(lat, 50)),
        "batch_ms_p99": float(np.percentile(lat, 99)), "replays": reps, "build_s": build_s,
        "stored_GB": st["stored_values"] * 4 / 1e9, "rel_err_vs_dense_fp64_sample": err,
        "gpu_launches_per_batch": st["launches_per_mul"], "schedule": sched,
    }


# ----------------------------------------------------------------- gradients

def spd_hodlr_gauss(hm, torch, dev, n, leaf, ell=0.15, shift=1e-2, tol=1e-12, seed=21, host_linalg=False):
    """A synthetic symmetric positive definite HierarchicalMatrix of the shape
    src/cholesky.jl factors: K(x_i, x_j) = exp(-(x_i - x_j)^2 / (2 ell^2)) +
    shift I on n sorted uniform points of [0, 1], halved recursively down to
    dense diagonal leaves of at most `leaf` rows, each upper off-diagonal
    block a LowRankMatrix (its singular values above tol times the largest,
    found on the device by a randomized range finder with two power steps),
    the lower block unassigned.  FP64, built on the device (setup, untimed);
    host_linalg: the range finder's QR and SVD in numpy instead (torch.linalg
    does not load under ncu)."""
    g = torch.Generator(device=dev).manual_seed(seed)
    x = torch.sort(torch.rand(n, generator=g, device=dev, dtype=torch.float64)).values

    def kblock(i0, i1, j0, j1):
        d = x[i0:i1, None] - x[None, j0:j1]
        return torch.exp(-d * d / (2 * ell * ell))

    def colmajor(t):
        return t.t().contiguous().t()

    def build(i0, i1):
        if i1 - i0 <= leaf:
            return colmajor(kblock(i0, i1, i0, i1) + shift * torch.eye(i1 - i0, dtype=torch.float64, device=dev))
        mid = (i0 + i1) // 2
        B = kblock(i0, mid, mid, i1)
        k = min(96, B.shape[0], B.shape[1])
        if host_linalg:
            def qr(M):
                return torch.tensor(np.linalg.qr(M.cpu().numpy())[0], device=dev)

            def svd(M):
                return [torch.tensor(t, device=dev) for t in np.linalg.svd(M.cpu().numpy(), full_matrices=False)]
        else:
            def qr(M):
                return torch.linalg.qr(M)[0]

            def svd(M):
                return torch.linalg.svd(M, full_matrices=False)
        Q = qr(B @ torch.randn(B.shape[1], k, generator=g, device=dev, dtype=torch.float64))
        for _ in range(2):
            Q = qr(B @ (B.t() @ Q))
        Uc, S, Vt = svd(Q.t() @ B)
        r = int((S > tol * S[0]).sum())
        H = hm.HierarchicalMatrix(2, 2)
        H[hm.Block(1), hm.Block(1)] = build(i0, mid)
        H[hm.Block(1), hm.Block(2)] = hm.LowRankMatrix(colmajor(Q @ Uc[:, :r]), S[:r].contiguous(), colmajor(Vt[:r].t()))
        H[hm.Block(2), hm.Block(2)] = build(mid, i1)
        return H

    return build(0, n)


def tree_ranks(H):
    """Largest rank of the LowRankMatrix blocks of a tree."""
    best = 0
    for b, _, _ in H.leaves():
        if hasattr(b, "sigma"):
            best = max(best, int(b.sigma.shape[0]))
    return best


def run_cholesky(hm, torch, dev, args, n=16384, leaf=64):
    """hierarchicalcholesky (src/cholesky.jl:12-92) of a Gaussian-kernel SPD
    HierarchicalMatrix, FP64, and one solvetransposed with the factor:
    wall time per factorisation (the host recursion and every batched block
    call included)."""
    from hierarchicalmatrices import algebra
    A = spd_hodlr_gauss(hm, torch, dev, n, leaf)
    R = algebra.hierarchicalcholesky(A)              # warm-up: kernels, attributes
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        R = algebra.hierarchicalcholesky(A)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    # the same recursion driven block operation by block operation from Python
    # (hierarchicalcholesky(A, native=False)), one run, for comparison
    algebra.hierarchicalcholesky(A, native=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    algebra.hierarchicalcholesky(A, native=False)
    torch.cuda.synchronize()
    rec_ms = (time.perf_counter() - t0) * 1e3
    b = torch.randn(n, device=dev, dtype=torch.float64)
    algebra.solvetransposed(R, b)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        xs = algebra.solvetransposed(R, b)
    torch.cuda.synchronize()
    solve_ms = (time.perf_counter() - t0) / reps * 1e3
    # residual of the solve through the factor's own product: R'x = b  <=>  x . (R e_j) = b_j;
    # checked on the dense factor for the leading 2048 x 2048 block (R is upper triangular)
    m = 2048
    Rd = algebra.todense(R)[:m, :m]
    resid = float(torch.linalg.norm(Rd.t() @ xs[:m] - b[:m]) / torch.linalg.norm(b[:m]))
    cpu = None if args.no_cpu_baseline else cholesky_cpu_baseline(hm, A, b.cpu().numpy())
    return {"workload": f"hierarchicalcholesky of K + 1e-2 I, K Gaussian exp(-(x-y)^2/(2*0.15^2)) on n={n} sorted "
                        f"uniform points, leaf {leaf}, off-diagonal LowRankMatrix blocks at 1e-12, FP64; "
                        "then solvetransposed of one vector",
            "path": "hm_hchol_factor (native recursion, A22-update SVDs on a stream pool)",
            "n": n, "ms_per_factorization": ms, "factorizations_per_s": 1e3 / ms,
            "ms_block_by_block_from_python": rec_ms, "solve_ms": solve_ms,
            "max_rank_A": tree_ranks(A), "max_rank_R": tree_ranks(R), "solve_rel_residual_leading_2048": resid,
            "reps": reps, "cpu_baseline": cpu}


def cholesky_cpu_baseline(hm, A, b):
    """The oracle's hierarchicalcholesky and solvetransposed (numpy/LAPACK on
    the host cores, the reference's block order) on the same matrix: one run
    each (the factorisation takes about a second at n = 16384)."""
    from oracle import algebra as OA

    def host_tree(H):
        if isinstance(H, hm.LowRankMatrix):
            return OA.LR(H.U.cpu().numpy(), H.sigma.cpu().numpy(), H.V.cpu().numpy())
        if not hasattr(H, "blocksize"):
            return H.cpu().numpy()
        M, N = H.blocksize()
        return OA.HB([[None if H.block(i, j) is None else host_tree(H.block(i, j)) for j in range(N)]
                      for i in range(M)])

    T = host_tree(A)
    t0 = time.perf_counter()
    R = OA.cholesky(T)
    chol_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    OA.solvetransposed(R, b)
    solve_ms = (time.perf_counter() - t0) * 1e3
    return {"kind": "port", "cores": os.cpu_count(), "ms_per_factorization": chol_ms, "solve_ms": solve_ms,
            "sample": "oracle/algebra.py cholesky + solvetransposed (numpy, LAPACK leaves) on the same matrix, one run"}


def stage_timeline(hm, torch, n, reps=50):
    """Start and end of every stage of the FP32 headline product (CUDA events on
    the stream that launches each stage, hm_profile_timeline), in microseconds
    from the product's start, averaged over reps products, for each stream
    schedule HM_OPT_OVERLAP 0-4.  Timing the tree stages records events between
    their kernels, so these products run with plain launches."""
    import ctypes
    from hierarchicalmatrices import _lib
    x, y = grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    b = torch.randn(n, device="cuda", dtype=torch.float32)
    u = torch.empty_like(b)
    out = {}
    for mode in (0, 1, 2, 3, 4):
        H.set_overlap(mode)
        for _ in range(20):
            H.mul(u, b, accumulate=False)
        torch.cuda.synchronize()
        H.profile()
        acc = {}
        buf = np.zeros(3 * 16)
        for _ in range(reps):
            H.mul(u, b, accumulate=False)
            cnt = _lib.lib.hm_profile_timeline(H.handle, buf.ctypes.data_as(ctypes.c_void_p), 16)
            for i in range(min(cnt, 16)):
                a = acc.setdefault(_lib.STAGES[int(buf[3 * i])], [0.0, 0.0])
                a[0] += buf[3 * i + 1] * 1e3 / reps
                a[1] += buf[3 * i + 2] * 1e3 / reps
        H.profile([])
        out[f"overlap{mode}"] = {k: [round(v[0], 1), round(v[1], 1)] for k, v in sorted(acc.items(), key=lambda kv: kv[1][0])}
    H.free()
    return out


def run_grad(hm, torch, dev, args, n=65536):
    """L = 1/2 |H(x,y) w - t|^2 for a Cauchy KernelMatrix on n uniform sorted
    points, FP32: loss and dL/dw, dL/dx, dL/dy (forward product, transposed
    product and the two row-derivative products)."""
    rng = np.random.default_rng(11)
    x = np.sort(rng.random(n))[::-1].copy()
    y = np.sort(rng.random(n))[::-1].copy()
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    w = torch.randn(n, device=dev, dtype=torch.float32)
    t = torch.randn(n, device=dev, dtype=torch.float32)
    for _ in range(3):
        H.loss_and_grad(w, t)                 # builds the transposed and derivative panels
    reps = max(5, min(100, args.steps // 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        H.loss_and_grad(w, t)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    return {"workload": f"Cauchy KernelMatrix n={n} uniform sorted points, FP32; loss + dL/dw + dL/dx + dL/dy "
                        "(forward, transposed and two row-derivative products)",
            "ms_per_grad": ms, "grads_per_s": 1e3 / ms, "reps": reps}


def profile_case(hm, torch, args):
    """Three products of one workload, for ncu captures (no timing); the
    hierarchical Cholesky case factors the bench's n = 16384 matrix twice."""
    if args.profile_case == "cholesky":
        from hierarchicalmatrices import algebra
        A = spd_hodlr_gauss(hm, torch, "cuda", 16384, 64, host_linalg=True)
        for _ in range(2):
            algebra.hierarchicalcholesky(A)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "cholesky", "n": 16384, "ok": True}), flush=True)
        return 0
    n = args.n
    x, y = grid_points(n)
    case = args.profile_case
    dtype = {"fp64": np.float64, "df64": "df64"}.get(case, np.float32)
    k = {"k8": 8, "k32": 32, "k256": 256}.get(case, 1)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    if args.wide_tree:
        H.set_wide_tree({"off": False, "on": True, "all": "all"}[args.wide_tree])
    if case == "headline":
        H.set_overlap(4)                        # the autotuner's choice for one FP32 right-hand side
        H.set_pdl(True)
    else:
        H.set_overlap(0)
    tdt = torch.float64 if case in ("fp64", "df64") else torch.float32
    B = torch.randn(k, n, device="cuda", dtype=tdt).t()
    U = torch.empty(k, n, device="cuda", dtype=tdt).t()
    if k == 1:
        B, U = B[:, 0].contiguous(), U[:, 0].contiguous()
    for _ in range(3):
        H.mul(U, B, accumulate=False)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": case, "n": n, "nrhs": k, "ok": True}), flush=True)
    return 0


# ----------------------------------------------------------------- GPU arm

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-cholesky", action="store_true",
                    help="skip the hierarchical Cholesky line (its matrix generator uses torch.linalg, which "
                         "fails to load under ncu)")
    ap.add_argument("--batch-instances", type=int, default=512,
                    help="instances of the batch workload (512 in the configuration it reports)")
    ap.add_argument("--only-batch", action="store_true",
                    help="run only the batch workload and print its result (for profiling)")
    ap.add_argument("--timeline", action="store_true",
                    help="print the headline product's stage timeline for each stream schedule (for profiling)")
    ap.add_argument("--autotune-reps", type=int, default=50,
                    help="products timed per candidate schedule by the autotuner (fewer for profiling runs)")
    ap.add_argument("--profile-case", default=None,
                    choices=["headline", "fp64", "df64", "k8", "k32", "k256", "cholesky"],
                    help="run three products of one workload at --n points and exit (for ncu captures): the "
                         "headline FP32 product with the autotuner's choice for it (near field after the leaf "
                         "stage, programmatic launches), the FP64 / FP64-double-float product, or FP32 with 8, 32 "
                         "or 256 right-hand sides with every stage on one stream; or two hierarchical Cholesky "
                         "factorisations of the bench's n = 16384 matrix")
    ap.add_argument("--wide-tree", default=None, choices=["off", "on", "all"],
                    help="HM_OPT_WIDE_TREE for --profile-case and --only-batch runs")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import hierarchicalmatrices as hm
    from hierarchicalmatrices import parallel

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    barrier = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        barrier = lambda: dist.barrier()  # noqa: E731

    if args.timeline:
        print(json.dumps({"timeline_us": stage_timeline(hm, torch, args.n)}), flush=True)
        return 0

    if args.profile_case:
        return profile_case(hm, torch, args)

    if args.only_batch:
        print(json.dumps({"batch": run_batch(hm, torch, torch.device("cuda", local), args,
                                             count=args.batch_instances)}), flush=True)
        return 0

    n = args.n
    x, y = grid_points(n)
    rng = np.random.default_rng(1234 + rank)
    b64_np = rng.standard_normal(n)
    dev = torch.device("cuda", local)
    b64 = torch.tensor(b64_np, device=dev)
    b32 = b64.to(torch.float32)
    nrows = 4096
    rows = torch.tensor(np.sort(rng.choice(n, size=nrows, replace=False)), device=dev)

    t0 = time.perf_counter()
    H32 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    torch.cuda.synchronize()
    build32_s = time.perf_counter() - t0
    st = H32.stats()
    u32 = torch.empty(n, device=dev, dtype=torch.float32)

    # ---- headline: FP32 storage, 1 RHS, device-resident inputs
    # the product's schedule is picked by the library's autotuner (untimed setup)
    sched = H32.autotune(1, reps=args.autotune_reps)
    # CUDA events around the dominant stage only, on the launching stream,
    # inside the timed region (two events per step).
    H32.profile(["expand"])
    with ClockSampler(local) as clk:
        ms = time_device(lambda: H32.mul(u32, b32, accumulate=False), args.steps, args.warmup,
                         torch, barrier, after_warmup=lambda: H32.stage_times(reset=True))
    exp_total, exp_launches = H32.stage_times(reset=True)["expand"]
    H32.profile([])
    ms = parallel.max_over_ranks(ms)             # the slowest rank's step time (N > 1)
    value = world * 1e3 / ms
    err32 = rel_err_sampled(H32, u32, b64, rows, torch)

    # dominant kernel: row-segment panels (stage "expand")
    hbm_peak, peak_kind = peaks()
    exp_ms = exp_total / max(1, exp_launches)
    # near-field panel kernel: streams the dense leaf values once, reads x
    # once and writes y once
    exp_bytes = st["dense_values"] * 4 + 2 * n * 4
    achieved = exp_bytes / (exp_ms * 1e-3) / 1e9
    canonical_bytes = st["canonical_values"] * 4 + 2 * n * 4
    stored_bytes = st["stored_values"] * 4 + 2 * n * 4

    # ---- end to end through the C ABI with pinned host buffers
    hb = torch.empty(n, dtype=torch.float32, pin_memory=True)
    hb.copy_(b32.cpu())
    hu = torch.empty(n, dtype=torch.float32, pin_memory=True)
    hb_np, hu_np = hb.numpy(), hu.numpy()
    for _ in range(args.warmup):
        H32.mul_host(hu_np, hb_np, accumulate=False)
    if barrier:
        barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        H32.mul_host(hu_np, hb_np, accumulate=False)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_value = world / e2e_s
    # per-stage breakdown: every stage timed in order on one stream (no
    # overlap; setting the stream option replaces the tuned schedule)
    stages = serial_stages(H32, lambda: H32.mul(u32, b32, accumulate=False), args.steps, torch)

    variants = {}
    if not args.no_variants:
        k_steps = max(3, args.steps)
        # plain FP64 product
        t0 = time.perf_counter()
        H64 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float64)
        torch.cuda.synchronize()
        build64_s = time.perf_counter() - t0
        u64 = torch.empty(n, device=dev, dtype=torch.float64)
        sched64 = H64.autotune(1, reps=20)
        ms64 = time_device(lambda: H64.mul(u64, b64, accumulate=False), k_steps, 3, torch)
        st64s = serial_stages(H64, lambda: H64.mul(u64, b64, accumulate=False), 10, torch)
        err64 = rel_err_sampled(H64, u64, b64, rows, torch)
        st64 = H64.stats()
        # end to end through hm_mul_host with page-locked host buffers, as the headline's e2e
        hb64 = torch.empty(n, dtype=torch.float64, pin_memory=True)
        hb64.copy_(b64.cpu())
        hu64 = torch.empty(n, dtype=torch.float64, pin_memory=True)
        hb64_np, hu64_np = hb64.numpy(), hu64.numpy()
        for _ in range(max(3, args.warmup)):
            H64.mul_host(hu64_np, hb64_np, accumulate=False)
        t0 = time.perf_counter()
        for _ in range(k_steps):
            H64.mul_host(hu64_np, hb64_np, accumulate=False)
        e2e64 = k_steps / (time.perf_counter() - t0)
        variants["fp64_k1"] = {
            "matvec_per_s": 1e3 / ms64, "ms": ms64, "rel_err_vs_dense_fp64": err64,
            "stored_GBs": (st64["stored_values"] * 8 + 2 * n * 8) / (ms64 * 1e-3) / 1e9,
            "effective_canonical_GBs": (st64["canonical_values"] * 8 + 2 * n * 8) / (ms64 * 1e-3) / 1e9,
            "build_s": build64_s, "stage_ms_serial": st64s, "schedule": sched64, "steps": k_steps,
            "e2e": {"value": e2e64, "unit": UNIT, "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
                    "api": "hm_mul_host, page-locked host buffers"}}
        del H64, u64
        torch.cuda.empty_cache()
        # the same FP64 product with HM_DF64 storage: row-segment panels as
        # double-float pairs multiplied on the FP32 pipes (tree passes FP64)
        t0 = time.perf_counter()
        Hd = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
        torch.cuda.synchronize()
        buildd_s = time.perf_counter() - t0
        ud = torch.empty(n, device=dev, dtype=torch.float64)
        schedd = Hd.autotune(1, reps=20)
        msd = time_device(lambda: Hd.mul(ud, b64, accumulate=False), k_steps, 3, torch)
        stds = serial_stages(Hd, lambda: Hd.mul(ud, b64, accumulate=False), 10, torch)
        errd = rel_err_sampled(Hd, ud, b64, rows, torch)
        stdd = Hd.stats()
        for _ in range(max(3, args.warmup)):
            Hd.mul_host(hu64_np, hb64_np, accumulate=False)
        t0 = time.perf_counter()
        for _ in range(k_steps):
            Hd.mul_host(hu64_np, hb64_np, accumulate=False)
        e2ed = k_steps / (time.perf_counter() - t0)
        variants["fp64_df_k1"] = {
            "storage": "HM_DF64: FP64 vectors, bases, far-field blocks and tree passes; row-segment panels as "
                       "double-float (h, l) FP32 pairs multiplied on the FP32 pipes",
            "matvec_per_s": 1e3 / msd, "ms": msd, "rel_err_vs_dense_fp64": errd,
            "stored_GBs": (stdd["stored_values"] * 8 + 2 * n * 8) / (msd * 1e-3) / 1e9,
            "build_s": buildd_s, "stage_ms_serial": stds, "schedule": schedd, "steps": k_steps,
            "e2e": {"value": e2ed, "unit": UNIT, "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
                    "api": "hm_mul_host, page-locked host buffers"}}
        del Hd, ud
        torch.cuda.empty_cache()
        # clustered points: Beta(1/2, 1/2), FP64 (a deeper, uneven tree)
        xb, yb = beta_points(n, 21)
        hi = float(max(xb[0], yb[0], 1.0))
        t0 = time.perf_counter()
        Hb = hm.KernelMatrix(hm.cauchykernel, xb, yb, hi, 0.0, hi, 0.0, dtype=np.float64)
        torch.cuda.synchronize()
        buildb_s = time.perf_counter() - t0
        ub = torch.empty(n, device=dev, dtype=torch.float64)
        schedb = Hb.autotune(1, reps=20)
        msb = time_device(lambda: Hb.mul(ub, b64, accumulate=False), k_steps, 3, torch)
        stb = Hb.stats()
        variants["fp64_k1_beta"] = {
            "points": "x, y i.i.d. Beta(1/2,1/2) sorted, min gap 1e-9, seed 21",
            "matvec_per_s": 1e3 / msb, "ms": msb, "rel_err_vs_dense_fp64": rel_err_sampled(Hb, ub, b64, rows, torch),
            "stored_GBs": (stb["stored_values"] * 8 + 2 * n * 8) / (msb * 1e-3) / 1e9,
            "build_s": buildb_s, "schedule": schedb, "depth": stb["depth"], "n_bary": stb["n_bary"], "n_dense": stb["n_dense"]}
        del Hb, ub
        torch.cuda.empty_cache()
        for k in (32, 256):
            B = torch.randn(k, n, device=dev, dtype=torch.float32).t()    # column-major n x k
            U = torch.empty(k, n, device=dev, dtype=torch.float32).t()
            schedk = H32.autotune(k, reps=10 if k <= 32 else 4)
            msk = time_device(lambda: H32.mul(U, B, accumulate=False), k_steps, 3, torch)
            stk = serial_stages(H32, lambda: H32.mul(U, B, accumulate=False), 3, torch)
            errk = rel_err_sampled(H32, U[:, k - 1].contiguous(), B[:, k - 1].to(torch.float64).contiguous(),
                                   rows, torch)
            variants[f"fp32_k{k}"] = {
                "matvec_per_s": k * 1e3 / msk, "ms_per_block": msk, "rel_err_vs_dense_fp64": errk,
                "stored_GBs": (st["stored_values"] * 4 + 2 * n * k * 4) / (msk * 1e-3) / 1e9,
                "stage_ms_serial": stk, "schedule": schedk}
            del B, U
            torch.cuda.empty_cache()

    batch = None
    if not args.no_variants and not args.no_batch:
        batch = run_batch(hm, torch, dev, args, count=args.batch_instances)
    grad = None
    chol = None
    if not args.no_variants:
        grad = run_grad(hm, torch, dev, args)
        chol = None if args.no_cholesky else run_cholesky(hm, torch, dev, args)

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cb = cpu_baseline(n)
        except Exception as e:  # report, never fake
            cb = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                  "sample": f"failed: {type(e).__name__}: {e}"}

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(n, world),
            "rel_err_vs_dense_fp64": err32,
            "hbm_GBs_stored": stored_bytes / (ms * 1e-3) / 1e9,
            "hbm_GBs_effective_canonical": canonical_bytes / (ms * 1e-3) / 1e9,
            "roofline": {
                "bound": "hbm",
                "kernel": ("stream_part<float,float,false,1> (near-field panels, streamed CTAs)"
                           if sched["near_kernel"] == 2 else
                           "expand_part<float,float,false,2> (near-field panels, one warp per row segment)"),
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": profiled_traffic(n), "traffic_unit": "GB per launch",
                "traffic_source": "not measured in this run: ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                  "one launch of this kernel on this workload, from the committed profile "
                                  "profiles/expand_near_kernelmatrix_cauchy_n2p20_fp32.md",
                "peak_source": peak_kind, "kernel_ms": exp_ms, "kernel_bytes": exp_bytes,
                "stage_ms_serial": stages,
            },
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 4,
                    "d2h_bytes_per_step": n * 4},
            "gpu_launches": st["launches_per_mul"] * args.steps,
            "clocks": clocks,
            "build_s": build32_s,
            "schedule": sched,
            "tree": {k: st[k] for k in ("n_bary", "n_dense", "depth", "canonical_values",
                                        "reference_values", "stored_values", "device_bytes")},
            "variants": variants,
            "batch": batch,
            "grad": grad,
            "cholesky": chol,
            "cpu_baseline": cb,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
