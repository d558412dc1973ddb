"""Benchmark of the sketch-then-factor path (one JSON line on stdout).

Workload: psvdfact of a dense 8192 x 8192 Float64 matrix A = U diag(s) V'
with U, V Haar-random (thin QR of seeded N(0,1) matrices; columns past
1024 carry s_i < 1e-25 and are dropped), s_i = 10^(-(i-1)/40), rtol 1e-10
(rank ~ 400).  One step = one psvdfact call.  `value` is matrices/s with A
resident in HBM; `e2e` is the same call from pinned host memory with the
host<->device copies inside the timed region.  The inputs (512 MB) are
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision mixed|native] [--n 8192]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "lowrankapprox.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "idfact/psvdfact matrices/s & GFLOP/s at rtol 1e-10 vs FP64 path; p50/p99 ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "native"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--rtol", type=float, default=1e-10)
    ap.add_argument("--no-fp64-leg", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests per precision in the serving measurement (0: skip)")
    ap.add_argument("--batch", type=int, default=2048,
                    help="kernel matrices in the batched measurement (0: skip)")
    ap.add_argument("--batch-native", type=int, default=0,
                    help="run the FP64 path on the first N of them only (0: the whole batch)")
    ap.add_argument("--no-tall", action="store_true", help="skip the tall Float32 idfact measurement")
    ap.add_argument("--srft-sweep", action="store_true",
                    help="only the SRFT sketch sweep on a Gaussian 65536x4096 Float32 matrix (one JSON line)")
    ap.add_argument("--tall-only", action="store_true",
                    help="only the tall Float32 idfact measurement (one JSON line)")
    return ap.parse_args()


def make_matrix(n: int, rank_cols: int = 1024, device: str = "cuda"):
    """A = U diag(s) V' built on the device (the GPU unless told otherwise)
    from seeded numpy Gaussians."""
    import torch
    r = min(n, rank_cols)
    facs = []
    for seed in (1, 2):
        Q, R = np.linalg.qr(np.random.default_rng(seed).standard_normal((n, r)))
        facs.append(torch.from_numpy(Q * np.sign(np.diag(R))[None, :]).to(device))
    U, V = facs
    s = torch.pow(10.0, -torch.arange(r, dtype=torch.float64, device=device) / 40.0)
    A = (U * s[None, :]) @ V.T
    del U, V, facs
    # column-major storage
    return A.t().contiguous().t()


def psvd_flops(m, n, k_id, k, orders, ks):
    """Algorithmic FLOPs of one psvdfact (sketch, QR, trsm, psvd extras)."""
    f = 0.0
    for l, kq in zip(orders, ks):
        f += 2.0 * l * m * n
        kq = min(kq + 1, l, n)
        f += 4.0 * l * n * kq - 2.0 * kq * kq * (l + n) + 4.0 / 3.0 * kq ** 3
    kk = k_id
    f += kk * kk * (n - kk)                                   # trsm
    f += 2.0 * m * kk * kk - 2.0 / 3.0 * kk ** 3              # QR(A[:, sk])
    f += 2.0 * kk * kk * (n - kk)                             # R V
    f += 4.0 * n * kk * kk + 8.0 * kk ** 3                    # SVD of R V
    f += 4.0 * m * kk * k                                     # Q U~
    return f


QR_KERNELS = ("geqp3_df_smem_kernel", "geqp3_f32_smem_kernel", "geqp3_df_kernel", "geqp3_v2_kernel")
SERVE_SLOTS = 2


def tuning_record(ctx) -> dict:
    """The shape table the library runs with (lra_ctx_get_tuning): its
    source and every entry, for the bench line."""
    t = {"source": None, "tc_tile_n": {"f32": [0] * 16, "f64": [0] * 16}, "srft_wide": [0] * 11}
    for line in ctx.tuning().splitlines():
        w = line.split()
        if not w:
            continue
        if w[0] == "#" and len(w) > 2 and w[1] == "source:":
            t["source"] = " ".join(w[2:]).split("/")[-1]
        elif w[0] == "tc_tile_n" and len(w) == 4:
            t["tc_tile_n"][w[1]][int(w[2])] = int(w[3])
        elif w[0] == "srft_wide" and len(w) == 3:
            t["srft_wide"][int(w[1])] = int(w[2])
        elif len(w) == 2 and w[0] in ("qr_seq_len", "qr_steps"):
            t[w[0]] = int(w[1])
    return t


def sketch_orders(k, nb=32):
    orders, ks, nt = [], [], nb
    while True:
        orders.append(nt + 8)
        if k < nt:
            ks.append(k)
            return orders, ks
        ks.append(nt)
        nt *= 2


def serving_workload(count: int, seed: int = 5, hi: int = 16384):
    """Requests shaped like the serving config, a bounded sample of it:
    70 % idfact / 30 % psvdfact, m and n log-uniform in [256, hi] (16384 in
    the config), F32 / F64 half and half, s_i = 10^(-(i-1)/r) with
    r ~ U[20, 200], rtol 1e-6 (F32) and 1e-10 (F64).  A = (G1 diag(s)) G2'
    from Gaussian G1, G2 on the GPU, over the first min(m, n, 16 r + 64)
    singular values (the rest lie below 1e-16 of the first)."""
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        m, n = (int(round(np.exp(rng.uniform(np.log(256), np.log(hi))))) for _ in range(2))
        dt = torch.float64 if rng.random() < 0.5 else torch.float32
        kind = "idfact" if rng.random() < 0.7 else "psvdfact"
        r = rng.uniform(20, 200)
        # singular values past 16 r are below 1e-16 of the first: left out
        k = min(m, n, int(16 * r) + 64)
        g = torch.Generator(device="cuda").manual_seed(int(rng.integers(1 << 31)))
        G1 = torch.randn(m, k, generator=g, device="cuda", dtype=torch.float64) / np.sqrt(m)
        G2 = torch.randn(n, k, generator=g, device="cuda", dtype=torch.float64) / np.sqrt(n)
        sv = torch.pow(10.0, -torch.arange(k, dtype=torch.float64, device="cuda") / r)
        A = ((G1 * sv[None, :]) @ G2.T).to(dt).t().contiguous().t()
        out.append((kind, A, 1e-10 if dt == torch.float64 else 1e-6))
    return out


def kernel_matrices(count: int, seed: int = 4):
    """Batched config sample: K(x, y) = 1 / (1 + |x - y|^2) between x ~ U[0,1]^2 and
    y ~ U[1.5,2.5] x U[0,1] (gap 0.5 in x1), m, n ~ U{128..2048}, Float64."""
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m, n = int(rng.integers(128, 2049)), int(rng.integers(128, 2049))
        x = torch.from_numpy(rng.uniform(0, 1, (m, 2))).cuda()
        y = torch.from_numpy(np.column_stack([rng.uniform(1.5, 2.5, n), rng.uniform(0, 1, n)])).cuda()
        d2 = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
        out.append((1.0 / (1.0 + d2)).t().contiguous().t())
    return out


def measure_serving(lra, work, precision: str, slots: int = 8):
    """Poisson arrivals at about 80 % of the rate the server sustains when the
    requests arrive all at once; p50 / p99 of submit -> done."""
    import torch
    opts = [lra.LRAOptions(np.float64 if A.dtype == torch.float64 else np.float32, rtol=rt,
                           precision=precision, seed=11 + i) for i, (_, A, rt) in enumerate(work)]
    srv = lra.Server(slots=slots, hbm_budget_bytes=150 << 30)
    try:
        t0 = time.perf_counter()
        ts = [srv.submit(kind, A, o) for (kind, A, _), o in zip(work, opts)]
        for t in ts:
            srv.result(t)
        burst = len(work) / (time.perf_counter() - t0)
    finally:
        srv.close()
    rate = 0.8 * burst
    gaps = np.random.default_rng(9).exponential(1.0 / rate, len(work))
    srv = lra.Server(slots=slots, hbm_budget_bytes=150 << 30)
    try:
        t0 = time.perf_counter()
        ts = []
        due = t0
        for (kind, A, _), o, gap in zip(work, opts, gaps):
            due += gap
            while time.perf_counter() < due:
                time.sleep(min(1e-3, max(0.0, due - time.perf_counter())))
            ts.append(srv.submit(kind, A, o))
        for t in ts:
            srv.result(t)
        wall = time.perf_counter() - t0
        st = srv.stats()
    finally:
        srv.close()
    return {"requests": len(work), "slots": slots, "arrival_rate_per_s": rate, "matrices_s": len(work) / wall,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "burst_matrices_s": burst}


def tall_f32_matrix(m: int = 65536, n: int = 4096, seed: int = 6):
    """The tall Float32 config: A = U diag(s) V' with U, V Haar (QR of seeded
    Gaussians, on the GPU) and s_i = exp(-(i-1)/60)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    U = torch.linalg.qr(torch.randn(m, n, generator=g, device="cuda", dtype=torch.float32)).Q
    V = torch.linalg.qr(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float32)).Q
    sv = torch.exp(-torch.arange(n, dtype=torch.float32, device="cuda") / 60.0)
    A = ((U * sv[None, :]) @ V.T).t().contiguous().t()
    del U, V
    return A


def measure_tall(lra, ctx, A, peaks, reps: int = 3):
    """idfact of the tall Float32 matrix at rtol 1e-6 with the SRFT and the
    Gaussian sketch: per call time, the sketch stage's achieved rate (the SRFT
    reads A once per adaptive step: GB/s against HBM; the Gaussian sketch as
    three BF16 digit planes on the tensor cores: TFLOP/s against BF16), rank
    and error."""
    import torch
    m, n = A.shape
    out = {"workload": f"idfact {m}x{n} F32 U diag(s) V', s_i=exp(-(i-1)/60), rtol 1e-6"}
    nrm = lra.snorm(A, ctx=ctx)
    for sk in ("srft", "randn"):
        o = lra.LRAOptions(np.float32, rtol=1e-6, sketch=sk, precision="mixed", seed=5)
        # two untimed calls: the loop holds the previous result while the
        # next runs, so its page-locked result buffers alternate between two
        # sets, both allocated by then
        for _ in range(2):
            V = lra.idfact(A, o, ctx=ctx)
        torch.cuda.synchronize()
        stages = {"sketch": 0.0, "qr": 0.0, "solve": 0.0, "post": 0.0}
        t = 0.0
        q0 = sum(ctx.kernel_launches(kn) for kn in QR_KERNELS)
        for _ in range(reps):
            t0 = time.perf_counter()
            V = lra.idfact(A, o, ctx=ctx)
            torch.cuda.synchronize()
            t += time.perf_counter() - t0
            for kk, v in ctx.stage_ms().items():
                stages[kk] = stages.get(kk, 0.0) + v
        t /= reps
        stages = {kk: v / reps for kk, v in stages.items()}
        sketch_ms = stages["sketch"]
        a, b = o.sketchfact_srft_samp if sk == "srft" else o.sketchfact_randn_samp
        orders = [a * (o.nb << j) + b for j in range(V.nsteps)]
        qr_launches = (sum(ctx.kernel_launches(kn) for kn in QR_KERNELS) - q0) / reps
        r = {"ms_per_call": 1e3 * t, "matrices_s": 1.0 / t, "rank": V.k, "steps": V.nsteps, "orders": orders,
             "sketch_ms": sketch_ms, "stage_ms": stages, "qr_launches_per_call": qr_launches,
             "rel_spectral_err": lra.snormdiff(A, V, ctx=ctx) / nrm}
        if sk == "srft":
            gbs = len(orders) * m * n * 4 / (sketch_ms * 1e-3) / 1e9
            hbm = peaks.get("hbm_gbs") or 6800.0
            r["sketch_roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                    "bytes": "A read once per step"}
        else:
            fl = sum(2.0 * 3 * l * m * n for l in orders)
            tf = fl / (sketch_ms * 1e-3) / 1e12
            bf = peaks.get("bf16_tflops") or 1900.0
            r["sketch_roofline"] = {"bound": "tensor", "achieved": tf, "peak": bf, "unit": "TFLOP/s", "frac": tf / bf,
                                    "flops": "3 BF16 digit planes x 2 l m n per step"}
        out[sk] = r
    return out


def load_peaks() -> dict:
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def measure_srft_sweep(lra, ctx, A, peaks, reps: int = 3):
    """The SRFT sketch alone at the tall config's orders (40, 72, ..., 1032)
    on a device-resident Float32 matrix, the sketch written to device memory:
    per call ms (signs, frequencies, twiddle tables and srft_dif_kernel)
    and GB/s of A read once against HBM."""
    import torch
    m, n = A.shape
    o = lra.LRAOptions(np.float32, sketch="srft", seed=5)
    hbm = peaks.get("hbm_gbs") or 6800.0
    out = {"workload": f"SRFT sketch of a {m}x{n} F32 matrix, device in and out"}
    for order in [8 + (32 << j) for j in range(6)]:
        B = torch.empty((n, order), dtype=torch.float32, device=A.device).t()
        lra.sketch(A, order, o, ctx=ctx, out=B)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            lra.sketch(A, order, o, ctx=ctx, out=B)
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / reps
        gbs = m * n * 4 / t / 1e9
        out[str(order)] = {"ms": 1e3 * t, "gbs": gbs, "frac_hbm": gbs / hbm}
    return out


def measure_batched(lra, mats, precision: str, ctx):
    """lra_idfact_batched over the kernel matrices (rtol 1e-10)."""
    import torch
    o = lra.LRAOptions(rtol=1e-10, precision=precision, seed=3)
    # warm-up with the whole batch: the context's workspace settles at its size
    for _ in range(2):
        lra.idfact_batched(mats, o, ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Vs = lra.idfact_batched(mats, o, ctx=ctx)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    return {"matrices": len(mats), "matrices_s": len(mats) / el, "mean_rank": float(np.mean([V.k for V in Vs]))}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu_index: int):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"lra_bench_clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def lattice_stream(seed, n):
    """N(0,1) draws on the 1/32 lattice (the values the mixed path multiplies
    exactly), shared by the oracle and the GPU."""
    rng = np.random.default_rng(seed)
    return np.clip(np.rint(rng.standard_normal(n) * 32), -127, 127) / 32.0


def cpu_reference_step(A_host, rtol, seed, threads, keep=False):
    """The oracle's psvdfact on the host cores (numpy/OpenBLAS + C xLAQPS)."""
    from oracle import oracle as O
    m, n = A_host.shape
    g = lattice_stream(seed, 2200 * m)
    backend = "lapack" if O.lapack_available() else "c"
    t0 = time.perf_counter()
    F = O.psvdfact(A_host, O.Opts(rtol=rtol), O.RandStream(gauss=g), backend=backend)
    dt = time.perf_counter() - t0
    if keep:
        return dt, F["k"], backend, F, g
    return dt, F["k"], backend


def rel_err_psvd(A, U, S, Vt, x0, iters=32):
    """||A - U diag(S) Vt||_2 / ||A||_2 by power iteration (float64 torch on
    A's device), the same start vector for every result compared."""
    import torch
    dev = A.device
    Ut, St, Vtt = (torch.as_tensor(np.asarray(X, np.float64), device=dev) for X in (U, S, Vt))

    def snorm(apply, applyc):
        x = torch.as_tensor(x0, dtype=torch.float64, device=dev)
        s = 0.0
        for _ in range(iters):
            x = applyc(apply(x / torch.linalg.vector_norm(x)))
            s = float(torch.linalg.vector_norm(x)) ** 0.5
        return s
    e = snorm(lambda x: A @ x - Ut @ (St * (Vtt @ x)), lambda y: A.T @ y - Vtt.T @ (St * (Ut.T @ y)))
    return e / snorm(lambda x: A @ x, lambda y: A.T @ y)


def replica_rate(elapsed: float, steps: int, world: int) -> tuple[float, float]:
    """Whole-job rate of `world` replicas that each ran `steps` steps: the
    slowest rank's time (a MAX all-reduce over the process group when
    world > 1) and world * steps / that time."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([elapsed], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t[0])
    return elapsed, world * steps / elapsed


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(threads))
    import torch
    # the same matrix as the GPU arm's; built on the host when no GPU is there
    A = make_matrix(args.n, device="cuda" if torch.cuda.is_available() else "cpu").cpu().numpy()
    A = np.asfortranarray(A)
    times = []
    k = 0
    backend = "c"
    for i in range(args.warmup + args.steps):
        dt, k, backend = cpu_reference_step(A, args.rtol, 100 + i, threads)
        if i >= args.warmup:
            times.append(dt)
    sec = sum(times) / len(times)
    val = 1.0 / sec
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "matrices/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"psvdfact {args.n}x{args.n} F64 U diag(s) V', s_i=10^-(i-1)/40, rtol {args.rtol}",
                   "m": args.n, "n": args.n, "rtol": args.rtol, "rank": k},
        "cpu_baseline": {"value": val, "unit": "matrices/s", "cores": threads, "kind": "port",
                         "sample": f"one full {args.n}^2 psvdfact per step (oracle restatement, "
                                   f"numpy/OpenBLAS BLAS-3, xLAQPS backend {backend}); Julia absent"},
        "e2e": {"value": val, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    import lowrankapprox as lra

    ctx = lra.Context(local)
    if args.srft_sweep:
        G = torch.randn((4096, 65536), dtype=torch.float32, device="cuda").t()
        print(json.dumps({"srft_sweep": measure_srft_sweep(lra, ctx, G, load_peaks())}), flush=True)
        return
    if args.tall_only:
        At = tall_f32_matrix()
        print(json.dumps({"tall_f32": measure_tall(lra, ctx, At, load_peaks(), reps=max(1, args.steps))}),
              flush=True)
        return
    n = args.n
    A = make_matrix(n)
    torch.cuda.synchronize()
    opts = lra.LRAOptions(rtol=args.rtol, precision=args.precision, seed=1234 + rank)

    def step(X, o=opts):
        return lra.psvdfact(X, o, ctx=ctx)

    for _ in range(max(1, args.warmup)):  # at least one untimed call: the rank
        F = step(A)
    k = F.k

    # ---- device-resident timed region ---------------------------------------
    def barrier():
        if world > 1:
            dist.barrier()

    stage_tot = {"sketch": 0.0, "qr": 0.0, "solve": 0.0, "post": 0.0}
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    l0 = ctx.launches
    q0 = sum(ctx.kernel_launches(kn) for kn in QR_KERNELS)
    per = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ts = time.perf_counter()
        F = step(A)
        per.append(time.perf_counter() - ts)
        for kk, v in ctx.stage_ms().items():
            stage_tot[kk] += v
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    barrier()
    clk = clocks.stop()
    launches = ctx.launches - l0
    qr_launches = (sum(ctx.kernel_launches(kn) for kn in QR_KERNELS) - q0) / args.steps
    elapsed, value = replica_rate(elapsed, args.steps, world)

    # ---- end to end from pinned host memory ------------------------------------
    Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ah.copy_(A.t())  # row-major buffer of A^T == column-major A
    A_host = Ah.numpy().T  # Fortran-ordered view of pinned memory
    assert A_host.flags.f_contiguous
    step(A_host)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Fe = step(A_host)
    torch.cuda.synchronize()
    e2e_el = time.perf_counter() - t0
    e2e_val = world * args.steps / e2e_el
    h2d = n * n * 8
    d2h = (Fe.U.size + Fe.S.size + Fe.Vt.size) * 8

    # ---- accuracy of the last result ----------------------------------------------
    g = np.random.default_rng(7).standard_normal(n)
    err = lra.snormdiff(A, F, rand=lra.RandStream(gauss=g), ctx=ctx)
    nrm = lra.snorm(A, rand=lra.RandStream(gauss=g), ctx=ctx)

    # ---- the plain FP64 GPU path (same call, native precision) ---------------------
    fp64 = None
    if not args.no_fp64_leg and args.precision != "native":
        on = opts.copy(precision="native")
        step(A, on)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = max(1, min(2, args.steps))
        for _ in range(reps):
            Fn = step(A, on)
        torch.cuda.synchronize()
        fsec = (time.perf_counter() - t0) / reps
        errn = lra.snormdiff(A, Fn, rand=lra.RandStream(gauss=g), ctx=ctx)
        fp64 = {"value": world / fsec, "unit": "matrices/s", "ms_per_step": fsec * 1e3,
                "rel_spectral_err": errn / nrm, "rank": Fn.k}

    # ---- roofline of the dominant kernel ------------------------------------------------
    # The launch list puts the pivoted QR of the sketch (geqp3_df_smem_kernel
    # on the mixed path) first: the first adaptive step alone, then the
    # following steps several to a launch (qr_launches per call, counted by
    # the library).  The library's "qr" stage timer brackets those launches
    # and their conversions with CUDA events on its stream.
    # The kernel keeps the sketch in shared memory and is latency-bound (one
    # exchange between the CTAs per pivot), so its algorithmic traffic (the
    # sketch read and written once per launch) sits far below the HBM
    # roofline; the tensor-core sketch, which streams the input, is reported
    # beside it.
    peaks = load_peaks()
    orders, ks = sketch_orders(k)
    k_id = k  # ID rank ~ psvd rank before truncation
    flops = psvd_flops(n, n, k_id, k, orders, ks)
    st = {kk: v / args.steps for kk, v in stage_tot.items()}
    nl = len(orders)
    hbm = peaks.get("hbm_gbs") or 6800.0
    bf16 = peaks.get("bf16_tflops") or 1900.0
    src = "MEASURED_PEAKS.json" if peaks else "fallback (6.8 TB/s, 1.9 PFLOP/s)"
    nq = qr_launches if qr_launches > 0 else nl
    qr_bytes = sum(2 * 8.0 * l * n for l in orders) / nq            # per launch
    qr_ms = st["qr"] / nq
    pivots = sum(min(l, kq + 32) if i == nl - 1 else l for i, (l, kq) in enumerate(zip(orders, ks)))
    qr_gbs = qr_bytes / (qr_ms * 1e-3) / 1e9
    # DRAM traffic per launch: one ncu capture of the 520-row launch of this
    # workload read 34.25 MB and wrote 0.16 MB (the sketch read once); the
    # figure is scaled to the average launch by its sketch size, not
    # measured in this run
    qr_traffic = (34.25e6 + 0.16e6) * (sum(orders) / nq) / 520.0
    roof = {"kernel": "geqp3_df_smem_kernel (pivoted QR of the sketch)", "bound": "hbm", "achieved": qr_gbs,
            "peak": hbm, "unit": "GB/s", "frac": qr_gbs / hbm, "traffic": qr_traffic,
            "traffic_source": "scaled by sketch size from one ncu capture of the 520-row launch (34.4 MB)",
            "peak_source": f"{src} hbm_gbs, burst",
            "bytes_per_launch": qr_bytes, "ms_per_launch": qr_ms, "launches_per_call": nq,
            "note": f"latency-bound: {1e3 * st['qr'] / pivots:.1f} us of QR stage per pivot over {pivots} pivots "
                    f"in {nq:g} launches (several adaptive steps share a launch, each on its own CTAs), "
                    "one exchange between a step's CTAs per pivot"}
    # the sketch: six BF16 digit planes of A against the lattice Gaussian
    sk_flops = sum(2.0 * 6 * (-(-l // 96) * 96) * n * n for l in orders) / nl
    sk_ms = st["sketch"] / nl
    sk_tf = sk_flops / (sk_ms * 1e-3) / 1e12
    roof_sketch = {"kernel": "tc_sketch_kernel (S op(A), six BF16 digit planes)", "bound": "tensor",
                   "achieved": sk_tf, "peak": bf16, "unit": "TFLOP/s", "frac": sk_tf / bf16,
                   "flops_per_launch": sk_flops, "ms_per_launch": sk_ms,
                   "peak_source": f"{src} bf16_tflops, burst",
                   "note": "the sketch stage also holds the Gaussian draw and the digit split of A"}
    roof["stage_ms"] = st

    # ---- CPU baseline (oracle on the host cores, one bounded sample) -------------------
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            Ac = np.asfortranarray(A.cpu().numpy())
            dt, kc, backend, Fo, gs = cpu_reference_step(Ac, args.rtol, 5, os.cpu_count(), keep=True)
            cpu = {"value": 1.0 / dt, "unit": "matrices/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"one full {n}^2 psvdfact (oracle: numpy/OpenBLAS BLAS-3 + xLAQPS {backend}), "
                             f"rank {kc}"}
            # parity on the same sketch: the GPU path fed the oracle's stream
            Fs = lra.psvdfact(A, opts, rand=lra.RandStream(gauss=gs), ctx=ctx)
            Vs = lra.idfact(A, opts, rand=lra.RandStream(gauss=gs), ctx=ctx)
            sk_ref = np.asarray(Fo["sk"])
            kk = min(len(sk_ref), Vs.k)
            agree = int(np.argmax(np.asarray(Vs.sk[:kk]) != sk_ref[:kk])) if not np.array_equal(
                Vs.sk[:kk], sk_ref[:kk]) else kk
            x0 = np.random.default_rng(7).standard_normal(n)
            e_gpu = rel_err_psvd(A, Fs.U, Fs.S, Fs.Vt, x0)
            e_ref = rel_err_psvd(A, Fo["U"], Fo["S"], Fo["Vt"], x0)
            parity = {"stream": "lattice N(0,1) seed 5, injected into both", "rank": Fs.k, "oracle_rank": Fo["k"],
                      "id_rank": Vs.k, "oracle_id_rank": Fo["id_k"], "skeleton_prefix_equal": agree,
                      "rel_spectral_err": e_gpu, "oracle_rel_spectral_err": e_ref, "err_ratio": e_gpu / e_ref,
                      "max_rel_sv_diff": float(np.abs(np.asarray(Fs.S[:min(Fs.k, Fo["k"])]) -
                                                      np.asarray(Fo["S"][:min(Fs.k, Fo["k"])])).max() /
                                               Fo["S"][0])}
        except Exception as e:  # pragma: no cover
            cpu = cpu or {"value": None, "unit": "matrices/s", "cores": os.cpu_count(), "kind": "port",
                          "sample": f"failed: {e}"}
            parity = {"failed": str(e)}

    # ---- serving loop and batched idfact (bounded samples of those configs) ------------
    serving, batched = None, None
    if rank == 0 and args.serve_requests > 0:
        try:
            work = serving_workload(args.serve_requests)
            # two slots: the burst rate of this mix on a GB300 peaks there for
            # both precisions (1 / 2 / 4 / 8 slots: mixed 31.3 / 30.7 / 25.7 /
            # 18.2 matrices/s, FP64 9.9 / 10.2 / 9.0 / 7.1); every kernel of a
            # large request fills the GPU, so more slots mostly contend
            serving = {"mixed": measure_serving(lra, work, "mixed", slots=SERVE_SLOTS),
                       "native": measure_serving(lra, work, "native", slots=SERVE_SLOTS),
                       "sample": f"{args.serve_requests} requests of the serving config's distribution: 70% "
                                 "idfact / 30% psvdfact, m, n log-uniform [256, 16384], F32/F64 half each, "
                                 "s_i = 10^(-i/r), r ~ U[20, 200], rtol 1e-6 / 1e-10, Poisson arrivals at 80% "
                                 f"of the burst rate, {SERVE_SLOTS} slots, 150 GB budget"}
            serving["mixed_vs_native"] = serving["mixed"]["matrices_s"] / serving["native"]["matrices_s"]
            del work
        except Exception as e:  # pragma: no cover
            serving = {"failed": str(e)}
    if rank == 0 and args.batch > 0:
        try:
            mats = kernel_matrices(args.batch)
            nn = len(mats) if args.batch_native <= 0 else max(1, min(args.batch_native, len(mats)))
            batched = {"mixed": measure_batched(lra, mats, "mixed", ctx),
                       "native": measure_batched(lra, mats[:nn], "native", ctx),
                       "sample": f"{args.batch} kernel matrices 1/(1+|x-y|^2), m, n ~ U{{128..2048}}, F64, "
                                 f"rtol 1e-10, lra_idfact_batched; the FP64 path on "
                                 + ("the same batch" if nn == len(mats) else f"the first {nn}")}
            batched["mixed_vs_native"] = batched["mixed"]["matrices_s"] / batched["native"]["matrices_s"]
            del mats
        except Exception as e:  # pragma: no cover
            batched = {"failed": str(e)}

    tall = None
    if rank == 0 and not args.no_tall:
        try:
            At = tall_f32_matrix()
            tall = measure_tall(lra, ctx, At, peaks)
            tall["srft_sweep"] = measure_srft_sweep(lra, ctx, At, peaks)
            del At
        except Exception as e:  # pragma: no cover
            tall = {"failed": str(e)}

    if rank == 0:
        per_ms = sorted(1e3 * p for p in per)
        line = {
            "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"psvdfact {n}x{n} F64 U diag(s) V', s_i=10^-(i-1)/40, rtol {args.rtol}",
                       "m": n, "n": n, "rtol": args.rtol, "precision": args.precision,
                       "l2": "inputs (512 MB) larger than L2; no flush"},
            "gflops": flops / (elapsed / args.steps) / 1e9,
            "p50_ms": per_ms[len(per_ms) // 2], "p99_ms": per_ms[min(len(per_ms) - 1, int(0.99 * len(per_ms)))],
            "rank": k, "rel_spectral_err": err / nrm,
            "e2e": {"value": e2e_val, "unit": "matrices/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "fp64_path": fp64, "serving": serving, "batched": batched, "tall_f32": tall,
            "roofline": roof, "roofline_sketch": roof_sketch, "cpu_baseline": cpu, "oracle_parity": parity,
            "tuning": tuning_record(ctx),
            "clocks": clk, "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
