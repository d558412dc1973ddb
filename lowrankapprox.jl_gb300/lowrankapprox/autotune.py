"""Autotuner of the engine's shapes: sweeps the alternatives on this GPU and
writes the table liblra reads when a context is created
(``tuning_gb300.txt`` beside liblra.so, or the file LRA_TUNING names).

  python -m lowrankapprox.autotune [--out PATH] [--reps 3] [--quick]

What it tunes (the keys of lra_ctx_set_tuning):

* ``tc_tile_n``: the tcgen05 sketch tile N (32, 64 or 96 sketch rows per
  CTA) per element type and ceil(log2(sketch order)), timed on the Gaussian
  sketch of the mixed path at the adaptive orders 40 ... 1032, on an
  8192 x 8192 Float64 and a 65536 x 4096 Float32 matrix.  A small tile pads
  the order less; a large one reads the digit planes of op(A) fewer times.
* ``qr_seq_len``: the row count below which the double-float pivoted QR
  sums a column with one thread instead of a warp per four columns, timed
  on the grouped QR of a batch of kernel matrices (128 ... 2048 per side)
  and on the shared-memory QR of an 8192-column sketch.
* ``srft_wide``: the Float32 SRFT kernel form for l' = 128 ... 1024 (512
  threads with swizzled rows, or 256 threads with padded rows), timed on a
  65536 x 4096 matrix.

Every timing is CUDA-event time of whole library calls on device-resident
data, best of ``reps`` after a warm-up call.  The chosen values and the
times behind them are written as comments in the table.
"""
from __future__ import annotations

import argparse
import math
import os
import time

import numpy as np

from . import Context, LRAOptions, idfact, idfact_batched, sketch

HERE = os.path.dirname(os.path.abspath(__file__))
ORDERS = [40, 72, 136, 264, 520, 1032]


def _lb(order: int) -> int:
    return max(0, math.ceil(math.log2(order)))


def _time(fn, reps: int) -> float:
    import torch
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def sweep_tile_n(ctx: Context, reps: int, quick: bool):
    import torch
    out, notes = {}, []
    cases = [("f64", torch.float64, 8192, 8192), ("f32", torch.float32, 65536, 4096)]
    for tag, tdt, M, N in cases:
        if quick:
            M, N = M // 4, N // 4
        A = torch.randn((N, M), dtype=tdt, device="cuda").t()       # column-major M x N
        npdt = np.float64 if tdt == torch.float64 else np.float32
        o = LRAOptions(npdt, precision="mixed", rtol=1e-10 if npdt == np.float64 else 1e-6, seed=7)
        for order in ORDERS:
            B = torch.empty((N, order), dtype=tdt, device="cuda").t()
            times = {}
            for tn in (32, 64, 96):
                ctx.set_tuning("tc_tile_n", (16 if tag == "f64" else 0) + _lb(order), tn)
                times[tn] = _time(lambda: sketch("left", "n", A, order, o, ctx=ctx, out=B), reps)
            best = min(times, key=times.get)
            ctx.set_tuning("tc_tile_n", (16 if tag == "f64" else 0) + _lb(order), best)
            out[(tag, _lb(order))] = best
            notes.append(f"# tc_tile_n {tag} order {order} ({M}x{N}): " +
                         ", ".join(f"N={k} {v:.3f} ms" for k, v in times.items()))
        del A
    return out, notes


def _kernel_matrices(count, seed=4):
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


def sweep_qr_seq(ctx: Context, reps: int, quick: bool):
    import torch
    mats = _kernel_matrices(64 if quick else 256)
    n = 2048 if quick else 8192
    g = torch.Generator(device="cuda").manual_seed(3)
    U = torch.linalg.qr(torch.randn(n, 1024, generator=g, dtype=torch.float64, device="cuda")).Q
    V = torch.linalg.qr(torch.randn(n, 1024, generator=g, dtype=torch.float64, device="cuda")).Q
    s = torch.pow(10.0, -torch.arange(1024, dtype=torch.float64, device="cuda") / 40.0)
    A = ((U * s) @ V.T).t().contiguous().t()
    del U, V
    o = LRAOptions(rtol=1e-10, precision="mixed", seed=3)
    res, notes = {}, []
    for v in (32, 64, 96, 128, 160):
        ctx.set_tuning("qr_seq_len", 0, v)
        tb = _time(lambda: idfact_batched(mats, o, ctx=ctx), reps)

        def single():
            idfact(A, o, ctx=ctx)
        single()
        qs = []
        for _ in range(reps):
            idfact(A, o, ctx=ctx)
            qs.append(ctx.stage_ms()["qr"])
        res[v] = (tb, min(qs))
        notes.append(f"# qr_seq_len {v}: batch of {len(mats)} kernel matrices {tb:.2f} ms, "
                     f"QR stage of idfact {n}^2 {min(qs):.3f} ms")
    base = res[96]
    best = min(res, key=lambda v: res[v][0] / base[0] + res[v][1] / base[1])
    ctx.set_tuning("qr_seq_len", 0, best)
    return best, notes


def sweep_srft(ctx: Context, reps: int, quick: bool):
    import torch
    M, N = (16384, 1024) if quick else (65536, 4096)
    A = torch.randn((N, M), dtype=torch.float32, device="cuda").t()
    o = LRAOptions(np.float32, sketch="srft", seed=5)
    out, notes = {}, []
    for lb, order in ((7, 136), (8, 264), (9, 520), (10, 1032)):
        B = torch.empty((N, order), dtype=torch.float32, device="cuda").t()
        times = {}
        for wide in (0, 1):
            ctx.set_tuning("srft_wide", lb, wide)
            times[wide] = _time(lambda: sketch("left", "n", A, order, o, ctx=ctx, out=B), reps)
        best = min(times, key=times.get)
        ctx.set_tuning("srft_wide", lb, best)
        out[lb] = best
        notes.append(f"# srft_wide l'=2^{lb} ({M}x{N} Float32): padded {times[0]:.3f} ms, swizzled {times[1]:.3f} ms")
    return out, notes


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=os.path.join(HERE, "tuning_gb300.txt"))
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--quick", action="store_true", help="quarter-size workloads (a smoke run)")
    args = ap.parse_args(argv)
    import torch
    ctx = Context(0)
    t0 = time.time()
    tiles, n1 = sweep_tile_n(ctx, args.reps, args.quick)
    seq, n2 = sweep_qr_seq(ctx, args.reps, args.quick)
    wide, n3 = sweep_srft(ctx, args.reps, args.quick)
    lines = [f"# liblra tuning table, written by lowrankapprox/autotune.py on {torch.cuda.get_device_name(0)}",
             f"# ({'quick' if args.quick else 'full'} sweep, {time.time() - t0:.0f} s; best of {args.reps})"]
    lines += n1 + n2 + n3
    for (tag, lb), v in sorted(tiles.items()):
        lines.append(f"tc_tile_n {tag} {lb} {v}")
    lines.append(f"qr_seq_len {seq}")
    for lb, v in sorted(wide.items()):
        lines.append(f"srft_wide {lb} {v}")
    tmp = args.out + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, args.out)
    print("\n".join(lines))
    ctx.close()


if __name__ == "__main__":
    main()
