"""Adaptive steps factored together (sketchfact_dev's launches of several
steps, geqp3_adap_steps): after a step whose rank reached its threshold, the
steps up to the one that should reveal the rank are sketched in order and
factored by one launch of the shared-memory pivoted QR, each on CTAs of its
own.  The pivoted QR's arithmetic per column does not depend on how many
CTAs hold the columns, so every result must be bit-identical to the
step-by-step loop (tuning qr_steps = 1), which follows the reference's
sketchfact loop (src/sketch.jl:223-240):

* Float64 on the mixed path and Float32 on both paths, Gaussian and SRFT
  sketches, the library generator and injected streams;
* a spectrum with a cliff, where the prediction overshoots and a step in the
  middle of the launch reveals the rank (the later steps are stopped);
* curfact, whose two sketchfact calls draw from one stream (a step drawn
  ahead and not used must leave the stream where the step-by-step loop
  would);
* an injected stream just long enough for the step-by-step loop (a step
  drawn ahead past its end is left out, not an error);
* fewer pivoted-QR launches than the step-by-step loop, so the shared
  launch did run."""
import numpy as np
import pytest

from test_gpu_mixed import decaying

pytestmark = pytest.mark.gpu

QR_KERNELS = ("geqp3_df_smem_kernel", "geqp3_f32_smem_kernel", "geqp3_df_kernel", "geqp3_v2_kernel")


def cliff(m, n, keep, seed, rate=200.0):
    """Slowly decaying singular values 10^(-i/rate) for i < keep, then 1e-15:
    the first step's diagonal predicts a rank far above keep."""
    rng = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = np.where(np.arange(r) < keep, 10.0 ** (-np.arange(r) / rate), 1e-15)
    return np.asfortranarray((U * s) @ V.T)


def two_ways(lra, call):
    """call(ctx) with the steps factored together and one at a time, each on
    a fresh context; the results and the launch counts."""
    out = []
    for steps in (8, 1):
        ctx = lra.Context(0)
        ctx.set_tuning("qr_steps", 0, steps)
        r = call(ctx)
        out.append((r, sum(ctx.kernel_launches(k) for k in QR_KERNELS)))
        ctx.close()
    return out


def same_id(a, b):
    assert a.k == b.k and a.nsteps == b.nsteps
    assert np.array_equal(a.sk, b.sk) and np.array_equal(a.rd, b.rd)
    assert np.array_equal(np.asarray(a.T), np.asarray(b.T))


@pytest.mark.parametrize("case", ["f64-mixed-randn", "f64-mixed-srft", "f32-mixed-randn", "f32-native-srft",
                                  "f32-native-randn"])
@pytest.mark.parametrize("stream", ["library", "injected"])
def test_steps_together_same_bits(lra, case, stream):
    dt = np.float64 if case.startswith("f64") else np.float32
    prec = "mixed" if "mixed" in case else "native"
    sk = case.split("-")[-1]
    rtol = 1e-10 if dt == np.float64 else 1e-5
    A = decaying(2400, 1500, 30.0 if dt == np.float64 else 50.0, 3).astype(dt)
    o = lra.LRAOptions(dt, rtol=rtol, sketch=sk, precision=prec, seed=11)
    g = lra.lattice_gauss(12, 8_000_000)
    q = np.random.default_rng(13).integers(1, 2**62, 400_000, dtype=np.int64)

    def call(ctx):
        rand = lra.RandStream(gauss=g, ints=q) if stream == "injected" else None
        return lra.idfact(A, o, rand=rand, ctx=ctx)

    (V1, n1), (V0, n0) = two_ways(lra, call)
    same_id(V1, V0)
    assert V1.nsteps >= 3
    # how many steps share a launch follows a prediction of the rank; on the
    # Gaussian sketch of this spectrum it groups
    if sk == "randn":
        assert n1 < n0, (n1, n0)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_rank_revealed_inside_a_launch(lra, dt):
    rtol = 1e-10 if dt == np.float64 else 1e-5
    A = cliff(2000, 1800, 150, 5).astype(dt)
    o = lra.LRAOptions(dt, rtol=rtol, precision="mixed", seed=3)
    (V1, n1), (V0, n0) = two_ways(lra, lambda ctx: lra.idfact(A, o, ctx=ctx))
    same_id(V1, V0)
    assert V1.k >= 150 - 2 and V1.k < 256


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_psvdfact_and_curfact(lra, dt):
    rtol = 1e-10 if dt == np.float64 else 1e-5
    A = decaying(1800, 1300, 28.0 if dt == np.float64 else 45.0, 8).astype(dt)
    o = lra.LRAOptions(dt, rtol=rtol, precision="mixed", seed=21)
    g = lra.lattice_gauss(22, 8_000_000)
    (P1, _), (P0, _) = two_ways(lra, lambda ctx: lra.psvdfact(A, o, rand=lra.RandStream(gauss=g), ctx=ctx))
    assert P1.k == P0.k
    for a, b in ((P1.U, P0.U), (P1.S, P0.S), (P1.Vt, P0.Vt)):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    # two sketchfact calls on one stream: the second sees the same positions
    (U1, _), (U0, _) = two_ways(lra, lambda ctx: lra.curfact(A, o, rand=lra.RandStream(gauss=g), ctx=ctx))
    assert np.array_equal(U1.rows, U0.rows) and np.array_equal(U1.cols, U0.cols)


def test_stream_just_long_enough(lra):
    """The Gaussian stream holds exactly the step-by-step loop's draws; the
    steps drawn ahead past its end are left out of the launch."""
    A = decaying(2200, 1400, 30.0, 9)
    M = A.shape[0]
    o = lra.LRAOptions(np.float64, rtol=1e-10, precision="mixed", seed=4)
    g = lra.lattice_gauss(31, 8_000_000)
    ctx = lra.Context(0)
    ctx.set_tuning("qr_steps", 0, 1)
    V = lra.idfact(A, o, rand=lra.RandStream(gauss=g), ctx=ctx)
    ctx.close()
    a, b = o.sketchfact_randn_samp
    need = sum((a * (o.nb << t) + b) * M for t in range(V.nsteps))
    gs = g[:need].copy()
    (V1, _), (V0, _) = two_ways(lra, lambda ctx: lra.idfact(A, o, rand=lra.RandStream(gauss=gs), ctx=ctx))
    same_id(V1, V0)
    same_id(V0, V)
