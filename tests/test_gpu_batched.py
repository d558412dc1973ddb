"""lra_idfact_batched on the mixed path: Float64 matrices, tensor-core sketch,
the sketches of the whole batch factored by one grouped launch (a CTA per
matrix).  Each result must be exactly what lra_idfact returns for the matrix
on a fresh context (stated tolerance 0: same rank, same skeleton, same T bit
for bit), and the interpolative decomposition must meet the requested rtol."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def kernel_matrix(m, n, seed):
    """K(x, y) = 1 / (1 + |x - y|^2), x ~ U[0,1]^2, y ~ U[1.5,2.5] x U[0,1]."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (m, 2))
    y = np.column_stack([rng.uniform(1.5, 2.5, n), rng.uniform(0, 1, n)])
    d2 = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    return np.asfortranarray(1.0 / (1.0 + d2))


def decaying(m, n, rate, seed):
    rng = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = 10.0 ** (-np.arange(r) / rate)
    return np.asfortranarray((U * s) @ V.T)


def batch():
    shapes = [(128, 128), (300, 170), (140, 900), (700, 700), (513, 257), (1000, 350), (200, 1500), (129, 131)]
    mats = [kernel_matrix(m, n, 10 + i) for i, (m, n) in enumerate(shapes)]
    # ranks beyond the first sketch sizes, so that matrices leave the batch in different rounds
    mats += [decaying(600, 400, 8.0, 3), decaying(400, 800, 25.0, 4), decaying(256, 256, 60.0, 5)]
    return mats


def single(lra, A, o):
    ctx = lra.Context()
    try:
        return lra.idfact(A, o, ctx=ctx)
    finally:
        ctx.close()


def id_error(A, V):
    k = V.k
    sk, rd = V.sk - 1, V.rd - 1
    E = A[:, rd] - A[:, sk] @ V.T
    return np.linalg.norm(E, 2) / np.linalg.norm(A, 2)


def test_grouped_batch_same_as_single(lra):
    mats = batch()
    o = lra.LRAOptions(rtol=1e-10, precision="mixed", seed=3)
    ctx = lra.Context()
    try:
        before = ctx.launches
        Vs = lra.idfact_batched(mats, o, ctx=ctx)
        # the grouped path runs on the caller's context (the fallback runs on
        # worker contexts of its own)
        assert ctx.launches - before > 0
    finally:
        ctx.close()
    steps = set()
    for A, V in zip(mats, Vs):
        R = single(lra, A, o)
        assert V.k == R.k and V.nsteps == R.nsteps
        assert np.array_equal(V.sk, R.sk) and np.array_equal(V.rd, R.rd)
        assert np.array_equal(V.T, R.T)
        # the ID's error is |R22| times a factor of order sqrt(1 + |T|^2),
        # with |R22| <= rtol |A| at the rank the QR stopped
        assert id_error(A, V) < 50 * 1e-10 * np.sqrt(1 + np.linalg.norm(V.T, 2) ** 2)
        steps.add(V.nsteps)
    assert len(steps) > 1  # the rounds retire matrices at different steps


def test_grouped_batch_chunks_and_order(lra):
    # the same matrix twice, far apart in a longer batch: equal results
    mats = batch()
    mats = mats + mats[::-1]
    o = lra.LRAOptions(rtol=1e-10, precision="mixed", seed=9)
    Vs = lra.idfact_batched(mats, o)
    n = len(mats) // 2
    for i in range(n):
        a, b = Vs[i], Vs[len(mats) - 1 - i]
        assert a.k == b.k and np.array_equal(a.sk, b.sk) and np.array_equal(a.T, b.T)


def test_grouped_batch_nonfinite(lra):
    mats = batch()[:3]
    mats[1] = mats[1].copy()
    mats[1][5, 7] = np.nan
    o = lra.LRAOptions(rtol=1e-10, precision="mixed")
    with pytest.raises(lra.LRAError):
        lra.idfact_batched(mats, o)


def test_native_batch_falls_back(lra):
    # native precision keeps the per-matrix path (worker contexts)
    mats = batch()[:4]
    o = lra.LRAOptions(rtol=1e-10, precision="native", seed=3)
    ctx = lra.Context()
    try:
        before = ctx.launches
        Vs = lra.idfact_batched(mats, o, ctx=ctx)
        assert ctx.launches == before
    finally:
        ctx.close()
    for A, V in zip(mats, Vs):
        R = single(lra, A, o)
        assert V.k == R.k and np.array_equal(V.sk, R.sk) and np.array_equal(V.T, R.T)
