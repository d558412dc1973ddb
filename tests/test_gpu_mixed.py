"""The mixed-precision path: the Gaussian sketch on tcgen05 tensor cores from
exact BF16 byte slices.  Checked against the FP64 product of the same
lattice sketch, at tile-edge shapes, and end to end against the oracle."""
import numpy as np
import pytest

from test_gpu_core import dev, relerr
from test_oracle import check_pivots

pytestmark = pytest.mark.gpu


def lattice(seed, n):
    import lowrankapprox as L
    return L.lattice_gauss(seed, n)


@pytest.mark.parametrize("shape,order", [((300, 200), 40), ((1000, 130), 136), ((64, 257), 264),
                                         ((2048, 640), 520), ((129, 1), 17)])
@pytest.mark.parametrize("trans", ["n", "c"])
def test_tc_sketch_exact(lra, shape, order, trans):
    rng = np.random.default_rng(sum(shape) + order)
    m, n = shape
    # columns with wildly different scales, exercising the per-column exponent
    A = np.asfortranarray(rng.standard_normal((m, n)) * np.exp(rng.uniform(-30, 30, (1, n))) *
                          np.exp(rng.uniform(-3, 3, (m, 1))))
    M = m if trans == "n" else n
    g = lattice(3, order * M + 10)
    B = lra.sketch("left", trans, A, order, lra.LRAOptions(precision="mixed", rtol=1e-10),
                   rand=lra.RandStream(gauss=g))
    S = g[:order * M].reshape((order, M), order="F")
    opA = A if trans == "n" else A.T
    R = S @ opA
    # truncation of op(A) at 2^-48 of each column's scale, times |S|, plus the
    # integer rounding of the tail accumulator (half a unit of 2^(e-45) per
    # 512-long chunk)
    colmax = np.abs(opA).max(axis=0)
    chunks = -(-M // 512)
    bound = 2.0 ** -47 * (np.abs(S).sum(axis=1)[:, None] * colmax[None, :]) + 4 * np.finfo(float).eps * np.abs(R) \
        + chunks * 2.0 ** -44 * colmax[None, :]
    assert np.all(np.abs(B - R) <= bound + 1e-300)


def test_tc_sketch_f32(lra):
    rng = np.random.default_rng(7)
    A = np.asfortranarray(rng.standard_normal((700, 333)).astype(np.float32))
    order = 72
    g = lattice(4, order * 700)
    B = lra.sketch("left", "n", A, order, lra.LRAOptions(np.float32, precision="mixed"),
                   rand=lra.RandStream(gauss=g))
    R = g.reshape((order, 700), order="F") @ A.astype(np.float64)
    assert np.abs(B - R).max() <= 1e-5 * np.abs(R).max()


def decaying(m, n, rate, seed):
    rng = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = 10.0 ** (-np.arange(r) / rate)
    return np.asfortranarray((U * s) @ V.T)


@pytest.mark.parametrize("trans", ["n", "c"])
def test_idfact_mixed_parity(lra, oracle, trans):
    A = decaying(1100, 900, 25.0, 1)
    g = lattice(5, 4_000_000)
    ref = oracle.idfact(trans, A, oracle.Opts(rtol=1e-10), oracle.RandStream(gauss=g))
    V = lra.idfact(trans, A, lra.LRAOptions(rtol=1e-10, precision="mixed"), rand=lra.RandStream(gauss=g))
    assert V.k == ref["k"]
    Aop = A if trans == "n" else A.T
    M = Aop.shape[0]
    # the final step's sketch, to assess near-ties
    off = sum((32 * 2 ** t + 8) * M for t in range(V.nsteps - 1))
    order = 32 * 2 ** (V.nsteps - 1) + 8
    B = g[off:off + order * M].reshape((order, M), order="F") @ Aop
    check_pivots(B, V.sk, ref["sk"], V.k, np.float64)
    e = np.linalg.norm(Aop - Aop[:, V.sk - 1] @ V.matrix(), 2) / np.linalg.norm(Aop, 2)
    e_ref = np.linalg.norm(Aop - Aop[:, ref["sk"] - 1] @ oracle._v_matrix(ref, Aop.shape[1], A.dtype), 2) / \
        np.linalg.norm(Aop, 2)
    assert e <= 2 * e_ref + 1e-15


def test_psvd_mixed_vs_native(lra):
    A = decaying(1536, 1024, 40.0, 2)
    g = lattice(6, 6_000_000)
    Fm = lra.psvdfact(A, lra.LRAOptions(rtol=1e-10, precision="mixed"), rand=lra.RandStream(gauss=g))
    Fn = lra.psvdfact(A, lra.LRAOptions(rtol=1e-10, precision="native"), rand=lra.RandStream(gauss=g))
    assert abs(Fm.k - Fn.k) <= 1
    nrm = np.linalg.norm(A, 2)
    em = np.linalg.norm(A - Fm.matrix(), 2) / nrm
    en = np.linalg.norm(A - Fn.matrix(), 2) / nrm
    assert em <= 2 * en + 1e-14
    assert em < 1e-9
    k = min(Fm.k, Fn.k)
    assert np.allclose(Fm.S[:k], Fn.S[:k], rtol=1e-8, atol=1e-12 * Fn.S[0])
    assert np.abs(Fm.U.T @ Fm.U - np.eye(Fm.k)).max() < 1e-11
    assert np.abs(Fm.Vt @ Fm.Vt.T - np.eye(Fm.k)).max() < 1e-10


def test_mixed_device_input(lra):
    A = decaying(800, 600, 20.0, 3)
    g = lattice(8, 2_000_000)
    o = lra.LRAOptions(rtol=1e-10, precision="mixed")
    V1 = lra.idfact(A, o, rand=lra.RandStream(gauss=g))
    V2 = lra.idfact(dev(A), o, rand=lra.RandStream(gauss=g))
    assert V1.k == V2.k and np.array_equal(V1.sk, V2.sk) and np.array_equal(V1.T, V2.T)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize(
    "M,order",
    [(4096, 72), (2048, 520), (1536, 136), (65536, 40), (65536, 72), (65536, 136), (65536, 264), (65536, 1032),
     (32768, 520), (8192, 264),
     # outside the FFT kernel's range: odd m2 = 3, and l' = 2048
     (1536, 520), (4096, 2100)])
def test_srft_fft_path(lra, oracle, dt, M, order):
    """SRFT through l'-point FFTs (l' a power of two) against the full-length
    FFT of the same signs and frequencies; the tall shapes run whole chunks
    of the decimation-in-frequency kernel, the short ones partial chunks and
    the fallback."""
    rng = np.random.default_rng(M + order)
    A = np.asfortranarray(rng.standard_normal((M, 300 if M <= 4096 else 48)).astype(dt))
    g = rng.standard_normal(M + 10)
    q = rng.integers(1, 2**62, order + 10, dtype=np.int64)
    B = lra.sketch("left", "n", A, order, lra.LRAOptions(dt, sketch="srft"), rand=lra.RandStream(gauss=g, ints=q))
    d = np.where(g[:M] > 0, 1.0, -1.0)
    idx = (q[:order] - 1) % M + 1
    R = oracle.srft_exact(A.astype(np.float64), d, idx, order)
    tol = 1e-10 if dt == np.float64 else 2e-5
    assert np.abs(B - R).max() <= tol * np.abs(R).max()


def test_sketch_into_device_tensor(lra):
    """sketch(..., out=B) with B a column-major CUDA tensor: the same values
    as the host result; a tensor of the wrong shape is refused."""
    import torch
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.standard_normal((4096, 64)).astype(np.float32))
    g = rng.standard_normal(5000)
    q = rng.integers(1, 2**62, 600, dtype=np.int64)
    o = lra.LRAOptions(np.float32, sketch="srft")
    H = lra.sketch("left", "n", A, 264, o, rand=lra.RandStream(gauss=g, ints=q))
    B = torch.empty((64, 264), dtype=torch.float32, device="cuda").t()
    R = lra.sketch("left", "n", A, 264, o, rand=lra.RandStream(gauss=g, ints=q), out=B)
    assert R is B
    assert np.array_equal(B.cpu().numpy(), H)
    with pytest.raises(lra.LRAError):
        lra.sketch("left", "n", A, 264, o, out=torch.empty((64, 263), dtype=torch.float32, device="cuda").t())


def test_psvd_mixed_clustered(lra):
    """Clusters of equal singular values: the Gram polish's simultaneous
    rotations interfere inside a cluster; the result must still match the
    FP64 path (the pairwise sweeps take over when the polish stalls)."""
    rng = np.random.default_rng(12)
    m, n = 1024, 768
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.concatenate([np.ones(40), 0.5 * np.ones(40), 0.25 * 10.0 ** (-np.arange(n - 80) / 20.0)])
    A = np.asfortranarray((U * s) @ V.T)
    g = lattice(13, 6_000_000)
    Fm = lra.psvdfact(A, lra.LRAOptions(rtol=1e-10, precision="mixed"), rand=lra.RandStream(gauss=g))
    Fn = lra.psvdfact(A, lra.LRAOptions(rtol=1e-10, precision="native"), rand=lra.RandStream(gauss=g))
    assert abs(Fm.k - Fn.k) <= 1
    nrm = np.linalg.norm(A, 2)
    em = np.linalg.norm(A - Fm.matrix(), 2) / nrm
    en = np.linalg.norm(A - Fn.matrix(), 2) / nrm
    assert em <= 2 * en + 1e-14 and em < 1e-9
    # orthonormal factors to well below rtol (the mixed path's products
    # carry tensor-core rounding of ~2^-45 per GEMM)
    k = Fm.k
    assert np.abs(Fm.U.T @ Fm.U - np.eye(k)).max() < 1e-11
    assert np.abs(Fm.Vt @ Fm.Vt.T - np.eye(k)).max() < 1e-10
    assert np.allclose(Fm.S[:80], s[:80], rtol=1e-12)


def test_mixed_q_factors(lra):
    """A Q built from the pivoted QR's reflectors on the mixed path (the
    double-float shared-memory kernel): pqrfact with sketch :none, the
    right sketchfact's Q and prange give orthonormal bases that reproduce
    A (the reflectors below the diagonal carry no scale)."""
    A = decaying(700, 500, 20.0, 9) * 37.0          # a scale far from 1
    rtol = 1e-10
    o = lra.LRAOptions(rtol=rtol, precision="mixed")
    F = lra.pqrfact(A, o.copy(sketch="none"))
    Q = np.asarray(F.Q)
    assert np.abs(Q.T @ Q - np.eye(F.k)).max() < 1e-12
    assert relerr(A, F.matrix()) < 100 * rtol
    g = lattice(14, 4_000_000)
    S = lra.sketchfact("right", "n", A, o.copy(pqrfact_retval="qr"), rand=lra.RandStream(gauss=g))
    Qs = np.asarray(S.Q)
    assert np.abs(Qs.T @ Qs - np.eye(S.k)).max() < 1e-12
    assert np.linalg.norm(A - Qs @ (Qs.T @ A)) <= 100 * rtol * np.linalg.norm(A)
    P = np.asarray(lra.prange("n", A, o, rand=lra.RandStream(gauss=g)))
    assert np.abs(P.T @ P - np.eye(P.shape[1])).max() < 1e-12
    assert np.linalg.norm(A - P @ (P.T @ A)) <= 100 * rtol * np.linalg.norm(A)


@pytest.mark.parametrize("shape", [(72, 900), (264, 4096), (1032, 4096), (40, 300)])
def test_f32_shared_memory_qr_vs_oracle(lra, oracle, shape):
    """Float32 sketches factored in shared memory (the one-word exchange
    kernel in FP32) against the real LAPACK SLAQPS: rank, pivots up to a
    demonstrated near-tie, R and tau."""
    import torch
    from test_oracle import assert_pqr_parity, check_rank
    m, n = shape
    rng = np.random.default_rng(m + n)
    B = (rng.standard_normal((m, n)) @ np.diag(np.exp(-np.arange(n) / (n / 12.0))) * 3.0).astype(np.float32)
    B = np.asfortranarray(B)
    rtol = 1e-5
    W = B.copy(order="F")
    be = "lapack" if oracle.lapack_available() else "c"
    p_ref, t_ref, k_ref = oracle.geqp3_adap(W, oracle.Opts(rtol=rtol).for_dtype(np.float32), backend=be)
    Bd = torch.from_numpy(B).cuda().t().contiguous().t()
    jpvt, tau, k = lra.geqp3_adap(Bd, lra.LRAOptions(np.float32, rtol=rtol))
    p = jpvt.cpu().numpy()
    check_rank(B, k, k_ref, p, p_ref, rtol, np.float32)
    same = check_pivots(B, p, p_ref, min(k, k_ref), np.float32)
    if same == k == k_ref:
        assert_pqr_parity(p, np.triu(Bd.cpu().numpy()[:k]), p_ref, np.triu(W[:k]), k, 5e-5)


@pytest.mark.parametrize("shape", [(2600, 1500, 110.0, 1024), (3000, 2200, 180.0, 1700)])
def test_psvd_large_rank(lra, shape):
    """psvdfact at ranks where the core SVD's FP32 block Jacobi keeps V in
    shared memory (k ~ 1100) and in global memory (k ~ 1800), and the Gram
    polish gives the near-equal pairs it leaves exact rotations: the
    reference test's criterion (test/psvd.jl:29), the singular values
    against numpy's to the rank threshold, orthonormal U and V."""
    m, n, rate, kmin = shape
    A = decaying(m, n, rate, 12)
    rtol = 1e-10
    F = lra.psvdfact(A, lra.LRAOptions(rtol=rtol, precision="mixed", seed=3))
    assert F.k >= kmin
    E = (np.asarray(F.U) * F.S) @ np.asarray(F.Vt)
    assert np.linalg.norm(A - E) < 100 * rtol * np.linalg.norm(A)
    s = np.linalg.svd(A, compute_uv=False)
    assert np.abs(F.S - s[:F.k]).max() <= 10 * rtol * s[0]
    for Q in (np.asarray(F.U), np.asarray(F.Vt).T):
        assert np.abs(Q.T @ Q - np.eye(F.k)).max() < 1e-8
