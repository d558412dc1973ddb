"""The oracle's complex element types, pinned before they are trusted:
its column-by-column restatement of ZLAQPS / CLAQPS against the real LAPACK
routine (numpy's bundled OpenBLAS, the routine the reference ccalls,
src/lapack.jl:117-139), and the reference tests' reconstruction criteria on
matrixlib(:fourier) for ComplexF32 / ComplexF64 (test/id.jl, test/pqr.jl,
test/psvd.jl, test/pheig.jl, test/prange.jl, test/cur.jl, test/snorm.jl)."""
import numpy as np
import pytest


def fourier(m, n, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(np.exp(-2j * np.pi * np.outer(rng.random(m), rng.random(n))))


def graded(m, n, rate, seed, dt):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, min(m, n))) + 1j * rng.standard_normal((m, min(m, n))))
    V, _ = np.linalg.qr(rng.standard_normal((n, min(m, n))) + 1j * rng.standard_normal((n, min(m, n))))
    return np.asfortranarray(((U * 10.0 ** (-np.arange(min(m, n)) / rate)) @ V.conj().T).astype(dt))


def rs(oracle, seed, n=200000):
    rng = np.random.default_rng(seed)
    return oracle.RandStream(gauss=rng.standard_normal(n), ints=rng.integers(1, 2**62, n, dtype=np.int64))


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).lapack_available()")
@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
@pytest.mark.parametrize("case", [(40, 60, 6.0, 1e-8), (90, 50, 4.0, 1e-6), (30, 200, 10.0, 1e-10)])
def test_complex_laqps_restatement_matches_lapack(oracle, dt, case):
    m, n, rate, rtol = case
    if dt == np.complex64:
        rtol = max(rtol, 1e-5)
    B = graded(m, n, rate, m + n, dt)
    o = oracle.Opts(rtol=rtol).for_dtype(dt)
    W1, W2 = B.copy(order="F"), B.copy(order="F")
    p1, t1, k1 = oracle.geqp3_adap(W1, o, backend="lapack")
    p2, t2, k2 = oracle.geqp3_adap(W2, o, backend="oracle")
    assert k1 == k2 > 0
    assert np.array_equal(p1[:k1], p2[:k1])
    tol = 1e-11 if dt == np.complex128 else 2e-5
    # R11 and R12 with the columns after the rank aligned by index (their
    # order is decided among pivots below the rank tolerance)
    from test_oracle import assert_pqr_parity
    assert_pqr_parity(p2, np.triu(W2[:k2]), p1, np.triu(W1[:k1]), k1, tol, str(case))
    # tau_i is fixed to ~eps ||B|| / |R_ii|: compare it scaled by |R_ii|
    d = np.abs(np.diag(W1[:k1, :k1]))
    assert np.all(np.abs(t1[:k1] - t2[:k1]) * d <= 10 * tol * d.max())


SKETCHES = ["none", "randn", "sub", "srft", "sprn"]


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_reference_criteria_complex(oracle, sketch, dt):
    """test/id.jl:31-32, test/pqr.jl:29, test/psvd.jl:29, test/pheig.jl:26
    on M = matrixlib(:fourier, rand(128), rand(64)), complex types, with the
    tests' options LRAOptions(maxdet_tol=0., sketch_randn_niter=1)."""
    A = fourier(128, 64, 1).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    o = oracle.Opts(rtol=rtol, sketch=sketch, maxdet_tol=0.0, sketch_randn_niter=1)
    nrm = np.linalg.norm(A)
    for trans in ("n", "c"):
        V = oracle.idfact(trans, A, o, rs(oracle, 3))
        Aop = A if trans == "n" else A.conj().T
        assert np.linalg.norm(Aop - oracle.id_matrix(trans, A, V)) < 100 * rtol * nrm
        F = oracle.pqrfact(trans, A, o, rs(oracle, 4))
        P = np.zeros(Aop.shape, np.complex128)
        P[:, F["p"] - 1] = F["Q"] @ F["R"]
        assert np.linalg.norm(Aop - P) < 100 * rtol * nrm
    S = oracle.psvdfact(A, o, rs(oracle, 5))
    assert np.linalg.norm(A - (S["U"] * S["S"]) @ S["Vt"]) < 100 * rtol * nrm
    H = fourier(64, 64, 2)
    H = (H + H.conj().T).astype(dt)
    E = oracle.pheigfact(H, o, rs(oracle, 6))
    assert np.linalg.norm(H - (E["vectors"] * E["values"]) @ E["vectors"].conj().T) < 100 * rtol * np.linalg.norm(H)
    Q = oracle.prange("n", A, o, rs(oracle, 7))
    assert np.linalg.norm(A - Q @ (Q.conj().T @ A)) < 100 * rtol * nrm


def test_complex_snorm(oracle):
    """test/snorm.jl:16-25: snorm of a complex matrix and a difference."""
    rng = np.random.default_rng(8)
    A = rng.random((20, 10)) + 1j * rng.random((20, 10))
    B = rng.random((20, 10)) + 1j * rng.random((20, 10))
    g = oracle.RandStream(gauss=rng.standard_normal(1000))
    assert abs(oracle.snorm_dense(A, oracle.Opts(), g) - np.linalg.norm(A, 2)) <= 1e-10 * np.linalg.norm(A, 2)
    g = oracle.RandStream(gauss=rng.standard_normal(1000))
    d = oracle.snormdiff_dense(A, B, oracle.Opts(), g)
    assert abs(d - np.linalg.norm(A - B, 2)) <= 1e-6 * np.linalg.norm(A - B, 2)
