"""Complex element types (ComplexF32 / ComplexF64) on the GPU against the
oracle on the same injected streams: every sketch on both sides and both
transposes (crandn pairs, SRFT phases, src/sketch.jl), the pivoted QR with
ZLAQPS / CLAQPS rules against the real LAPACK routine, and idfact / pqrfact
/ psvdfact / pheigfact / curfact / prange / snorm on matrixlib(:fourier) as
the reference tests sweep them (test/id.jl:6-14 and the other test files),
with the reference tests' criteria and the oracle's ranks and pivots."""
import numpy as np
import pytest

from test_gpu_core import assert_id_parity, threshold_tie
from test_oracle import assert_pqr_parity, check_pivots
from test_oracle_complex import fourier, graded

pytestmark = pytest.mark.gpu

CDT = [np.complex64, np.complex128]
SKETCHES = ["none", "randn", "sub", "srft", "sprn"]


def streams(lra, oracle, seed, n=400000):
    rng = np.random.default_rng(seed)
    g, q = rng.standard_normal(n), rng.integers(1, 2**62, n, dtype=np.int64)
    return oracle.RandStream(gauss=g, ints=q), lra.RandStream(gauss=g, ints=q)


def rel(A, E):
    return np.linalg.norm(A - E) / np.linalg.norm(A)


@pytest.mark.parametrize("sketch", ["randn", "sub", "srft", "sprn"])
@pytest.mark.parametrize("dt", CDT)
def test_complex_sketch_values(lra, oracle, sketch, dt):
    rng = np.random.default_rng(4)
    A = np.asfortranarray((rng.standard_normal((96, 40)) + 1j * rng.standard_normal((96, 40))).astype(dt))
    tol = 1e-10 if dt == np.complex128 else 2e-4
    for side, trans in (("left", "n"), ("left", "c"), ("right", "n"), ("right", "c")):
        ors, grs = streams(lra, oracle, 12)
        B = lra.sketch(side, trans, A, 17, lra.LRAOptions(dt, sketch=sketch), rand=grs)
        R = oracle.sketch(side, trans, A, 17, oracle.Opts(sketch=sketch), ors)
        assert B.shape == R.shape and B.dtype == A.dtype
        assert np.abs(B - R).max() <= tol * max(1.0, np.abs(R).max()), (sketch, side, trans)


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).lapack_available()")
@pytest.mark.parametrize("dt", CDT)
def test_complex_geqp3_vs_lapack(lra, oracle, dt):
    import torch
    for case in [(40, 60, 6.0, 1e-8), (90, 50, 4.0, 1e-6), (30, 200, 10.0, 1e-10), (300, 120, 8.0, 1e-9)]:
        m, n, rate, rtol = case
        if dt == np.complex64:
            rtol = max(rtol, 1e-5)
        B = graded(m, n, rate, m + n, dt)
        W = B.copy(order="F")
        p_ref, t_ref, k_ref = oracle.geqp3_adap(W, oracle.Opts(rtol=rtol).for_dtype(dt), backend="lapack")
        Bd = torch.from_numpy(np.asfortranarray(B)).cuda().t().contiguous().t()
        jpvt, tau, k = lra.geqp3_adap(Bd, lra.LRAOptions(dt, rtol=rtol))
        p = jpvt.cpu().numpy()
        assert k == k_ref, case
        same = check_pivots(B, p, p_ref, k, dt, str(case))
        if same == k:
            tol = 1e-11 if dt == np.complex128 else 5e-5
            assert_pqr_parity(p, np.triu(Bd.cpu().numpy()[:k]), p_ref, np.triu(W[:k]), k, tol, str(case))


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", CDT)
@pytest.mark.parametrize("trans", ["n", "c"])
def test_complex_idfact_parity(lra, oracle, sketch, dt, trans):
    A = fourier(128, 64, 1).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    ors, grs = streams(lra, oracle, 11)
    trace = []
    ref = oracle.idfact(trans, A, oracle.Opts(rtol=rtol, sketch=sketch), ors, trace=trace)
    V = lra.idfact(trans, A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=grs)
    assert V.T.dtype == A.dtype
    Aop = A if trans == "n" else A.conj().T
    assert rel(Aop, Aop[:, V.sk - 1] @ V.matrix()) < 100 * rtol               # test/id.jl:31-32
    assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["k"], rtol, dt)


REF_OPTS = dict(maxdet_tol=0.0, sketch_randn_niter=1)


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", CDT)
def test_complex_factorizations_reference_criteria(lra, oracle, sketch, dt):
    """The reference tests' options and criteria for the complex types
    (test/pqr.jl:8-30, test/psvd.jl:29-32, test/pheig.jl:26-29,
    test/prange.jl:7-29, test/cur.jl:22-31)."""
    rtol = 5 * np.finfo(dt).eps
    A = fourier(128, 64, 1).astype(dt)
    o = lra.LRAOptions(dt, rtol=rtol, sketch=sketch, **REF_OPTS)
    oo = oracle.Opts(rtol=rtol, sketch=sketch, **REF_OPTS)
    for trans in ("n", "c"):
        ors, grs = streams(lra, oracle, 21)
        F = lra.pqrfact(trans, A, o, rand=grs)
        Aop = A if trans == "n" else A.conj().T
        assert rel(Aop, F.matrix()) < 100 * rtol                                 # test/pqr.jl:29
        Q = np.asarray(F.Q)
        assert np.abs(Q.conj().T @ Q - np.eye(F.k)).max() < 1e3 * rtol * max(1, F.k)
    for (m, n) in ((128, 64), (64, 128)):
        B = fourier(m, n, 3).astype(dt)
        ors, grs = streams(lra, oracle, 22)
        ref = oracle.psvdfact(B, oo, ors)
        P = lra.psvdfact(B, o, rand=grs)
        assert rel(B, P.matrix()) < 100 * rtol                                   # test/psvd.jl:29
        assert P.S.dtype == np.dtype(np.float32 if dt == np.complex64 else np.float64)
        assert threshold_tie(ref["S"] if ref["k"] > P.k else P.S, P.k, ref["k"], rtol * ref["S"][0], dt)
        k = min(P.k, ref["k"])
        assert np.allclose(P.S[:k], ref["S"][:k], rtol=100 * rtol, atol=100 * rtol * ref["S"][0])
    H = fourier(64, 64, 2)
    H = np.asfortranarray((H + H.conj().T).astype(dt))
    ors, grs = streams(lra, oracle, 23)
    ref = oracle.pheigfact(H, oo, ors)
    E = lra.pheigfact(H, o, rand=grs)
    assert rel(H, E.matrix()) < 100 * rtol                                       # test/pheig.jl:26
    w = ref["values"] if ref["k"] > E.k else E.values
    assert threshold_tie(w, E.k, ref["k"], rtol * np.abs(ref["values"]).max(), dt)
    for trans in ("n", "c", "b"):
        S = fourier(96, 96, 6).astype(dt)
        ors, grs = streams(lra, oracle, 24)
        Qb = np.asarray(lra.prange(trans, S, o, rand=grs), np.complex128)
        S64 = S.astype(np.complex128)
        if trans == "n":
            err = np.linalg.norm(S64 - Qb @ (Qb.conj().T @ S64))
        elif trans == "c":
            err = np.linalg.norm(S64 - (S64 @ Qb) @ Qb.conj().T)
        else:
            err = np.linalg.norm(S64 - Qb @ (Qb.conj().T @ S64 @ Qb) @ Qb.conj().T)
        assert err < 100 * rtol * np.linalg.norm(S64)                            # test/prange.jl:20-29


@pytest.mark.parametrize("dt", CDT)
def test_complex_curfact_and_snorm(lra, oracle, dt):
    rtol = 1e-4 if dt == np.complex64 else 1e-8
    A = fourier(120, 80, 7).astype(dt)
    for X in (A, np.asfortranarray(A.conj().T)):
        ors, grs = streams(lra, oracle, 31)
        U = lra.curfact(X, lra.LRAOptions(dt, rtol=rtol), rand=grs)
        F = lra.CUR(X, U)
        X64 = X.astype(np.complex128)
        E = np.asarray(F.C, np.complex128) @ ((np.asarray(F.U.U, np.complex128) * F.U.S) @
                                              np.asarray(F.U.Vt, np.complex128)) @ np.asarray(F.R, np.complex128)
        assert rel(X64, E) < 1e3 * rtol                                          # test/cur.jl:22-31
    H = fourier(50, 50, 8)
    H = np.asfortranarray((H + H.conj().T).astype(dt))
    U = lra.curfact(H, lra.LRAOptions(dt, rtol=rtol), rand=streams(lra, oracle, 32)[1])
    assert U.kind == 1
    rng = np.random.default_rng(9)
    g = rng.standard_normal(1000)
    B = (rng.random((20, 10)) + 1j * rng.random((20, 10))).astype(dt)
    C = (rng.random((20, 10)) + 1j * rng.random((20, 10))).astype(dt)
    tol = 1e-4 if dt == np.complex64 else 1e-9
    nb = np.linalg.norm(B.astype(np.complex128), 2)
    assert abs(lra.snorm(B, rand=lra.RandStream(gauss=g)) - nb) <= tol * nb             # test/snorm.jl:16
    d = lra.snormdiff(B, C, rand=lra.RandStream(gauss=g))
    dref = oracle.snormdiff_dense(B, C, oracle.Opts(), oracle.RandStream(gauss=g))
    assert abs(d - dref) <= 1e-3 * dref
