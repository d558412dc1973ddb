"""maxdet (strong rank-revealing QR, maxdet_swapcols! / maxdet_update!,
src/pqr.jl:445-501) with Q and R factors, and prange with maxdet, against
the oracle on the same injected streams.

* Under the reference tests' own options, LRAOptions(maxdet_tol=0.,
  sketch_randn_niter=1) (test/pqr.jl:8, test/prange.jl:7): every sketch,
  Float32 and Float64, the tests' reconstruction criteria (test/pqr.jl:29-30,
  test/prange.jl:20-29), the oracle's rank (check_rank) and the maxdet
  property max |R11^-1 R12| <= 1 + maxdet_tol.
* At a tolerance where the pivots are unambiguous and swaps do happen:
  the permutation equal to the oracle's, and R = [R1 | R1 T] and Q (after
  the re-factored R1 rotates it) equal to the oracle's to rounding."""
import numpy as np
import pytest

from test_gpu_core import both_rs
from test_oracle import check_rank, real_fourier

pytestmark = pytest.mark.gpu

SKETCHES = ["none", "randn", "sub", "srft", "sprn"]
REF_OPTS = dict(maxdet_tol=0.0, sketch_randn_niter=1)


def maxdet_t(R, k):
    """T = R11 \\ R12 of a returned R = [R11 | R12]."""
    R = np.asarray(R, np.float64)
    return np.linalg.solve(np.triu(R[:, :k]), R[:, k:]) if R.shape[1] > k else np.zeros((k, 0))


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("trans", ["n", "c"])
def test_pqrfact_reference_options(lra, oracle, sketch, dt, trans):
    A = real_fourier(128, 64).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    ors, grs = both_rs(oracle, lra, 41)
    trace = []
    ref = oracle.pqrfact(trans, A, oracle.Opts(rtol=rtol, sketch=sketch, **REF_OPTS), ors, trace=trace)
    F = lra.pqrfact(trans, A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch, **REF_OPTS), rand=grs)
    Aop = (A if trans == "n" else A.T).astype(np.float64)
    nrm = np.linalg.norm(Aop)
    assert np.linalg.norm(Aop - F.matrix()) < 100 * rtol * nrm          # test/pqr.jl:29-30
    check_rank(trace[-1]["B"], F.k, ref["k"], F.p, ref["p"], rtol, dt, name=f"{sketch} {trans}")
    k = F.k
    Q = np.asarray(F.Q, np.float64)
    assert np.abs(Q.T @ Q - np.eye(k)).max() < 1e3 * rtol * max(1, k)
    if sketch == "none" and 0 < k < Aop.shape[1]:
        # the swaps ran on the returned factors: R11 \ R12 is bounded
        T = maxdet_t(F.R, k)
        assert np.abs(T).max() <= 1 + 1e-3 * (1 if dt == np.float64 else 1e3)


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("trans", ["n", "c", "b"])
def test_prange_reference_options(lra, oracle, sketch, dt, trans):
    """prange under LRAOptions(maxdet_tol=0., sketch_randn_niter=1)
    (test/prange.jl:7-29), on a square Fourier matrix as the test builds."""
    A = real_fourier(128, 128, 6).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    ors, grs = both_rs(oracle, lra, 43)
    Qr = oracle.prange(trans, A, oracle.Opts(rtol=rtol, sketch=sketch, **REF_OPTS), ors)
    Q = lra.prange(trans, A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch, **REF_OPTS), rand=grs)
    A64, Q64 = A.astype(np.float64), np.asarray(Q, np.float64)
    nrm = np.linalg.norm(A64)
    if trans == "n":
        err = np.linalg.norm(A64 - Q64 @ (Q64.T @ A64))
    elif trans == "c":
        err = np.linalg.norm(A64 - (A64 @ Q64) @ Q64.T)
    else:
        err = np.linalg.norm(A64 - Q64 @ (Q64.T @ A64 @ Q64) @ Q64.T)
    assert err < 100 * rtol * nrm                                        # test/prange.jl:20-29
    assert np.abs(Q64.T @ Q64 - np.eye(Q.shape[1])).max() < 100 * rtol * max(1, Q.shape[1])
    assert abs(Q.shape[1] - Qr.shape[1]) <= 1


def graded(m, n, rate, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, min(m, n))))
    V, _ = np.linalg.qr(rng.standard_normal((n, min(m, n))))
    return np.asfortranarray((U * 10.0 ** (-np.arange(min(m, n)) / rate)) @ V.T)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("entry", ["pqrfact", "sketchfact"])
def test_maxdet_factors_match_oracle(lra, oracle, dt, entry):
    """Swaps that happen, on unambiguous pivots: p, R = [R1 | R1 T] and Q
    equal to the oracle's (maxdet_update!'s R1 column update, the QR of R1,
    and Q rotated by its reflectors)."""
    A = graded(120, 90, 9.0, 5).astype(dt)
    rtol = 1e-8 if dt == np.float64 else 1e-3
    tol = 1e-9 if dt == np.float64 else 2e-3
    kw = dict(rtol=rtol, maxdet_tol=0.0, pqrfact_retval="qr", sketch="none" if entry == "pqrfact" else "randn")
    ors, grs = both_rs(oracle, lra, 47)
    if entry == "pqrfact":
        ref = oracle.pqrfact("n", A, oracle.Opts(**kw), ors)
        F = lra.pqrfact(A, lra.LRAOptions(dt, **kw), rand=grs)
        plain = lra.pqrfact(A, lra.LRAOptions(dt, **dict(kw, maxdet_tol=-1.0)), rand=both_rs(oracle, lra, 47)[1])
    else:
        ref = oracle.sketchfact("left", "n", A, oracle.Opts(**kw), ors)
        F = lra.sketchfact("left", "n", A, lra.LRAOptions(dt, **kw), rand=grs)
        plain = lra.sketchfact("left", "n", A, lra.LRAOptions(dt, **dict(kw, maxdet_tol=-1.0)),
                               rand=both_rs(oracle, lra, 47)[1])
    k = F.k
    assert k == ref["k"] and 0 < k
    assert not np.array_equal(np.asarray(F.p), np.asarray(plain.p)), "no swap happened"
    assert np.array_equal(np.asarray(F.p), np.asarray(ref["p"]))
    R, R_ref = np.asarray(F.R, np.float64), np.asarray(ref["R"], np.float64)
    assert np.abs(R - R_ref).max() <= tol * np.abs(R_ref).max()
    # Q's trailing columns are fixed only up to eps / sigma_min(R11): compare
    # what Q R reproduces, and Q's orthonormality
    Q, Q_ref = np.asarray(F.Q, np.float64), np.asarray(ref["Q"], np.float64)
    assert np.abs(Q @ R - Q_ref @ R_ref).max() <= tol * np.abs(R_ref).max()
    assert np.abs(Q.T @ Q - np.eye(k)).max() <= 10 * tol
    assert np.abs(maxdet_t(R, k)).max() <= 1 + 10 * tol
