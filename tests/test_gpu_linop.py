"""Matrix-free operators (LinearOperator / HermitianLinearOperator,
src/linop.jl:9-40) through the lra_*_linop entry points: the library calls
back into the operator's products on its own stream.

* The operator algebra of test/linop.jl (products, adjoints, scalar
  multiples, sums), on the Python mirror.
* idfact / pqrfact / psvdfact / pheigfact / curfact / prange / snorm of an
  operator against the oracle run on the operator's dense matrix with the
  Gaussian sketch (the reference forces :randn for operators, chkopts!,
  src/LowRankApprox.jl:142-148), on the same injected stream; the reference
  tests' reconstruction criteria (test/id.jl:31, test/psvd.jl:29,
  test/pheig.jl:26, test/pqr.jl:29)."""
import numpy as np
import pytest

from test_gpu_core import assert_id_parity, both_rs, dev, relerr
from test_oracle import real_fourier

pytestmark = pytest.mark.gpu


def _op(lra, A, hermitian=None):
    return lra.LinearOperator.from_matrix(dev(A), hermitian=hermitian)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("herm", [False, True])
def test_operator_algebra(lra, dt, herm):
    """test/linop.jl:6-60: an operator applies like its matrix, and so do
    its adjoint, scalar multiples, sums and products."""
    import torch
    rng = np.random.default_rng(3)
    A = rng.random((10, 10)).astype(dt)
    if herm:
        A = A + A.T
    L = _op(lra, A)
    assert L.hermitian == herm
    tol = 1e-5 if dt == np.float32 else 1e-12
    Ad = dev(A)
    X = torch.as_tensor(rng.random((10, 4)).astype(dt), device="cuda")
    close = lambda P, Q: torch.allclose(P, Q, rtol=tol, atol=tol)
    assert close(L.matrix(), Ad)
    assert close(L.H.matrix(), Ad.T)
    assert close(L @ X, Ad @ X) and close(L.H @ X, Ad.T @ X)
    c = 0.37
    assert close((c * L) @ X, c * (Ad @ X)) and close((L / c).H @ X, (Ad.T @ X) / c)
    M = L + c * L
    assert close(M @ X, (1 + c) * (Ad @ X))
    P = L @ L.H
    assert close(P @ X, Ad @ (Ad.T @ X)) and close(P.H @ X, Ad @ (Ad.T @ X))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("trans", ["n", "c"])
def test_idfact_operator_vs_oracle(lra, oracle, dt, trans):
    A = real_fourier(128, 64, 2).astype(dt)
    rtol = 1e-5 if dt == np.float32 else 1e-10
    ors, grs = both_rs(oracle, lra, 61)
    trace = []
    # an operator's sketch is the Gaussian one whatever the options say
    ref = oracle.idfact(trans, A, oracle.Opts(rtol=rtol, sketch="randn"), ors, trace=trace)
    V = lra.idfact(trans, _op(lra, A), lra.LRAOptions(dt, rtol=rtol, sketch="srft"), rand=grs)
    assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["k"], rtol, dt)
    Aop = (A if trans == "n" else A.T).astype(np.float64)
    assert relerr(Aop, Aop[:, V.sk - 1] @ V.matrix().astype(np.float64)) < 100 * rtol   # test/id.jl:31


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_factorizations_of_an_operator(lra, oracle, dt):
    rtol = 1e-5 if dt == np.float32 else 1e-10
    A = real_fourier(120, 90, 4).astype(dt)
    L = _op(lra, A)
    o = lra.LRAOptions(dt, rtol=rtol, sketch_randn_niter=1)
    ors, grs = both_rs(oracle, lra, 63)
    # pqrfact (src/pqr.jl:290-307): Q R P' reconstructs A
    F = lra.pqrfact(L, o, rand=grs)
    assert relerr(A.astype(np.float64), F.matrix()) < 100 * rtol                      # test/pqr.jl:29
    # psvdfact (src/psvd.jl:238-272) against the oracle's singular values
    ref = oracle.psvdfact(A, oracle.Opts(rtol=rtol, sketch_randn_niter=1), ors)
    P = lra.psvdfact(L, o, rand=both_rs(oracle, lra, 63)[1])
    assert relerr(A.astype(np.float64), P.matrix()) < 100 * rtol                      # test/psvd.jl:29
    k = min(P.k, ref["k"])
    assert abs(P.k - ref["k"]) <= 1
    assert np.allclose(P.S[:k], ref["S"][:k], rtol=100 * rtol, atol=100 * rtol * ref["S"][0])
    s = lra.psvdvals(L, o, rand=both_rs(oracle, lra, 63)[1])
    assert np.allclose(s, P.S, rtol=100 * rtol, atol=100 * rtol * P.S[0])
    # prange (src/prange.jl:14-61)
    Q = np.asarray(lra.prange("n", L, o, rand=both_rs(oracle, lra, 63)[1]), np.float64)
    A64 = A.astype(np.float64)
    assert np.linalg.norm(A64 - Q @ (Q.T @ A64)) < 100 * rtol * np.linalg.norm(A64)   # test/prange.jl:20
    # curfact (src/cur.jl:532-564): rows and cols of A
    U = lra.curfact(L, o, rand=both_rs(oracle, lra, 63)[1])
    Cm = A64[:, U.cols - 1]
    Rm = A64[U.rows - 1, :]
    u, sv, vt = np.linalg.svd(Cm[U.rows - 1, :])
    keep = sv > sv[0] * rtol
    E = Cm @ ((vt[keep].T / sv[keep]) @ u[:, keep].T) @ Rm
    assert relerr(A64, E) < 1e3 * rtol
    # snorm (src/snorm.jl:14-45)
    nrm = lra.snorm(L, rand=lra.RandStream(gauss=np.random.default_rng(5).standard_normal(200)))
    assert abs(nrm - np.linalg.norm(A64, 2)) <= 1e-4 * np.linalg.norm(A64, 2)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_pheigfact_hermitian_operator(lra, oracle, dt):
    rtol = 1e-5 if dt == np.float32 else 1e-10
    H = real_fourier(100, 100, 5)
    H = (H + H.T).astype(dt)
    L = _op(lra, H)
    assert L.hermitian
    ors, grs = both_rs(oracle, lra, 65)
    ref = oracle.pheigfact(H, oracle.Opts(rtol=rtol), ors)
    F = lra.pheigfact(L, lra.LRAOptions(dt, rtol=rtol), rand=grs)
    assert relerr(H.astype(np.float64), F.matrix()) < 100 * rtol                      # test/pheig.jl:26
    if F.k == ref["k"]:
        assert np.allclose(F.values, ref["values"], atol=100 * rtol * np.abs(ref["values"]).max())
    # a non-Hermitian operator is refused as a matrix is (src/pheig.jl:279)
    with pytest.raises(ValueError, match="Hermitian"):
        lra.pheigfact(_op(lra, real_fourier(30, 30, 6).astype(dt), hermitian=False), lra.LRAOptions(dt))


def test_operator_callback_error_is_reported(lra):
    """A product that fails makes the call fail with LRA_ECUDA, and the
    context stays usable."""
    import torch

    def bad(X):
        raise RuntimeError("no product today")
    L = lra.LinearOperator(50, 40, bad, bad)
    with pytest.raises(lra.LRAError) as e:
        lra.idfact(L)
    assert e.value.status == 6 and "matmat" in str(e.value)
    A = torch.randn(50, 40, dtype=torch.float64, device="cuda")
    assert lra.idfact(lra.LinearOperator.from_matrix(A)).k == 40
