"""The Float64 GEMM of the mixed-precision path: tcgen05 products of six
exact BF16 byte slices per operand (lra_dgemm, precision "mixed"), checked
against the FP64 product at tile-edge shapes, all transpose combinations,
operands whose rows and columns span many binades, alpha / beta, and
non-finite entries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def colmajor(X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda().t()


def operands(rng, m, n, k, ta, tb, spread=20.0):
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-spread, spread, (m, 1)))
    B = rng.standard_normal((k, n)) * np.exp(rng.uniform(-spread, spread, (1, n)))
    A *= np.exp(rng.uniform(-2, 2, (1, k)))  # uneven entries inside each row / column
    Ad = A.T.copy() if ta == "t" else A
    Bd = B.T.copy() if tb == "t" else B
    return A, B, Ad, Bd


def bound(A, B, k):
    # representation, dropped slice products and FP32 rounding of the two
    # lowest diagonals, all within 13 k 2^(ea + eb - 48) <= 2^-42 k max|A_i.| max|B_.j|
    eps = np.finfo(float).eps
    return 2.0 ** -42 * k * np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] \
        + 4 * k * eps * (np.abs(A) @ np.abs(B))


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (130, 70, 65), (128, 64, 64), (300, 200, 1000), (1000, 9, 3000),
                                   (257, 129, 8200), (64, 700, 130)])
@pytest.mark.parametrize("ta,tb", [("n", "n"), ("t", "n"), ("n", "t"), ("t", "t")])
def test_dgemm_mixed(lra, m, n, k, ta, tb):
    rng = np.random.default_rng(m * 7 + n * 3 + k + ord(ta) + 2 * ord(tb))
    A, B, Ad, Bd = operands(rng, m, n, k, ta, tb)
    C = lra.dgemm(ta, tb, colmajor(Ad), colmajor(Bd), precision="mixed").cpu().numpy()
    R = A @ B
    assert np.all(np.abs(C - R) <= bound(A, B, k))
    # typical error far below the bound: a wrong slice weight shows up here
    rel = np.abs(C - R) / (np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * np.sqrt(k))
    assert np.median(rel) < 2.0 ** -46


def test_dgemm_alpha_beta(lra):
    rng = np.random.default_rng(11)
    A, B, _, _ = operands(rng, 333, 222, 777, "n", "n", spread=3.0)
    C0 = rng.standard_normal((333, 222))
    Ct = colmajor(C0)
    lra.dgemm("n", "n", colmajor(A), colmajor(B), alpha=-1.5, beta=0.25, C_=Ct, precision="mixed")
    R = -1.5 * (A @ B) + 0.25 * C0
    assert np.all(np.abs(Ct.cpu().numpy() - R) <= 1.5 * bound(A, B, 777) + 4 * np.finfo(float).eps * np.abs(R))


def test_dgemm_native_matches(lra):
    rng = np.random.default_rng(12)
    A, B, _, _ = operands(rng, 200, 150, 500, "n", "n", spread=5.0)
    Cm = lra.dgemm("n", "n", colmajor(A), colmajor(B), precision="mixed").cpu().numpy()
    Cn = lra.dgemm("n", "n", colmajor(A), colmajor(B), precision="native").cpu().numpy()
    R = A @ B
    assert np.all(np.abs(Cn - R) <= 4 * 500 * np.finfo(float).eps * (np.abs(A) @ np.abs(B)))
    assert np.all(np.abs(Cm - Cn) <= 2 * bound(A, B, 500))


def test_dgemm_nonfinite(lra):
    rng = np.random.default_rng(13)
    A, B, _, _ = operands(rng, 150, 90, 200, "n", "n", spread=2.0)
    A[3, 5] = np.nan
    B[7, 11] = np.inf
    C = lra.dgemm("n", "n", colmajor(A), colmajor(B), precision="mixed").cpu().numpy()
    assert np.all(np.isnan(C[3, :])) and np.all(np.isnan(C[:, 11]))
    mask = np.ones(C.shape, bool)
    mask[3, :] = False
    mask[:, 11] = False
    assert np.all(np.isfinite(C[mask]))
