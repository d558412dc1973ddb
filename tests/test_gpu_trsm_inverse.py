"""FP64 triangular solves on the tensor-core path by the explicit inverse
(tri_inv_upper_kernel: a CTA per column of R^{-1}, then one GEMM) against
the blocked substitution (tuning trsm_inv 1): the ID's T = R11 \\ R12
(src/id.jl:447) reconstructs the same columns, and psvdfact -- whose
skeleton Cholesky QR divides by R11 and by its Cholesky factor, and whose
V factor divides by R_v -- meets the reference test's criterion
(test/psvd.jl:29) either way."""
import numpy as np
import pytest

from test_gpu_mixed import decaying

pytestmark = pytest.mark.gpu


def _ctx(lra, inv):
    ctx = lra.Context(0)
    ctx.set_tuning("trsm_inv", 0, 0 if inv else 1)
    return ctx


@pytest.mark.parametrize("rate", [20.0, 45.0])
def test_id_solve_by_inverse(lra, rate):
    A = decaying(2500, 1800, rate, 41)
    o = lra.LRAOptions(rtol=1e-10, precision="mixed", seed=6)
    res, used = [], []
    for inv in (True, False):
        ctx = _ctx(lra, inv)
        res.append(lra.idfact(A, o, ctx=ctx))
        used.append(ctx.kernel_launches("tri_inv_upper_kernel"))
        ctx.close()
    V, W = res
    assert V.k == W.k and np.array_equal(V.sk, W.sk)
    assert used[1] == 0
    if V.k > 128:
        assert used[0] >= 1
    from test_oracle import reconstruction_gap
    assert reconstruction_gap(A, V.sk, V.rd, V.T, W.rd, W.T) <= 1e-12


@pytest.mark.parametrize("rate", [25.0, 41.0])
def test_psvd_by_inverse(lra, rate):
    A = decaying(3000, 2000, rate, 42)
    rtol = 1e-10
    o = lra.LRAOptions(rtol=rtol, precision="mixed", seed=7)
    s = np.linalg.svd(A, compute_uv=False)
    out = []
    for inv in (True, False):
        ctx = _ctx(lra, inv)
        F = lra.psvdfact(A, o, ctx=ctx)
        ctx.close()
        E = (np.asarray(F.U) * F.S) @ np.asarray(F.Vt)
        assert np.linalg.norm(A - E) < 100 * rtol * np.linalg.norm(A)
        assert np.abs(F.S - s[:F.k]).max() <= 10 * rtol * s[0]
        for Q in (np.asarray(F.U), np.asarray(F.Vt).T):
            assert np.abs(Q.T @ Q - np.eye(F.k)).max() < 1e-10
        out.append(F)
    assert out[0].k == out[1].k
