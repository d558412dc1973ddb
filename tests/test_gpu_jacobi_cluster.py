"""The FP32 one-sided Jacobi of psvdfact's core SVD run inside one
thread-block cluster (every column pair in the registers of a warp, the
columns moved along the round-robin tournament through distributed shared
memory) against the block-pair kernel it replaces for k up to 448: the same
rank, singular values to the rank threshold, the reference test's criterion
(test/psvd.jl:29) and orthonormal factors, on the mixed path (FP32 sweeps,
then the Gram polish) and on the Float32 path (FP32 sweeps to convergence)."""
import numpy as np
import pytest

from test_gpu_mixed import decaying

pytestmark = pytest.mark.gpu


def _psvd(lra, A, opts, cluster):
    ctx = lra.Context(0)
    ctx.set_tuning("jacobi_cluster", 0, 0 if cluster else 1)
    F = lra.psvdfact(A, opts, ctx=ctx)
    launches = ctx.kernel_launches("jacobi_cluster_kernel")
    ctx.close()
    return F, launches


# core orders from about 70 to 450: the kernel's three register tiles (rows
# a lane 4, 8, 14 for orders up to 128, 256, 448) and both sides of each
# boundary, odd and even orders alike
@pytest.mark.parametrize("rate", [7.0, 12.3, 13.1, 20.0, 24.9, 25.9, 30.0, 41.0, 44.0])
def test_cluster_jacobi_mixed(lra, rate):
    m, n = 1400, 1000
    A = decaying(m, n, rate, 31)
    rtol = 1e-10
    o = lra.LRAOptions(rtol=rtol, precision="mixed", seed=4)
    F, used = _psvd(lra, A, o, True)
    G, unused = _psvd(lra, A, o, False)
    assert unused == 0
    if 64 <= F.k <= 400:  # the core SVD is of the ID's rank, a little above F.k
        assert used >= 1
    assert F.k == G.k
    s = np.linalg.svd(A, compute_uv=False)
    for H in (F, G):
        E = (np.asarray(H.U) * H.S) @ np.asarray(H.Vt)
        assert np.linalg.norm(A - E) < 100 * rtol * np.linalg.norm(A)
        assert np.abs(H.S - s[:H.k]).max() <= 10 * rtol * s[0]
        for Q in (np.asarray(H.U), np.asarray(H.Vt).T):
            assert np.abs(Q.T @ Q - np.eye(H.k)).max() < 1e-10


@pytest.mark.parametrize("rate", [15.0, 40.0])
def test_cluster_jacobi_float32(lra, rate):
    """Float32 psvdfact: the core SVD is the FP32 Jacobi run to convergence."""
    A = decaying(1200, 900, rate, 32).astype(np.float32)
    rtol = 1e-5
    o = lra.LRAOptions(np.float32, rtol=rtol, seed=5)
    F, used = _psvd(lra, A, o, True)
    G, _ = _psvd(lra, A, o, False)
    if 64 <= F.k <= 400:
        assert used >= 1
    assert abs(F.k - G.k) <= 1
    A64 = A.astype(np.float64)
    s = np.linalg.svd(A64, compute_uv=False)
    defect = []
    for H in (F, G):
        E = (np.asarray(H.U, dtype=np.float64) * H.S) @ np.asarray(H.Vt, dtype=np.float64)
        assert np.linalg.norm(A64 - E) < 100 * rtol * np.linalg.norm(A64)
        assert np.abs(H.S - s[:H.k]).max() <= 10 * rtol * s[0]
        defect.append(max(np.abs(Q.T @ Q - np.eye(H.k)).max()
                          for Q in (np.asarray(H.U, dtype=np.float64), np.asarray(H.Vt, dtype=np.float64).T)))
    # FP32 factors of a spectrum reaching rtol: orthonormal to a few 1e-4,
    # and the cluster kernel's no worse than the block kernel's
    assert max(defect) < 1e-3
    assert defect[0] <= 2 * defect[1] + 1e-5
