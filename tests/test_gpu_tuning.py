"""The autotuned shapes (lra_ctx_set_tuning / lra_ctx_get_tuning): a context
reads the committed table when it is created; every tile N of the tensor-
core sketch gives the same bits (the exact integer sums do not depend on
the tiling); the QR's row threshold changes only rounding, never the pivot
order or the rank of a well-separated case; bad keys are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_context_reads_the_table(lra):
    import os
    ctx = lra.Context(0)
    txt = ctx.tuning()
    here = os.path.dirname(lra.__file__)
    if os.path.exists(os.path.join(here, "tuning_gb300.txt")):
        assert "tuning_gb300.txt" in txt.splitlines()[0]
    assert "qr_seq_len" in txt and "tc_tile_n f64 10" in txt
    from lowrankapprox import _ffi
    lib = _ffi.load()
    assert lib.lra_ctx_set_tuning(ctx.handle, b"tc_tile_n", 16 + 10, 48) == _ffi.LRA_EINVAL
    assert lib.lra_ctx_set_tuning(ctx.handle, b"no_such_key", 0, 1) == _ffi.LRA_EINVAL
    ctx.close()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("order", [40, 136, 520])
def test_tile_n_gives_the_same_bits(lra, dt, order):
    import torch
    rng = np.random.default_rng(order)
    A = np.asfortranarray(rng.standard_normal((3000, 700)).astype(dt))
    ctx = lra.Context(0)
    g = lra.lattice_gauss(9, order * 3000 + 8)
    o = lra.LRAOptions(dt, precision="mixed", rtol=1e-10 if dt == np.float64 else 1e-6)
    lb = int(np.ceil(np.log2(order)))
    outs = []
    for tn in (32, 64, 96):
        ctx.set_tuning("tc_tile_n", (16 if dt == np.float64 else 0) + lb, tn)
        outs.append(lra.sketch("left", "n", A, order, o, rand=lra.RandStream(gauss=g), ctx=ctx))
    for B in outs[1:]:
        assert np.array_equal(B, outs[0])
    R = g[:order * 3000].reshape((order, 3000), order="F") @ A.astype(np.float64)
    assert np.abs(outs[0] - R).max() <= (1e-12 if dt == np.float64 else 1e-5) * np.abs(R).max()
    ctx.close()


def test_qr_seq_len_changes_only_rounding(lra):
    from test_gpu_mixed import decaying
    A = decaying(900, 700, 12.0, 4)
    g = lra.lattice_gauss(10, 4_000_000)
    ctx = lra.Context(0)
    o = lra.LRAOptions(rtol=1e-10, precision="mixed")
    res = []
    for v in (32, 96, 160):
        ctx.set_tuning("qr_seq_len", 0, v)
        res.append(lra.idfact(A, o, rand=lra.RandStream(gauss=g), ctx=ctx))
    from test_oracle import reconstruction_gap
    for V in res[1:]:
        assert V.k == res[0].k and np.array_equal(V.sk, res[0].sk)
        # T = R11 \ R12 carries cond(R11) ~ 1 / rtol: compare what it reconstructs
        assert reconstruction_gap(A, V.sk, V.rd, V.T, res[0].rd, res[0].T) <= 1e-12
    ctx.close()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(3000, 700, 40), (20000, 300, 136), (9000, 1200, 264)])
def test_k_split_gives_the_same_bits(lra, dt, shape):
    """The tensor-core sketch split over K (a few column tiles, many rows):
    whole 512-long chunks per part and the parts' exact integer sums added,
    so the split gives the bits of the unsplit kernel."""
    m, n, order = shape
    rng = np.random.default_rng(m + n)
    A = np.asfortranarray(rng.standard_normal((m, n)).astype(dt))
    A[:, 5] *= 1e-30                       # a column far below the others
    g = lra.lattice_gauss(17, order * m + 8)
    o = lra.LRAOptions(dt, precision="mixed", rtol=1e-10 if dt == np.float64 else 1e-6)
    outs = []
    for split in (1, 0, 2):
        ctx = lra.Context(0)
        ctx.set_tuning("tc_split", 0, split)
        outs.append(lra.sketch("left", "n", A, order, o, rand=lra.RandStream(gauss=g), ctx=ctx))
        ctx.close()
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    R = g[:order * m].reshape((order, m), order="F") @ A.astype(np.float64)
    scale = np.abs(R).max(axis=0) + 1e-300
    assert (np.abs(outs[0] - R) / scale).max() <= (1e-12 if dt == np.float64 else 1e-5)


@pytest.mark.parametrize("jb", [4, 8, 16, 32])
def test_jacobi_block_sizes(lra, jb):
    """The FP32 block Jacobi of psvdfact's core SVD with every block size
    (the block pair in shared memory; 32-column blocks gather their
    rotations into a 64 x 64 matrix): the same rank and singular values to
    the rank threshold, and the reference test's criterion (test/psvd.jl:29)."""
    from test_gpu_mixed import decaying
    A = decaying(1500, 1100, 30.0, 21)
    rtol = 1e-10
    ctx = lra.Context(0)
    ctx.set_tuning("jacobi_jb", 0, jb)
    F = lra.psvdfact(A, lra.LRAOptions(rtol=rtol, precision="mixed", seed=2), ctx=ctx)
    ctx.close()
    E = (np.asarray(F.U) * F.S) @ np.asarray(F.Vt)
    assert np.linalg.norm(A - E) < 100 * rtol * np.linalg.norm(A)
    s = np.linalg.svd(A, compute_uv=False)
    assert np.abs(F.S - s[:F.k]).max() <= 10 * rtol * s[0]
    for Q in (np.asarray(F.U), np.asarray(F.Vt).T):
        assert np.abs(Q.T @ Q - np.eye(F.k)).max() < 1e-10
