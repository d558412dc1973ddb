"""GPU parity of the sketch-then-factor path against the oracle, through the
C ABI (ctypes), on the same injected random streams.

Bar (floating point): rank equal; skeleton columns p[:k] bit-exact; the
rest of the permutation equal as a set; factors reconstruct A to within 2x
of the oracle's own error and within the reference tests' criteria
(test/id.jl:31, test/psvd.jl:29, test/pheig.jl:26, test/pqr.jl:29)."""
import numpy as np
import pytest

from test_oracle import assert_pqr_parity, check_pivots, check_rank, real_fourier, reconstruction_gap

pytestmark = pytest.mark.gpu


def dev(A):
    import torch
    return torch.from_numpy(np.asfortranarray(A)).cuda().t().contiguous().t()


def streams(seed, n=400000):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n), rng.integers(1, 2**62, n, dtype=np.int64)


def both_rs(oracle, lra, seed):
    g, q = streams(seed)
    return oracle.RandStream(gauss=g, ints=q), lra.RandStream(gauss=g, ints=q)


def relerr(A, E):
    return np.linalg.norm(A - E) / np.linalg.norm(A)


def assert_id_parity(trace, p, k, p_ref, k_ref, rtol, dt, name=""):
    """The bar on a pivoted QR's integer outputs against the oracle's, on
    the oracle's final sketch B: ranks equal unless the stop threshold is
    a near-tie (check_rank), pivots equal over all min(k, k_ref) positions
    up to the first demonstrated near-tie (check_pivots).  Returns the
    number of leading pivots that agree."""
    B = trace[-1]["B"]
    p, p_ref = np.asarray(p), np.asarray(p_ref)
    check_rank(B, k, k_ref, p, p_ref, rtol, dt, name=name)
    return check_pivots(B, p, p_ref, min(k, k_ref), dt, name)


def threshold_tie(values, k, k_ref, ptol, dt):
    """A rank decided on a list of values (singular values, eigenvalue
    magnitudes) may differ from the oracle's by one only when a value sits
    on the threshold ptol within the precision's tie tolerance."""
    if k == k_ref:
        return True
    eps = float(np.finfo(dt).eps)
    tie = 5e-4 if np.dtype(dt) == np.float32 else 1e-9
    v = np.abs(np.asarray(values, np.float64))
    return abs(k - k_ref) == 1 and bool(np.any(np.abs(v - ptol) <= tie * ptol + 1e3 * eps * v.max()))


# ---------------------------------------------------------------------------
# pivoted QR core vs the real-LAPACK goldens
# ---------------------------------------------------------------------------

def test_geqp3_goldens(lra, golden):
    import torch
    z = golden["qr"]
    names = sorted({k.split("/")[1] for k in z.files})
    for nm in names:
        B = np.asfortranarray(z[f"qr/{nm}/B"])
        Bd = dev(B)
        opts = lra.LRAOptions(B.dtype.type, rtol=float(z[f"qr/{nm}/rtol"]), rank=int(z[f"qr/{nm}/rank"]))
        jpvt, tau, k = lra.geqp3_adap(Bd, opts)
        assert k == int(z[f"qr/{nm}/k"]), nm
        W = Bd.cpu().numpy()
        p = jpvt.cpu().numpy()
        tol = 1e-11 if B.dtype == np.float64 else 5e-5
        same = check_pivots(B, p, z[f"qr/{nm}/p"], k, B.dtype, nm)
        if same == k:
            assert_pqr_parity(p, np.triu(W[:k, :]), z[f"qr/{nm}/p"], z[f"qr/{nm}/R"], k, tol, nm)
        assert torch.isfinite(tau).all()


def test_hilbert1024_id(lra, oracle, golden):
    h = golden["hilb"]
    A = oracle.hilb(1024)
    g = h["stream"].astype(np.float64) / 32.0
    for tag, rtol in (("1e-12", 1e-12), ("default", None)):
        kw = {} if rtol is None else {"rtol": rtol}
        for Ain in (A, dev(A)):
            V = lra.idfact(Ain, rand=lra.RandStream(gauss=g), **kw)
            assert V.k == int(h[f"{tag}/k"])
            B = g[:40 * 1024].reshape((40, 1024), order="F") @ A     # the (only) sketch
            check_pivots(B, V.sk, h[f"{tag}/sk"], V.k, np.float64, tag)
            E = lra.IDPackedV.matrix(V)
            err = np.linalg.norm(A - A[:, V.sk - 1] @ E, 2) / np.linalg.norm(A, 2)
            assert err <= 2 * float(h[f"{tag}/relerr2"]) + 1e-15


# ---------------------------------------------------------------------------
# every sketch and element type, reference-test matrices
# ---------------------------------------------------------------------------

SKETCHES = ["none", "randn", "sub", "srft", "sprn"]


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("trans", ["n", "c"])
def test_idfact_parity(lra, oracle, sketch, dt, trans):
    A = real_fourier(128, 64).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    ors, grs = both_rs(oracle, lra, 11)
    trace = []
    ref = oracle.idfact(trans, A, oracle.Opts(rtol=rtol, sketch=sketch), ors, trace=trace)
    V = lra.idfact(trans, A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=grs)
    Aop = A if trans == "n" else A.T
    E = Aop[:, V.sk - 1] @ V.matrix()
    assert relerr(Aop, E) < 100 * rtol            # test/id.jl:31-32
    agree = assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["k"], rtol, dt)
    if agree == V.k == ref["k"]:
        # same skeleton: the interpolation matrices put the columns within
        # the reference test's tolerance of each other
        assert reconstruction_gap(Aop, V.sk, V.rd, V.T, ref["rd"], ref["T"]) < 100 * rtol


@pytest.mark.parametrize("sketch", ["randn", "sub", "srft", "sprn"])
@pytest.mark.parametrize("side", ["left", "right"])
@pytest.mark.parametrize("trans", ["n", "c"])
def test_sketchfact_parity(lra, oracle, sketch, side, trans):
    """sketchfact on both sides (src/sketch.jl:52-63): rank, pivots up to the
    noise floor, and the factors of the sketch (Q orthonormal, Q R = B P)."""
    A = real_fourier(128, 64)
    rtol = 5 * np.finfo(np.float64).eps
    ors, grs = both_rs(oracle, lra, 17)
    trace = []
    ref = oracle.sketchfact(side, trans, A, oracle.Opts(rtol=rtol, sketch=sketch, pqrfact_retval="qr"), ors,
                            trace=trace)
    F = lra.sketchfact(side, trans, A, lra.LRAOptions(np.float64, rtol=rtol, sketch=sketch, pqrfact_retval="qr"),
                       rand=grs)
    k = F.k
    Aop = A if trans == "n" else A.T
    assert F.Q.shape[1] == k and (side == "left" or F.Q.shape[0] == Aop.shape[0])
    assert np.abs(F.Q.T @ F.Q - np.eye(k)).max() < 1e-12
    assert_id_parity(trace, F.p, F.k, ref["p"], ref["k"], rtol, np.float64, f"{sketch} {side} {trans}")
    if side == "right":
        # the basis spans op(A)'s range up to the tolerance
        E = Aop - F.Q @ (F.Q.T @ Aop)
        assert np.linalg.norm(E) <= 100 * rtol * np.linalg.norm(Aop) * max(1, k)


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("trans", ["n", "c", "b"])
def test_prange_parity(lra, oracle, sketch, dt, trans):
    """prange (src/prange.jl:14-77) against the oracle on the same streams:
    the reference test's criteria (test/prange.jl:20-29), an orthonormal
    basis, and the oracle's rank within one."""
    A = real_fourier(128, 128, 6).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    ors, grs = both_rs(oracle, lra, 23)
    Qr = oracle.prange(trans, A, oracle.Opts(rtol=rtol, sketch=sketch), ors)
    Q = lra.prange(trans, A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=grs)
    nrm = np.linalg.norm(A)
    Q64 = Q.astype(np.float64)
    if trans == "n":
        err = np.linalg.norm(A - Q64 @ (Q64.T @ A))
    elif trans == "c":
        err = np.linalg.norm(A - (A @ Q64) @ Q64.T)
    else:
        err = np.linalg.norm(A - Q64 @ (Q64.T @ A @ Q64) @ Q64.T)
    assert err < 100 * rtol * nrm
    assert np.abs(Q64.T @ Q64 - np.eye(Q.shape[1])).max() < 100 * rtol * max(1, Q.shape[1])
    assert abs(Q.shape[1] - Qr.shape[1]) <= 1


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_cur_build_parity(lra, oracle, sketch, dt):
    """CUR(A, curfact(A)) (src/cur.jl:85-115): the reference test's
    reconstruction bound (test/cur.jl:28-31) for the general, Hermitian and
    symmetric forms, and the middle factor's singular values against the
    oracle's SVD of the same A[rows, cols]."""
    M = real_fourier(128, 64, 10).astype(dt)
    Mh = np.asfortranarray(M[:64, :64] + M[:64, :64].T)
    # the pseudo-inverse of A[rows, cols] carries rounding errors of order
    # eps / rtol: the bound is checked at an rtol well above the noise floor
    rtol = 1e-8 if dt == np.float64 else 1e-4
    for i, A in enumerate((M, Mh)):
        ors, grs = both_rs(oracle, lra, 31 + i)
        U = lra.curfact(A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch, maxdet_tol=0.0), rand=grs)
        F = lra.CUR(A, U)
        A64 = A.astype(np.float64)
        E = F.C.astype(np.float64) @ ((F.U.U.astype(np.float64) * F.U.S) @ F.U.Vt.astype(np.float64)) @ F.R
        assert np.linalg.norm(A64 - E) < 1000 * rtol * np.linalg.norm(A64)
        ref = oracle.cur_build(A64, {"rows": U.cols if U.kind else U.rows, "cols": U.cols})
        assert np.allclose(np.sort(F.U.S.astype(np.float64)), np.sort(ref["U"][1]),
                           rtol=1e-5 if dt == np.float64 else 1e-2)


@pytest.mark.parametrize("sketch", ["randn", "sub", "srft", "sprn"])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_sketch_values(lra, oracle, sketch, dt):
    rng = np.random.default_rng(4)
    A = np.asfortranarray(rng.standard_normal((96, 40)).astype(dt))
    for side, trans in (("left", "n"), ("left", "c"), ("right", "n")):
        # injected streams restart at offset 0 on every C-ABI call
        ors, grs = both_rs(oracle, lra, 12)
        order = 17
        B = lra.sketch(side, trans, A, order, lra.LRAOptions(dt, sketch=sketch), rand=grs)
        R = oracle.sketch(side, trans, A, order, oracle.Opts(sketch=sketch), ors)
        tol = 1e-10 if dt == np.float64 else 2e-4
        assert B.shape == R.shape
        assert np.abs(B - R).max() <= tol * max(1.0, np.abs(R).max()), (sketch, side, trans)


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_psvd_parity(lra, oracle, sketch, dt):
    rtol = 5 * np.finfo(dt).eps
    for (m, n) in ((128, 64), (64, 128)):
        A = real_fourier(m, n, 3).astype(dt)
        ors, grs = both_rs(oracle, lra, 13)
        trace = []
        ref = oracle.psvdfact(A, oracle.Opts(rtol=rtol, sketch=sketch), ors, trace=trace)
        F = lra.psvdfact(A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=grs)
        assert relerr(A, F.matrix()) < 100 * rtol          # test/psvd.jl:29
        # the ID psvdfact starts from (src/psvd.jl:243,257) on the same stream
        V = lra.idfact("n" if m >= n else "c", A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch),
                       rand=both_rs(oracle, lra, 13)[1])
        assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["id_k"], rtol, dt)
        # psvdrank (src/psvd.jl:301-308): the truncation threshold rtol * s_1
        assert threshold_tie(ref["S"] if ref["k"] > F.k else F.S, F.k, ref["k"], rtol * ref["S"][0], dt)
        k = min(F.k, ref["k"])
        assert np.allclose(F.S[:k], ref["S"][:k], rtol=100 * rtol, atol=100 * rtol * ref["S"][0])
        Uo = F.U.T @ F.U
        assert np.abs(Uo - np.eye(F.k)).max() < 1e3 * rtol * max(1, F.k)
        s = lra.psvdvals(A, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=both_rs(oracle, lra, 13)[1])
        assert np.allclose(s, F.S, rtol=100 * rtol, atol=100 * rtol * F.S[0])


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_pheig_parity(lra, oracle, sketch, dt):
    rtol = 5 * np.finfo(dt).eps
    H = real_fourier(128, 128, 4)
    H = np.asfortranarray((H + H.T).astype(dt))
    ors, grs = both_rs(oracle, lra, 14)
    trace = []
    ref = oracle.pheigfact(H, oracle.Opts(rtol=rtol, sketch=sketch), ors, trace=trace)
    F = lra.pheigfact(H, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=grs)
    assert relerr(H, F.matrix()) < 100 * rtol                # test/pheig.jl:26
    # the ID pheigfact starts from (src/pheig.jl:281) on the same stream
    V = lra.idfact(H, lra.LRAOptions(dt, rtol=rtol, sketch=sketch), rand=both_rs(oracle, lra, 14)[1])
    assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["id_k"], rtol, dt)
    # pheigrank (src/pheig.jl:314-330): |w| against rtol * max |w|
    w = ref["values"] if ref["k"] > F.k else F.values
    assert threshold_tie(w, F.k, ref["k"], rtol * np.abs(ref["values"]).max(), dt)
    if F.k == ref["k"]:
        assert np.allclose(F.values, ref["values"], atol=100 * rtol * np.abs(ref["values"]).max())


@pytest.mark.parametrize("sketch", SKETCHES)
def test_pqrfact_parity(lra, oracle, sketch):
    rtol = 5 * np.finfo(np.float64).eps
    A = real_fourier(128, 64, 6)
    ors, grs = both_rs(oracle, lra, 15)
    trace = []
    ref = oracle.pqrfact("n", A, oracle.Opts(rtol=rtol, sketch=sketch), ors, trace=trace)
    F = lra.pqrfact(A, lra.LRAOptions(rtol=rtol, sketch=sketch), rand=grs)
    assert isinstance(F, lra.PartialQR)
    assert relerr(A, F.matrix()) < 100 * rtol                # test/pqr.jl:29
    assert_id_parity(trace, F.p, F.k, ref["p"], ref["k"], rtol, np.float64, sketch)
    assert np.abs(F.Q.T @ F.Q - np.eye(F.k)).max() < 1e-12


@pytest.mark.parametrize("sketch", SKETCHES)
def test_curfact_parity(lra, oracle, sketch):
    rtol = 5 * np.finfo(np.float64).eps
    M = real_fourier(128, 64, 7)
    Mh = M[:64, :64] + M[:64, :64].T
    for A in (M, M.T.copy(order="F"), np.asfortranarray(Mh)):
        ors, grs = both_rs(oracle, lra, 16)
        ref = oracle.curfact(A, oracle.Opts(rtol=rtol, sketch=sketch), ors)
        U = lra.curfact(A, lra.LRAOptions(rtol=rtol, sketch=sketch), rand=grs)
        assert U.kind == ref["kind"]
        assert abs(len(U.cols) - len(ref["cols"])) <= 1
        # CUR(A, U) (src/cur.jl:85-93): C * inv(C[rows, :]) * R through an SVD
        def cur_err(rows, cols):
            C, R = A[:, cols - 1], A[rows - 1, :]
            u, s, vt = np.linalg.svd(C[rows - 1, :])
            return relerr(A, C @ ((vt.T / s) @ u.T) @ R)
        e_gpu = cur_err(U.rows, U.cols)
        e_ref = cur_err(ref["rows"], ref["cols"])
        assert e_gpu <= max(2 * e_ref, 1000 * rtol)         # test/cur.jl:22-31


def test_maxdet(lra, oracle):
    A = real_fourier(128, 64, 8)
    ors, grs = both_rs(oracle, lra, 17)
    ref = oracle.idfact("n", A, oracle.Opts(rtol=1e-10, maxdet_tol=0.0), ors)
    V = lra.idfact(A, lra.LRAOptions(rtol=1e-10, maxdet_tol=0.0), rand=grs)
    assert np.abs(V.T).max() <= 1 + 1e-9
    assert V.k == ref["k"]
    assert sorted(V.sk) == sorted(ref["sk"])


def test_power_iterations(lra, oracle):
    A = real_fourier(128, 64, 9)
    ors, grs = both_rs(oracle, lra, 18)
    opts = dict(rtol=1e-10, sketch_randn_niter=1)
    ref = oracle.idfact("n", A, oracle.Opts(**opts), ors)
    V = lra.idfact(A, lra.LRAOptions(**opts), rand=grs)
    assert abs(V.k - ref["k"]) <= 1
    E = A[:, V.sk - 1] @ V.matrix()
    assert relerr(A, E) < 1e-8


# ---------------------------------------------------------------------------
# spectral norms
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_snorm(lra, dt):
    rng = np.random.default_rng(8)
    rtol = 100 * np.finfo(dt).eps
    A = rng.random((20, 10)).astype(dt)
    g = rng.standard_normal(1000)
    nrm = np.linalg.norm(A.astype(np.float64), 2)
    assert abs(lra.snorm(A, rand=lra.RandStream(gauss=g)) - nrm) <= rtol * nrm * 10   # test/snorm.jl:16
    H = rng.random((10, 10)).astype(dt)
    H = H + H.T
    nh = np.linalg.norm(H.astype(np.float64), 2)
    assert abs(lra.snorm(H, rand=lra.RandStream(gauss=g)) - nh) <= rtol * nh * 10
    B = rng.random((20, 10)).astype(dt)
    nd = np.linalg.norm((A - B).astype(np.float64), 2)
    d = lra.snormdiff(A, B, rand=lra.RandStream(gauss=g))
    # snorm stops after snorm_niter = 32 power steps; the oracle runs the same
    from oracle import oracle as O
    dref = O.snormdiff_dense(A, B, O.Opts(), O.RandStream(gauss=g))
    assert abs(d - dref) <= 1e-5 * nd
    assert abs(d - nd) <= 1e-4 * nd


def test_snormdiff_factored(lra):
    rng = np.random.default_rng(9)
    A = real_fourier(200, 90, 2)
    F = lra.psvdfact(A, rtol=1e-8)
    g = rng.standard_normal(1000)
    d1 = lra.snormdiff(A, F, rand=lra.RandStream(gauss=g))
    assert abs(d1 - np.linalg.norm(A - F.matrix(), 2)) <= 1e-3 * max(d1, 1e-300) + 1e-14
    V = lra.idfact(A, rtol=1e-8)
    d2 = lra.snormdiff(A, V, rand=lra.RandStream(gauss=g))
    E = A[:, V.sk - 1] @ V.matrix()
    assert abs(d2 - np.linalg.norm(A - E, 2)) <= 1e-3 * max(d2, 1e-300) + 1e-14


# ---------------------------------------------------------------------------
# edge cases and errors
# ---------------------------------------------------------------------------

def test_edge_shapes(lra, oracle):
    rng = np.random.default_rng(1)
    # n < nb, order > m, rank 0, full rank, single column / row
    for (m, n) in ((5, 3), (3, 5), (40, 7), (1, 9), (9, 1), (33, 33)):
        A = np.asfortranarray(rng.standard_normal((m, n)))
        ors, grs = both_rs(oracle, lra, 19)
        V = lra.idfact(A, rand=grs)
        ref = oracle.idfact("n", A, oracle.Opts(), ors)
        assert V.k == ref["k"] == min(m, n)
        assert np.array_equal(V.sk, ref["sk"])
    A = np.asfortranarray(rng.standard_normal((30, 20)))
    V = lra.idfact(A, rank=0, sketchfact_adap=False)
    assert V.k == 0 and len(V.rd) == 20
    V = lra.idfact(A, rank=5)
    assert V.k == 5
    Z = np.zeros((0, 4))
    V = lra.idfact(Z)
    assert V.k == 0
    Zc = np.zeros((12, 10))
    V = lra.idfact(Zc)
    assert V.k == 0


def test_device_and_host_inputs_agree(lra):
    rng = np.random.default_rng(2)
    A = np.asfortranarray(rng.standard_normal((300, 200)) @ np.diag(0.7 ** np.arange(200)))
    g, q = streams(21)
    V1 = lra.idfact(A, rtol=1e-10, rand=lra.RandStream(gauss=g))
    import torch
    V2 = lra.idfact(dev(A), rtol=1e-10, rand=lra.RandStream(gauss=torch.from_numpy(g).cuda()))
    assert V1.k == V2.k and np.array_equal(V1.sk, V2.sk)
    assert np.array_equal(V1.T, V2.T)  # same kernels, same data: bit-identical


def test_errors(lra):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((20, 20))
    with pytest.raises(ValueError, match="Hermitian"):
        lra.pheigfact(A)
    B = A.copy()
    B[3, 4] = np.nan
    with pytest.raises(ValueError):
        lra.idfact(B)
    with pytest.raises(lra.LRAError) as e:
        lra.idfact(A, rand=lra.RandStream(gauss=np.zeros(10)))
    assert e.value.status == 7
    with pytest.raises(ValueError):
        lra.idfact(A, nb=0)
    with pytest.raises(ValueError):
        lra.idfact(A, rtol=-1.0)
    # the context stays usable after errors
    assert lra.idfact(A).k == 20


def test_batched_ragged(lra, oracle):
    import ctypes as C
    from lowrankapprox import _ffi
    rng = np.random.default_rng(4)
    mats, keep = [], []
    sizes = [(50, 30), (16, 70), (128, 128), (7, 3)]
    for (m, n) in sizes:
        A = np.asfortranarray(rng.standard_normal((m, n)) @ np.diag(0.5 ** np.arange(n)))
        keep.append(A)
        mats.append(_ffi.lra_matdesc(m, n, m, A.ctypes.data))
    arr = (_ffi.lra_matdesc * len(mats))(*mats)
    outs = (C.POINTER(_ffi.lra_id) * len(mats))()
    o = lra.LRAOptions(rtol=1e-9).to_c()
    lib = _ffi.load()
    ctx = lra.default_context()
    assert lib.lra_idfact_batched(ctx.handle, 1, len(mats), arr, C.byref(o), None, outs) == 0
    for i, A in enumerate(keep):
        r = outs[i].contents
        assert 0 < r.k <= min(A.shape)
        lib.lra_id_free(outs[i])
