"""The CPU oracle pinned before it is trusted: against the golden fixtures
made with the real LAPACK xLAQPS (the routine the reference ccalls,
src/lapack.jl:117-139), the README's published Hilbert ranks
(README.md:107,122), and the reference tests' reconstruction criteria
(test/id.jl:31-32, test/pqr.jl, test/psvd.jl:29-32, test/pheig.jl:26-29,
test/cur.jl:31, test/snorm.jl:16-25)."""
import numpy as np
import pytest


def assert_pqr_parity(p, R, p_ref, R_ref, k, tol, name=""):
    """Skeleton pivots p[:k] bit-exact; the columns after the rank are
    compared as a set, with R12 aligned by column index (their order is
    decided among pivots below the rank tolerance)."""
    assert np.array_equal(p[:k], p_ref[:k]), name
    assert sorted(p[k:]) == sorted(p_ref[k:]), name
    scale = max(np.abs(R_ref).max(), 1e-300)
    assert np.abs(R[:, :k] - R_ref[:, :k]).max() <= tol * scale, name
    if R.shape[1] > k:
        o, o_ref = np.argsort(p[k:]), np.argsort(p_ref[k:])
        assert np.abs(R[:, k:][:, o] - R_ref[:, k:][:, o_ref]).max() <= tol * scale, name


def _wide(B):
    """B in double precision (complex128 for complex types)."""
    return np.asarray(B, np.complex128 if np.iscomplexobj(B) else np.float64)


def residual_norms(B, piv, cols):
    """Norms of columns `cols` of B after projecting out B[:, piv] (double
    precision)."""
    B = _wide(B)
    X = B[:, np.asarray(cols) - 1]
    if len(piv):
        Q, _ = np.linalg.qr(B[:, np.asarray(piv) - 1])
        X = X - Q @ (Q.conj().T @ X)
    return np.linalg.norm(X, axis=0)


def _single(dt):
    return np.dtype(dt) in (np.float32, np.complex64)


def check_pivots(B, p, p_ref, k, dt, name=""):
    """p[:k] must equal p_ref[:k] up to the first step where the two choices
    are a near-tie: there, the exact residual norms of both candidates agree
    to the precision's tie tolerance, and the sequences may differ after.
    Returns the number of leading pivots that agree."""
    tie = 5e-4 if _single(dt) else 1e-9
    eps = float(np.finfo(dt).eps)
    floor = 1e3 * eps * float(np.linalg.norm(_wide(B), axis=0).max())
    for i in range(k):
        if p[i] == p_ref[i]:
            continue
        r = residual_norms(B, p[:i], [p[i], p_ref[i]])
        # a tie relative to the candidates, or both at the rounding floor
        assert abs(r[0] - r[1]) <= tie * r.max() + floor, (name, i, r)
        return i
    return k


def tie_tolerances(B, dt):
    tie = 5e-4 if _single(dt) else 1e-9
    eps = float(np.finfo(dt).eps)
    return tie, 1e3 * eps * float(np.linalg.norm(_wide(B), axis=0).max())


def check_rank(B, k, k_ref, p, p_ref, rtol, dt, atol=0.0, nb=32, name=""):
    """Ranks equal, or different only where geqp3_adap!'s stop test
    (|R_ii| <= ptol, src/pqr.jl:404-413) sits on a near-tie: among the
    pivots of the blocks around the two ranks, some exact residual norm
    equals ptol = max(atol, rtol * max column norm) to within the
    precision's tie tolerance (or lies at the rounding floor)."""
    if k == k_ref:
        return
    assert abs(k - k_ref) <= nb, (name, k, k_ref)
    tie, floor = tie_tolerances(B, dt)
    ptol = max(atol, rtol * float(np.linalg.norm(_wide(B), axis=0).max()))
    big = np.asarray(p if k > k_ref else p_ref)
    lo, hi = max(0, min(k, k_ref) - nb), min(len(big), max(k, k_ref) + 1)
    r = [residual_norms(B, big[:i], [big[i]])[0] for i in range(lo, hi)]
    assert any(abs(ri - ptol) <= tie * ptol + floor for ri in r), (name, k, k_ref, ptol, min(r), max(r))


def reconstruction_gap(A, sk, rd, T, rd_ref, T_ref):
    """||A[:, sk] (T - T_ref)||_F / ||A||_F with the columns of the two
    interpolation matrices aligned by their redundant column (the order of
    rd comes from pivots below the rank tolerance): how far apart the two
    put the reconstructed columns (same skeleton)."""
    C = np.asarray(A)[:, np.asarray(sk) - 1].astype(np.complex128 if np.iscomplexobj(A) else np.float64)
    o, o_ref = np.argsort(np.asarray(rd)), np.argsort(np.asarray(rd_ref))
    D = np.asarray(T)[:, o].astype(C.dtype) - np.asarray(T_ref)[:, o_ref].astype(C.dtype)
    return np.linalg.norm(C @ D) / np.linalg.norm(A)


def qr_cases(golden):
    z = golden["qr"]
    names = sorted({k.split("/")[1] for k in z.files})
    return z, names


def test_c_laqps_matches_lapack_goldens(oracle, golden):
    z, names = qr_cases(golden)
    assert len(names) >= 10
    for nm in names:
        B = np.asfortranarray(z[f"qr/{nm}/B"])
        opts = oracle.Opts(rtol=float(z[f"qr/{nm}/rtol"]), rank=int(z[f"qr/{nm}/rank"])).for_dtype(B.dtype)
        W = B.copy(order="F")
        p, tau, k = oracle.geqp3_adap(W, opts, backend="c")
        assert k == int(z[f"qr/{nm}/k"]), nm
        assert_pqr_parity(p, np.triu(W[:k, :]), z[f"qr/{nm}/p"], z[f"qr/{nm}/R"], k,
                          1e-12 if B.dtype == np.float64 else 2e-5, nm)


def test_block_loop_equals_c_loop(oracle, golden):
    z, names = qr_cases(golden)
    for nm in names[:6]:
        B = np.asfortranarray(z[f"qr/{nm}/B"])
        opts = oracle.Opts(rtol=float(z[f"qr/{nm}/rtol"]), rank=int(z[f"qr/{nm}/rank"])).for_dtype(B.dtype)
        W1, W2 = B.copy(order="F"), B.copy(order="F")
        p1, _, k1 = oracle.geqp3_adap(W1, opts, backend="oracle")
        p2, _, k2 = oracle.geqp3_adap(W2, opts, backend="c")
        assert k1 == k2 and np.array_equal(p1, p2)


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).lapack_available()")
def test_lapack_pin_live(oracle):
    rng = np.random.default_rng(5)
    B = np.asfortranarray(rng.standard_normal((50, 200)) @ np.diag(np.exp(-np.arange(200) / 4)))
    opts = oracle.Opts(rtol=1e-11).for_dtype(np.float64)
    W1, W2 = B.copy(order="F"), B.copy(order="F")
    p1, _, k1 = oracle.geqp3_adap(W1, opts, backend="lapack")
    p2, _, k2 = oracle.geqp3_adap(W2, opts, backend="c")
    assert k1 == k2 and np.array_equal(p1, p2)


def test_hilbert_readme_ranks(oracle, golden):
    h = golden["hilb"]
    A = oracle.hilb(1024)
    g = h["stream"].astype(np.float64) / 32.0
    for tag, rtol, want in (("1e-12", 1e-12, {22}), ("default", None, {26, 27})):
        V = oracle.idfact("n", A, oracle.Opts(rtol=rtol), oracle.RandStream(gauss=g))
        assert V["k"] in want                       # README.md:107,122
        assert V["k"] == int(h[f"{tag}/k"])
        assert np.array_equal(V["sk"], h[f"{tag}/sk"])
        # T = R11 \ R12 inherits cond(R11) (~1/rtol): compare it normwise
        # loosely and the reconstruction it gives tightly
        Tg = h[f"{tag}/T"]
        if tag == "1e-12":   # at 5 eps, cond(R11) ~ 1/eps leaves T undetermined
            assert np.linalg.norm(V["T"] - Tg) <= 1e-3 * np.linalg.norm(Tg)
        E = oracle.id_matrix("n", A, V)
        err = np.linalg.norm(A - E, 2) / np.linalg.norm(A, 2)
        assert err <= 2 * float(h[f"{tag}/relerr2"]) + 1e-15


def test_srft_restatement_matches_fft(oracle):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((96, 5))
    d = np.where(rng.standard_normal(96) > 0, 1.0, -1.0)
    for k in (7, 8, 40):
        idx = rng.integers(1, 97, k)
        a = oracle._srft_apply_columns(X, d, idx, k)
        b = oracle.srft_exact(X, d, idx, k)
        assert np.allclose(a, b, rtol=1e-10, atol=1e-10)


def real_fourier(m, n, seed=0):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(np.real(np.exp(-2j * np.pi * np.outer(rng.random(m), rng.random(n)))))


def streams(seed, n=200000):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n), rng


SKETCHES = ["none", "randn", "sub", "srft", "sprn"]


def rs_for(oracle, sketch, M, seed):
    g, rng = streams(seed)
    return oracle.RandStream(gauss=g, ints=rng.integers(1, 2**62, 200000, dtype=np.int64))


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_criteria_id(oracle, sketch, dt):
    A = real_fourier(128, 64).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    # the defaults, and the reference test's options (test/id.jl:8: maxdet_tol
    # = 0, one power iteration)
    for extra in ({}, {"maxdet_tol": 0.0, "sketch_randn_niter": 1}):
        opts = oracle.Opts(rtol=rtol, sketch=sketch, **extra)
        V = oracle.idfact("n", A, opts, rs_for(oracle, sketch, 128, 1))
        E = oracle.id_matrix("n", A, V)
        assert np.linalg.norm(A - E) < 100 * rtol * np.linalg.norm(A)     # test/id.jl:31


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("ref_opts", [False, True])
def test_reference_criteria_psvd_pheig_cur(oracle, sketch, ref_opts):
    A = real_fourier(128, 64)
    rtol = 5 * np.finfo(np.float64).eps
    # ref_opts: the reference tests' options (test/psvd.jl:10, test/pheig.jl:8)
    extra = {"maxdet_tol": 0.0, "sketch_randn_niter": 1} if ref_opts else {}
    opts = oracle.Opts(rtol=rtol, sketch=sketch, **extra)
    F = oracle.psvdfact(A, opts, rs_for(oracle, sketch, 128, 2))
    assert np.linalg.norm(A - (F["U"] * F["S"]) @ F["Vt"]) < 100 * rtol * np.linalg.norm(A)
    H = real_fourier(128, 128, 4)
    H = np.asfortranarray(H + H.T)
    E = oracle.pheigfact(H, opts, rs_for(oracle, sketch, 128, 3))
    assert np.linalg.norm(H - (E["vectors"] * E["values"]) @ E["vectors"].T) < 100 * rtol * np.linalg.norm(H)
    U = oracle.curfact(A, opts, rs_for(oracle, sketch, 128, 5))
    assert len(U["rows"]) == len(U["cols"]) > 0


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_criteria_prange(oracle, sketch, dt):
    # test/prange.jl:20-29 (maxdet off here: the build's prange refuses it)
    A = real_fourier(128, 128, 6).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    opts = oracle.Opts(rtol=rtol, sketch=sketch)
    nrm = np.linalg.norm(A)
    Q = oracle.prange("n", A, opts, rs_for(oracle, sketch, 128, 7))
    assert np.linalg.norm(A - Q @ (Q.T @ A)) < 100 * rtol * nrm
    Q = oracle.prange("c", A, opts, rs_for(oracle, sketch, 128, 8))
    assert np.linalg.norm(A - (A @ Q) @ Q.T) < 100 * rtol * nrm
    Q = oracle.prange("b", A, opts, rs_for(oracle, sketch, 128, 9))
    assert np.linalg.norm(A - Q @ (Q.T @ A @ Q) @ Q.T) < 100 * rtol * nrm


@pytest.mark.parametrize("sketch", SKETCHES)
def test_reference_criteria_cur_build(oracle, sketch):
    # test/cur.jl:10-31: ||A - C U R|| < 1000 rtol ||A|| for the general
    # and Hermitian forms, with the test's maxdet_tol = 0.  The pseudo-inverse
    # of A[rows, cols] carries rounding errors of order eps / rtol, so rtol
    # is 1e-8 here: at the test's 5 eps the bound sits at the noise floor
    M = real_fourier(128, 64, 10)
    Mh = M[:64, :64] + M[:64, :64].T
    rtol = 1e-8
    opts = oracle.Opts(rtol=rtol, sketch=sketch, maxdet_tol=0.0)
    for i, A in enumerate((M, np.asfortranarray(Mh))):
        U = oracle.curfact(A, opts, rs_for(oracle, sketch, 128, 11 + i))
        F = oracle.cur_build(A, U)
        V, s, Ut = F["U"]
        assert np.linalg.norm(A - F["C"] @ ((V * s) @ Ut) @ F["R"]) < 1000 * rtol * np.linalg.norm(A)


@pytest.mark.parametrize("sketch", SKETCHES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_criteria_pqr(oracle, sketch, dt):
    # test/pqr.jl:8-30, with its options (maxdet_tol = 0, one power iteration)
    A = real_fourier(128, 64, 12).astype(dt)
    rtol = 5 * np.finfo(dt).eps
    opts = oracle.Opts(rtol=rtol, sketch=sketch, maxdet_tol=0.0, sketch_randn_niter=1)
    nrm = np.linalg.norm(A)
    for i, trans in enumerate(("n", "c")):
        F = oracle.pqrfact(trans, A, opts, rs_for(oracle, sketch, 128, 13 + i))
        Aop = A if trans == "n" else A.T
        P = np.empty_like(F["p"])
        P[F["p"] - 1] = np.arange(len(F["p"]))
        E = F["Q"].astype(np.float64) @ F["R"].astype(np.float64)[:, P]
        assert np.linalg.norm(Aop - E) < 100 * rtol * nrm


@pytest.mark.parametrize("sketch", ["randn", "sub", "srft", "sprn"])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_sketch_shapes(oracle, sketch, dt):
    # test/sketch.jl:9-31: shapes of the four sides / transposes, niter = 1
    A = np.asfortranarray(np.random.default_rng(14).random((20, 10)).astype(dt))
    opts = oracle.Opts(sketch=sketch, sketch_randn_niter=1)
    rs = rs_for(oracle, sketch, 20, 15)
    assert oracle.sketch("left", "n", A, 5, opts, rs).shape == (5, 10)
    assert oracle.sketch("left", "c", A, 5, opts, rs).shape == (5, 20)
    assert oracle.sketch("right", "n", A, 5, opts, rs).shape == (20, 5)
    assert oracle.sketch("right", "c", A, 5, opts, rs).shape == (10, 5)


def test_snorm_criteria(oracle):
    rng = np.random.default_rng(7)
    A = rng.random((20, 10))
    rs = oracle.RandStream(gauss=rng.standard_normal(100))
    s = oracle.snorm_dense(A, oracle.Opts(), rs)
    assert abs(s - np.linalg.norm(A, 2)) <= 100 * np.finfo(float).eps * np.linalg.norm(A, 2) * 10


def test_maxdet_bounds_T(oracle):
    A = real_fourier(128, 64)
    opts = oracle.Opts(rtol=1e-10, maxdet_tol=0.0)
    V = oracle.idfact("n", A, opts, rs_for(oracle, "randn", 128, 9))
    assert np.abs(V["T"]).max() <= 1 + 1e-12


def test_srft_sampled_dft_matches_fft(oracle):
    """The sampled-DFT form the large-sketch checks use gives the full
    FFT's values (odd and even orders, a non-power-of-two length)."""
    rng = np.random.default_rng(4)
    for M in (96, 1000):
        X = rng.standard_normal((M, 7))
        d = np.where(rng.standard_normal(M) > 0, 1.0, -1.0)
        for k in (7, 40):
            idx = rng.integers(1, M + 1, k)
            a = oracle.srft_sampled_dft(X, d, idx, k, chunk=64)
            b = oracle.srft_exact(X, d, idx, k)
            assert np.allclose(a, b, rtol=1e-10, atol=1e-10 * np.abs(b).max())


def test_check_rank_accepts_only_threshold_ties():
    """check_rank: a rank off by one passes only when a pivot residual sits
    on the stop threshold; a genuine gap fails."""
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.standard_normal((60, 40)))
    s = 10.0 ** (-np.arange(40) / 4.0)
    B = (Q * s) @ np.linalg.qr(rng.standard_normal((40, 40)))[0]
    p = np.arange(1, 41)
    # the exact residual of pivot 10 after pivots 1..10 (0-based position 10)
    r10 = residual_norms(B, p[:10], [p[10]])[0]
    rtol = r10 / np.linalg.norm(B, axis=0).max()
    check_rank(B, 10, 11, p, p, rtol, np.float64)            # on the threshold: a tie
    with pytest.raises(AssertionError):
        check_rank(B, 10, 11, p, p, 1e3 * rtol, np.float64)  # far from it
