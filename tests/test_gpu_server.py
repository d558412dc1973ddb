"""The serving loop (lra_server_*): continuous batching of idfact / psvdfact
requests over several worker streams under an HBM budget.  Every result must
be the same alone and in the mix: each request is compared with a standalone
call on a fresh context (bit-for-bit, stated tolerance 0: the kernels are
deterministic and the in-library generator restarts from the request's
seed).  Admission by budget and the latency statistics are checked too."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def decaying(m, n, rate, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = 10.0 ** (-np.arange(r) / rate)
    return np.asfortranarray(((U * s) @ V.T).astype(dtype))


def requests():
    out = []
    shapes = [(300, 200), (900, 700), (512, 1500), (1200, 400), (640, 640), (256, 1024), (1000, 1000), (700, 300)]
    for i, (m, n) in enumerate(shapes):
        dt = np.float64 if i % 3 else np.float32
        A = decaying(m, n, 15.0 + 5 * i, 100 + i, dt)
        kind = "psvdfact" if i % 2 else "idfact"
        prec = "mixed" if i % 4 in (1, 2) else "native"
        rtol = 1e-10 if dt == np.float64 else 1e-5
        out.append((kind, A, prec, rtol, 7 + i))
    return out


def same(a, b):
    if hasattr(a, "sk"):
        assert np.array_equal(a.sk, b.sk) and np.array_equal(a.rd, b.rd)
        assert np.array_equal(a.T, b.T)
    else:
        assert a.S.shape == b.S.shape
        assert np.array_equal(a.S, b.S) and np.array_equal(a.U, b.U) and np.array_equal(a.Vt, b.Vt)


def test_server_same_alone_and_in_mix(lra):
    reqs = requests()
    alone = []
    for kind, A, prec, rtol, seed in reqs:
        o = lra.LRAOptions(A.dtype, rtol=rtol, precision=prec, seed=seed)
        ctx = lra.Context()
        alone.append(lra.idfact(A, o, ctx=ctx) if kind == "idfact" else lra.psvdfact(A, o, ctx=ctx))
        ctx.close()
    srv = lra.Server(slots=4, hbm_budget_bytes=32 << 30)
    try:
        # twice over, so that every request meets different neighbours
        tickets = []
        for rep in range(2):
            for kind, A, prec, rtol, seed in (reqs if rep == 0 else reqs[::-1]):
                o = lra.LRAOptions(A.dtype, rtol=rtol, precision=prec, seed=seed)
                tickets.append(srv.submit(kind, A, o))
        results = [srv.result(t) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    n = len(reqs)
    for i, r in enumerate(results):
        j = i if i < n else n - 1 - (i - n)
        same(r, alone[j])
    assert {r.slot for r in results} > {0}  # more than one slot did work
    assert st["completed"] == 2 * n and st["submitted"] == 2 * n
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    assert st["matrices_per_s"] > 0


def test_server_budget_admission(lra):
    A = decaying(800, 600, 20.0, 3)
    o = lra.LRAOptions(rtol=1e-10, seed=5)
    # a budget that holds one request at a time: all still complete, in order
    one = 800 * 600 * 8 * 4 + 6 * 600 * 800 * 8 + (64 << 20) + 2 * 600 * 800 * 8 + 1
    srv = lra.Server(slots=3, hbm_budget_bytes=one)
    try:
        ts = [srv.submit("idfact", A, o) for _ in range(4)]
        rs = [srv.result(t) for t in ts]
        for r in rs[1:]:
            same(r, rs[0])
        # a request larger than the whole budget is refused at submission
        big = decaying(2000, 2000, 20.0, 4)
        with pytest.raises(lra.LRAError):
            srv.submit("idfact", big, o)
        assert srv.stats()["rejected"] == 1
    finally:
        srv.close()


def test_server_injected_streams(lra):
    A = decaying(600, 500, 20.0, 9)
    g = lra.lattice_gauss(11, 2_000_000)
    o = lra.LRAOptions(rtol=1e-10, precision="mixed")
    ref = lra.idfact(A, o, rand=lra.RandStream(gauss=g))
    srv = lra.Server(slots=2, hbm_budget_bytes=8 << 30)
    try:
        ts = [srv.submit("idfact", A, o, rand=lra.RandStream(gauss=g)) for _ in range(3)]
        for t in ts:
            same(srv.result(t), ref)
    finally:
        srv.close()
