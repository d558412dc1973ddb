"""lra_geqp3_adap_noalloc: the pivoted QR for callers that cannot allocate
device memory while they factor (a serving loop whose memory was reserved up
front, a host whose device allocator belongs to another framework).  Called
through the C ABI and compared with the allocating entry point
lra_geqp3_adap, on two calls in a row so that the reused scratch array is
exercised, in both precisions and on a tall sketch whose reflector does not
fit shared memory; also the size limit and the rank-0 request.

This file is collected last on purpose: a run that stops at the first
failure has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, ctx, fn, Bd, opts):
    import torch
    m, n = Bd.shape
    dt = 1 if Bd.dtype == torch.float64 else 0
    jpvt = torch.zeros(n, dtype=torch.int64, device=Bd.device)
    tau = torch.zeros(min(m, n), dtype=Bd.dtype, device=Bd.device)
    k = C.c_int64(-1)
    st = getattr(lib, fn)(ctx.handle, dt, m, n, C.c_void_p(Bd.data_ptr()), m, C.c_void_p(jpvt.data_ptr()),
                          C.c_void_p(tau.data_ptr()), C.byref(opts), C.byref(k))
    return st, k.value, jpvt.cpu().numpy(), tau.cpu().numpy(), Bd.cpu().numpy()


def _sketch(rng, m, n, rate, dtype):
    B = rng.standard_normal((m, n)) @ np.diag(10.0 ** (-np.arange(n) / (rate * 10))) + \
        rng.standard_normal((m, 1)) @ rng.standard_normal((1, n))
    return B.astype(dtype)


# (m, n, decay rate): two wide sketches, then a tall one with m - 1 above the
# shared-memory reflector capacity (20480 Float64 / 40960 Float32 rows)
CASES = {np.float64: [(72, 900, 9.0), (136, 2000, 14.0), (24000, 300, 3.0)],
         np.float32: [(72, 900, 4.0), (136, 2000, 5.0), (44000, 200, 2.0)]}


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_noalloc_matches_allocating_entry_point(dtype):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import lowrankapprox as lra
    from lowrankapprox import _ffi
    lib = _ffi.load()
    ctx = lra.default_context()
    rng = np.random.default_rng(2024)
    rtol = 1e-10 if dtype == np.float64 else 1e-5
    tol = 1e-11 if dtype == np.float64 else 2e-5
    for call, (m, n, rate) in enumerate(CASES[dtype]):
        B = _sketch(rng, m, n, rate, dtype)
        opts = lra.LRAOptions(dtype, rtol=rtol).to_c()
        col = lambda X: torch.from_numpy(np.asfortranarray(X)).cuda().t().contiguous().t()
        ref = _run(lib, ctx, "lra_geqp3_adap", col(B), opts)
        got = _run(lib, ctx, "lra_geqp3_adap_noalloc", col(B), opts)
        assert ref[0] == 0 and got[0] == 0, (call, lib.lra_last_error(ctx.handle))
        assert got[1] == ref[1] > 0, call                 # rank
        assert np.array_equal(got[2], ref[2]), call       # pivots, bit-exact
        k = ref[1]
        R, Rref = np.triu(got[4][:k, :]), np.triu(ref[4][:k, :])
        assert np.abs(R - Rref).max() <= tol * np.abs(Rref).max(), call
        assert np.allclose(got[3][:k], ref[3][:k], rtol=tol, atol=10 * tol), call


def test_noalloc_rank_zero_gives_identity():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import lowrankapprox as lra
    from lowrankapprox import _ffi
    lib = _ffi.load()
    ctx = lra.default_context()
    B = torch.ones((8, 50), dtype=torch.float64, device="cuda").t().contiguous().t()
    opts = lra.LRAOptions(rank=0).to_c()
    ref = _run(lib, ctx, "lra_geqp3_adap", B.clone(), opts)
    got = _run(lib, ctx, "lra_geqp3_adap_noalloc", B.clone(), opts)
    assert ref[0] == 0 and got[0] == 0, lib.lra_last_error(ctx.handle)
    assert got[1] == ref[1] == 0
    assert np.array_equal(got[2], np.arange(1, 51)) and np.array_equal(ref[2], got[2])


def test_noalloc_rejects_too_many_columns():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import lowrankapprox as lra
    from lowrankapprox import _ffi
    lib = _ffi.load()
    ctx = lra.default_context()
    Bd = torch.zeros((2, 32769), dtype=torch.float64, device="cuda").t().contiguous().t()
    st, *_ = _run(lib, ctx, "lra_geqp3_adap_noalloc", Bd, lra.LRAOptions().to_c())
    assert st == _ffi.LRA_EINVAL
    assert b"32768" in lib.lra_last_error(ctx.handle)
