"""Failure detection without a GPU fault: every device-side wait of the
engine is bounded.  A cooperative kernel meets at a grid barrier that no
arrival can complete (its count starts at the grid size); with the limit
set to 1 ms both CTAs give up, the call returns LRA_ETIMEDOUT, and the
same context then factors a matrix with the oracle's result."""
import time

import numpy as np
import pytest

from test_gpu_core import assert_id_parity, both_rs
from test_oracle import real_fourier

pytestmark = pytest.mark.gpu


def test_grid_barrier_wait_runs_out_and_context_survives(lra, oracle):
    from lowrankapprox import _ffi
    ctx = lra.Context(0)
    try:
        ctx.set_wait_limit(1_000_000)            # 1 ms
        t0 = time.perf_counter()
        st = ctx.probe_wait()
        dt = time.perf_counter() - t0
        assert st == _ffi.LRA_ETIMEDOUT, _ffi.load().lra_last_error(ctx.handle)
        assert b"both CTAs returned" in _ffi.load().lra_last_error(ctx.handle)
        assert 1e-3 <= dt < 2.0
        # a longer limit waits longer: the barrier really waited
        ctx.set_wait_limit(50_000_000)           # 50 ms
        t0 = time.perf_counter()
        assert ctx.probe_wait() == _ffi.LRA_ETIMEDOUT
        assert time.perf_counter() - t0 >= 0.05
    finally:
        ctx.set_wait_limit(0)                    # back to the default
    # the context is still usable: an idfact on it matches the oracle
    A = real_fourier(128, 64, 9)
    ors, grs = both_rs(oracle, lra, 51)
    trace = []
    ref = oracle.idfact("n", A, oracle.Opts(rtol=1e-10), ors, trace=trace)
    V = lra.idfact(A, lra.LRAOptions(rtol=1e-10), rand=grs, ctx=ctx)
    assert_id_parity(trace, V.p, V.k, np.concatenate([ref["sk"], ref["rd"]]), ref["k"], 1e-10, np.float64)
    ctx.close()


def test_wait_limit_rejects_negative(lra):
    from lowrankapprox import _ffi
    ctx = lra.default_context()
    assert _ffi.load().lra_ctx_set_wait_limit(ctx.handle, -1) == _ffi.LRA_EINVAL
