"""LowRankApprox.jl's sketch-then-factor API on the GB300 engine (liblra).

The names, arguments and result types mirror the Julia package
(src/LowRankApprox.jl:27-73): ``LRAOptions``, ``idfact`` / ``id``,
``pqrfact`` / ``pqr``, ``psvdfact`` / ``psvdvals`` / ``psvd``,
``pheigfact`` / ``pheigvals`` / ``pheig``, ``curfact`` / ``cur``,
``sketch`` / ``sketchfact``, ``snorm`` / ``snormdiff``, ``matrixlib``.
Every call goes through the C ABI of liblra (include/lra.h) -- the same
entry points a Julia ``ccall`` shim binds -- and runs on the GPU.

Matrices are numpy arrays (host) or column-major torch CUDA tensors
(device); index outputs are 1-based like Julia's.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _ffi
from ._ffi import LRA_C32, LRA_C64, LRA_F32, LRA_F64

_NP_OF = {LRA_F32: np.float32, LRA_F64: np.float64, LRA_C32: np.complex64, LRA_C64: np.complex128}
_DT_OF = {np.dtype(v): k for k, v in _NP_OF.items()}


def _real_of(np_dtype):
    """The real type of an element type (Float32 for ComplexF32, ...)."""
    return np.float32 if np.dtype(np_dtype) in (np.float32, np.complex64) else np.float64

__all__ = [
    "LRAOptions", "RandStream", "Context", "IDPackedV", "PartialQRFactors", "PartialQR", "PartialSVD",
    "PartialHermitianEigen", "CURPackedU", "CURFactor", "CUR", "idfact", "id", "pqrfact", "pqr", "psvdfact", "psvdvals",
    "psvd", "pheigfact", "pheigvals", "pheig", "curfact", "cur", "sketch", "sketchfact", "prange", "snorm",
    "snormdiff", "geqp3_adap", "matrixlib", "LRAError", "ArgumentError", "DimensionMismatch",
    "LinearOperator", "LinOp", "HermLinOp", "lattice_gauss", "library_gauss", "library_sketch_stream", "default_context", "Server", "idfact_batched",
]


# ---------------------------------------------------------------------------
# errors (the Julia shim maps the same statuses to Julia exceptions)
# ---------------------------------------------------------------------------

class LRAError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class ArgumentError(LRAError, ValueError):
    pass


class DimensionMismatch(LRAError, ValueError):
    pass


def _raise(status: int, ctx) -> None:
    if status == _ffi.LRA_OK:
        return
    lib = _ffi.load()
    msg = (lib.lra_last_error(ctx.handle) if ctx is not None else b"").decode() or \
        lib.lra_status_string(status).decode()
    if status in (_ffi.LRA_EINVAL, _ffi.LRA_ENOTHERM, _ffi.LRA_ENONFINITE):
        raise ArgumentError(status, msg)
    if status == _ffi.LRA_EDIM:
        raise DimensionMismatch(status, msg)
    raise LRAError(status, msg)


# ---------------------------------------------------------------------------
# options (src/LowRankApprox.jl:77-148)
# ---------------------------------------------------------------------------

class LRAOptions:
    """Mirror of LRAOptions; ``*_samp`` take (a, b) for n -> a n + b."""

    _fields = ("atol", "maxdet_niter", "maxdet_tol", "nb", "pheig_orthtol", "pqrfact_retval", "rank",
               "rtol", "sketch", "sketch_randn_niter", "sketchfact_adap", "sketchfact_randn_samp",
               "sketchfact_srft_samp", "sketchfact_sub_samp", "snorm_niter", "verb", "precision", "seed",
               "check_finite")

    def __init__(self, T=np.float64, **kwargs):
        eps = float(np.finfo(np.dtype(T)).eps)
        self.atol = 0.0
        self.maxdet_niter = -1
        self.maxdet_tol = -1.0
        self.nb = 32
        self.pheig_orthtol = float(np.sqrt(eps))
        self.pqrfact_retval = "qr"
        self.rank = -1
        self.rtol = 5 * eps
        self.sketch = "randn"
        self.sketch_randn_niter = 0
        self.sketchfact_adap = True
        self.sketchfact_randn_samp = (1, 8)
        self.sketchfact_srft_samp = (1, 8)
        self.sketchfact_sub_samp = (4, 8)
        self.snorm_niter = 32
        self.verb = True
        self.precision = "native"
        self.seed = 0x4C5241
        self.check_finite = True
        for k, v in kwargs.items():
            self._set(k, v)

    def _set(self, k, v):
        if k == "sketch" and v == "subs":
            v = "sub"
        if k not in self._fields:
            raise ArgumentError(_ffi.LRA_EINVAL, f"unknown option {k}")
        setattr(self, k, v)

    def copy(self, **kwargs) -> "LRAOptions":
        o = LRAOptions.__new__(LRAOptions)
        o.__dict__.update(self.__dict__)
        for k, v in kwargs.items():
            o._set(k, v)
        return o

    def to_c(self) -> _ffi.lra_opts:
        c = _ffi.lra_opts()
        c.atol = float(self.atol)
        c.maxdet_niter = int(self.maxdet_niter)
        c.maxdet_tol = float(self.maxdet_tol)
        c.nb = int(self.nb)
        c.pheig_orthtol = float(self.pheig_orthtol)
        rv = str(self.pqrfact_retval).lower()
        c.pqrfact_retval = (_ffi.RET_Q if "q" in rv else 0) | (_ffi.RET_R if "r" in rv else 0) | \
            (_ffi.RET_T if "t" in rv else 0)
        if self.sketch not in _ffi.SKETCH:
            raise ArgumentError(_ffi.LRA_EINVAL, "sketch")
        c.sketch = _ffi.SKETCH[self.sketch]
        c.rank = int(self.rank)
        c.rtol = float(self.rtol)
        c.sketch_randn_niter = int(self.sketch_randn_niter)
        c.sketchfact_adap = 1 if self.sketchfact_adap else 0
        c.verb = 1 if self.verb else 0
        for name in ("sketchfact_randn_samp", "sketchfact_srft_samp", "sketchfact_sub_samp"):
            a, b = getattr(self, name)
            arr = getattr(c, name)
            arr[0], arr[1] = int(a), int(b)
        c.snorm_niter = int(self.snorm_niter)
        if self.precision not in _ffi.PREC:
            raise ArgumentError(_ffi.LRA_EINVAL, "precision")
        c.precision = _ffi.PREC[self.precision]
        c.check_finite = 1 if self.check_finite else 0
        c.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return c


def lattice_gauss(rng_or_seed, n: int) -> np.ndarray:
    """N(0,1) draws rounded to the 1/32 lattice, clipped to +-127/32: the
    sketch entries the mixed-precision path multiplies exactly."""
    rng = np.random.default_rng(rng_or_seed) if not isinstance(rng_or_seed, np.random.Generator) \
        else rng_or_seed
    return np.clip(np.rint(rng.standard_normal(n) * 32.0), -127, 127) / 32.0


def library_gauss(seed: int, n: int, counter: int = 0, ctx=None) -> np.ndarray:
    """The in-library generator's draws (lra_rand_gauss): n lattice
    Gaussians of the Philox stream of `seed` from `counter` on -- what a call
    with no injected stream multiplies as its Gaussian sketch."""
    ctx = ctx or default_context()
    out = np.empty(int(n), np.float64)
    _raise(_ffi.load().lra_rand_gauss(ctx.handle, int(seed) & 0xFFFFFFFFFFFFFFFF, int(counter), int(n),
                                      out.ctypes.data), ctx)
    return out


def library_sketch_stream(seed: int, M: int, orders, ctx=None) -> np.ndarray:
    """The Gaussian draws of a fresh-context call's adaptive steps, in order
    (step t: orders[t] * M values at counter c_t, c_(t+1) = c_t +
    (orders[t] * M + 1) // 2), as one injectable stream."""
    parts, c = [], 0
    for l in orders:
        parts.append(library_gauss(seed, l * M, c, ctx))
        c += (l * M + 1) // 2
    return np.concatenate(parts) if parts else np.zeros(0)


class RandStream:
    """Injected random numbers (lra_rand): a float64 Gaussian stream and an
    int64 index stream, host numpy arrays or CUDA tensors."""

    def __init__(self, gauss=None, ints=None):
        self._keep = []
        self.c = _ffi.lra_rand()
        if gauss is not None:
            p, n = self._ptr(gauss, np.float64)
            self.c.gauss, self.c.gauss_len = p, n
        if ints is not None:
            p, n = self._ptr(ints, np.int64)
            self.c.ints, self.c.ints_len = p, n

    def _ptr(self, a, dt):
        if _is_torch(a):
            import torch
            want = torch.float64 if dt == np.float64 else torch.int64
            if a.dtype != want or not a.is_contiguous():
                a = a.to(want).contiguous()
            self._keep.append(a)
            return a.data_ptr(), a.numel()
        a = np.ascontiguousarray(a, dtype=dt)
        self._keep.append(a)
        return a.ctypes.data, a.size


# ---------------------------------------------------------------------------
# context and matrix arguments
# ---------------------------------------------------------------------------

class Context:
    """An lra_ctx: one CUDA stream, a workspace arena, stage timers."""

    def __init__(self, device: int = 0):
        lib = _ffi.load()
        h = C.c_void_p()
        st = lib.lra_ctx_create(int(device), C.byref(h))
        if st != _ffi.LRA_OK:
            raise LRAError(st, f"lra_ctx_create: {lib.lra_status_string(st).decode()}")
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            _ffi.load().lra_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(_ffi.load().lra_ctx_launches(self.handle))

    def kernel_launches(self, name: str) -> int:
        """Launches of the kernel called `name` on this context so far
        (lra_ctx_kernel_launches)."""
        return int(_ffi.load().lra_ctx_kernel_launches(self.handle, name.encode()))

    def stage_ms(self):
        out = (C.c_double * 4)()
        _ffi.load().lra_ctx_stage_ms(self.handle, out)
        return {"sketch": out[0], "qr": out[1], "solve": out[2], "post": out[3]}

    def set_stream(self, stream_ptr: int):
        _raise(_ffi.load().lra_ctx_set_stream(self.handle, C.c_void_p(stream_ptr)), self)

    def tuning(self) -> str:
        """The autotuned shapes in force and the table they came from."""
        lib = _ffi.load()
        n = lib.lra_ctx_get_tuning(self.handle, None, 0)
        buf = C.create_string_buffer(max(int(n), 1))
        lib.lra_ctx_get_tuning(self.handle, buf, len(buf))
        return buf.value.decode()

    def set_tuning(self, key: str, index: int, value: int):
        """Override one tuning entry of this context (lra_ctx_set_tuning)."""
        _raise(_ffi.load().lra_ctx_set_tuning(self.handle, key.encode(), int(index), int(value)), self)

    def set_wait_limit(self, ns: int):
        """Limit of the device-side bounded waits on this device (0: 4 s)."""
        _raise(_ffi.load().lra_ctx_set_wait_limit(self.handle, int(ns)), self)

    def probe_wait(self) -> int:
        """The bounded-wait self-test (lra_ctx_probe_wait); returns its
        status, LRA_ETIMEDOUT when the barrier gave up as designed."""
        return int(_ffi.load().lra_ctx_probe_wait(self.handle))


_DEFAULT = None


def default_context() -> Context:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


class _DevArray:
    """A column-major device array (rows x cols, leading dimension ld) seen
    through the CUDA array interface, for a zero-copy torch view."""

    def __init__(self, ptr, rows, cols, ld, np_dtype):
        isz = np.dtype(np_dtype).itemsize
        self.__cuda_array_interface__ = {"shape": (rows, cols), "typestr": np.dtype(np_dtype).str,
                                         "data": (int(ptr), False), "strides": (isz, max(ld, 1) * isz),
                                         "version": 2}


class LinearOperator:
    """LinearOperator / HermitianLinearOperator (src/linop.jl:9-40): an m x n
    operator known only through its products.  ``mul(X)`` returns A X and
    ``mulc(Y)`` returns A' Y for CUDA tensors (X: n x k, Y: m x k); a
    Hermitian operator needs ``mul`` only.  The factorizations take it in
    place of a matrix (the lra_*_linop entry points): the library calls back
    into ``mul`` / ``mulc`` on its own stream, which is torch's current
    stream while they run.  Scalar multiples, sums, products and adjoints
    build new operators, as the reference's operator algebra does
    (src/linop.jl:96-153)."""

    def __init__(self, m: int, n: int, mul, mulc=None, T=np.float64, hermitian: bool = False):
        if hermitian and m != n:
            raise DimensionMismatch(_ffi.LRA_EDIM, "a Hermitian operator must be square")
        if mulc is None and not hermitian:
            raise ArgumentError(_ffi.LRA_EINVAL, "mulc is required unless the operator is Hermitian")
        self.m, self.n, self.hermitian = int(m), int(n), bool(hermitian)
        self.mul, self.mulc = mul, (mul if hermitian else mulc)
        self.np_dtype = np.dtype(T).type
        if self.np_dtype not in (np.float32, np.float64):
            raise ArgumentError(_ffi.LRA_EINVAL, "Float32 or Float64 operator expected")
        self._cb = _ffi.MATMAT(self._matmat)
        self.c = _ffi.lra_linop(self.m, self.n, LRA_F64 if self.np_dtype == np.float64 else LRA_F32,
                                1 if hermitian else 0, self._cb, None)

    @classmethod
    def from_matrix(cls, A, hermitian=None):
        """LinOp(A) (src/linop.jl:24-31) of a CUDA tensor: Hermitian when A
        equals A' unless told otherwise."""
        import torch
        if hermitian is None:
            hermitian = A.shape[0] == A.shape[1] and bool(torch.equal(A, A.T))
        T = np.float64 if A.dtype == torch.float64 else np.float32
        return cls(A.shape[0], A.shape[1], lambda X: A @ X, None if hermitian else (lambda Y: A.T @ Y), T,
                   hermitian)

    @property
    def shape(self):
        return (self.m, self.n)

    @property
    def H(self) -> "LinearOperator":
        """adjoint(A) (src/linop.jl:42-43)."""
        if self.hermitian:
            return self
        return LinearOperator(self.n, self.m, self.mulc, self.mul, self.np_dtype)

    def __matmul__(self, X):
        if isinstance(X, LinearOperator):
            if self.n != X.m:
                raise DimensionMismatch(_ffi.LRA_EDIM, "operator sizes")
            a, b = self, X
            return LinearOperator(a.m, b.n, lambda Z: a.mul(b.mul(Z)), lambda Z: b.mulc(a.mulc(Z)), a.np_dtype)
        return self.mul(X)

    def __mul__(self, c):
        if isinstance(c, LinearOperator):
            return self @ c
        c = float(c)
        return LinearOperator(self.m, self.n, lambda X: c * self.mul(X), lambda Y: c * self.mulc(Y),
                              self.np_dtype, self.hermitian)

    __rmul__ = __mul__

    def __truediv__(self, c):
        return self * (1.0 / float(c))

    def __add__(self, o: "LinearOperator"):
        if (self.m, self.n) != (o.m, o.n):
            raise DimensionMismatch(_ffi.LRA_EDIM, "operator sizes")
        return LinearOperator(self.m, self.n, lambda X: self.mul(X) + o.mul(X),
                              lambda Y: self.mulc(Y) + o.mulc(Y), self.np_dtype, self.hermitian and o.hermitian)

    def __neg__(self):
        return self * -1.0

    def __sub__(self, o):
        return self + (-o)

    def matrix(self):
        """Matrix(A) = A * I (src/linop.jl:54)."""
        import torch
        dt = torch.float64 if self.np_dtype == np.float64 else torch.float32
        return self.mul(torch.eye(self.n, dtype=dt, device="cuda"))

    def _matmat(self, user, trans, ncols, X, ldx, Y, ldy, stream):
        try:
            import torch
            tr = trans.decode() if isinstance(trans, bytes) else str(trans)
            rin, rout = (self.n, self.m) if tr == "n" else (self.m, self.n)
            Xt = torch.as_tensor(_DevArray(X, rin, ncols, ldx, self.np_dtype), device="cuda")
            Yt = torch.as_tensor(_DevArray(Y, rout, ncols, ldy, self.np_dtype), device="cuda")
            with torch.cuda.stream(torch.cuda.ExternalStream(int(stream or 0))):
                Yt.copy_(self.mul(Xt) if tr == "n" else self.mulc(Xt))
            return 0
        except Exception as e:  # reported as LRA_ECUDA by the library
            self.last_error = e
            return 1


def _lcall(lib, name, ctx, M, pre=(), post=()):
    """lra_<name>(ctx, dtype, *pre, m, n, A, lda, *post) for a matrix, or
    lra_<name>_linop(ctx, *pre, &op, *post) for a LinearOperator."""
    if M.lin is not None:
        return getattr(lib, name + "_linop")(ctx.handle, *pre, C.byref(M.lin.c), *post)
    return getattr(lib, name)(ctx.handle, M.dtype, *pre, M.m, M.n, C.c_void_p(M.ptr), M.ld, *post)


@dataclass
class _Mat:
    ptr: int
    m: int
    n: int
    ld: int
    dtype: int
    np_dtype: type
    keep: object
    lin: object = None


def _mat(A) -> _Mat:
    if isinstance(A, LinearOperator):
        return _Mat(0, A.m, A.n, max(A.m, 1), A.c.dtype, A.np_dtype, A, A)
    if _is_torch(A):
        import torch
        if A.dim() != 2:
            raise DimensionMismatch(_ffi.LRA_EDIM, "matrix expected")
        tmap = {torch.float32: LRA_F32, torch.float64: LRA_F64, torch.complex64: LRA_C32,
                torch.complex128: LRA_C64}
        if A.dtype not in tmap:
            raise ArgumentError(_ffi.LRA_EINVAL, "Float32, Float64, ComplexF32 or ComplexF64 matrix expected")
        if not A.is_cuda:
            return _mat(A.numpy())
        # the library works on its own stream: what torch queued to make A
        # must be done before the library reads it
        torch.cuda.current_stream(A.device).synchronize()
        m, n = A.shape
        if not (A.stride(0) == 1 and A.stride(1) >= max(1, m)):
            A = A.t().contiguous().t()
        dt = tmap[A.dtype]
        return _Mat(A.data_ptr(), m, n, max(A.stride(1), 1), dt, _NP_OF[dt], A)
    A = np.asarray(A)
    if A.ndim != 2:
        raise DimensionMismatch(_ffi.LRA_EDIM, "matrix expected")
    if A.dtype not in _DT_OF:
        A = A.astype(np.complex128 if np.iscomplexobj(A) else np.float64)
    A = np.asfortranarray(A)
    m, n = A.shape
    dt = _DT_OF[A.dtype]
    return _Mat(A.ctypes.data, m, n, max(m, 1), dt, A.dtype.type, A)


def _host(ptr, shape, dtype, order="F") -> np.ndarray:
    count = int(np.prod(shape)) if len(shape) else 1
    if count == 0 or not ptr:
        return np.zeros(shape, dtype=dtype, order=order)
    buf = (C.c_byte * (count * np.dtype(dtype).itemsize)).from_address(int(ptr) if not isinstance(ptr, int) else ptr)
    return np.array(np.frombuffer(buf, dtype=dtype, count=count).reshape(shape, order=order), copy=True)


class _Result:
    """Keeps a library result struct alive while numpy arrays view its memory
    (no host copy of the factors); the matching lra_*_free runs when the last
    view is gone."""

    def __init__(self, free, ptr):
        self._free, self._ptr = free, ptr

    def __del__(self):
        try:
            self._free(self._ptr)
        except Exception:  # pragma: no cover - interpreter shutdown
            pass


def _view(ptr, shape, dtype, owner, order="F") -> np.ndarray:
    """A numpy array on library result memory, kept alive by owner."""
    count = int(np.prod(shape)) if len(shape) else 1
    if count == 0 or not ptr:
        return np.zeros(shape, dtype=dtype, order=order)
    buf = (C.c_byte * (count * np.dtype(dtype).itemsize)).from_address(int(ptr) if not isinstance(ptr, int) else ptr)
    buf._owner = owner
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(shape, order=order)


def _iptr(p) -> int:
    return C.cast(p, C.c_void_p).value or 0


def _args(args, kwargs, default_trans="n"):
    """Julia-style (trans, A, opts) / (A, opts) positional forms."""
    args = list(args)
    trans = default_trans
    if args and isinstance(args[0], str):
        trans = args.pop(0)
    if not args:
        raise ArgumentError(_ffi.LRA_EINVAL, "matrix argument missing")
    A = args.pop(0)
    opts = args.pop(0) if args and isinstance(args[0], LRAOptions) else None
    ctx = kwargs.pop("ctx", None) or default_context()
    rand = kwargs.pop("rand", None)
    M = _mat(A)
    opts = (opts or LRAOptions(M.np_dtype)).copy(**kwargs) if (opts is None or kwargs) else opts
    if trans not in ("n", "c", "t"):
        raise ArgumentError(_ffi.LRA_EINVAL, "trans")
    return trans, M, opts, ctx, rand


def _rand(rand):
    return C.byref(rand.c) if rand is not None else None


# ---------------------------------------------------------------------------
# result types
# ---------------------------------------------------------------------------

class IDPackedV:
    """IDPackedV (src/id.jl:15-92): A[:, rd] ~= A[:, sk] * T."""

    def __init__(self, sk, rd, T, nsteps=0):
        self.sk, self.rd, self.T, self.nsteps = sk, rd, T, nsteps

    @property
    def k(self) -> int:
        return len(self.sk)

    @property
    def p(self) -> np.ndarray:
        return np.concatenate([self.sk, self.rd])

    def __getitem__(self, d):
        return {"k": self.k, "sk": self.sk, "rd": self.rd, "T": self.T, "p": self.p, "P": self.p}[d]

    def matrix(self) -> np.ndarray:
        """Matrix(V) = [I T] P' (k x n)."""
        n = self.k + len(self.rd)
        out = np.zeros((self.k, n), self.T.dtype)
        out[:, self.sk - 1] = np.eye(self.k, dtype=self.T.dtype)
        if len(self.rd):
            out[:, self.rd - 1] = self.T
        return out


class PartialQRFactors:
    """PartialQRFactors (src/pqr.jl:14-32)."""

    def __init__(self, Q, R, p, k, T):
        self.Q, self.R, self.p, self.k, self.T = Q, R, p, k, T

    def __getitem__(self, d):
        return {"Q": self.Q, "R": self.R, "p": self.p, "P": self.p, "k": self.k, "T": self.T}[d]


class PartialQR(PartialQRFactors):
    """PartialQR (src/pqr.jl:36-40): A[:, p] ~= Q R."""

    def matrix(self) -> np.ndarray:
        out = np.zeros((self.Q.shape[0], self.R.shape[1]), self.Q.dtype)
        out[:, self.p - 1] = self.Q @ self.R
        return out


class PartialSVD:
    """PartialSVD (src/psvd.jl:4-16): A ~= U diagm(S) Vt."""

    def __init__(self, U, S, Vt):
        self.U, self.S, self.Vt = U, S, Vt

    @property
    def k(self) -> int:
        return len(self.S)

    def __getitem__(self, d):
        return {"U": self.U, "S": self.S, "Vt": self.Vt, "V": None if self.Vt is None else self.Vt.conj().T,
                "k": self.k}[d]

    def matrix(self) -> np.ndarray:
        return (self.U * self.S) @ self.Vt


class PartialHermitianEigen:
    """PartialHermitianEigen (src/pheig.jl:4-7)."""

    def __init__(self, values, vectors):
        self.values, self.vectors = values, vectors

    @property
    def k(self) -> int:
        return len(self.values)

    def __getitem__(self, d):
        return {"values": self.values, "vectors": self.vectors, "k": self.k}[d]

    def matrix(self) -> np.ndarray:
        return (self.vectors * self.values) @ self.vectors.conj().T


class CURPackedU:
    """CURPackedU / HermitianCURPackedU (src/cur.jl:14-57)."""

    def __init__(self, rows, cols, kind=0):
        self.rows, self.cols, self.kind = rows, cols, kind

    def __getitem__(self, d):
        return {"rows": self.rows, "cols": self.cols, "k": len(self.cols)}[d]


# ---------------------------------------------------------------------------
# entry points
# ---------------------------------------------------------------------------

def idfact(*args, **kwargs) -> IDPackedV:
    """idfact([trans,] A[, opts]; kwargs) (src/id.jl:434-450)."""
    trans, M, opts, ctx, rand = _args(args, kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_id)()
    co = opts.to_c()
    st = _lcall(lib, "lra_idfact", ctx, M, (trans.encode(),), (C.byref(co), _rand(rand), C.byref(out)))
    _raise(st, ctx)
    r = out.contents
    own = _Result(lib.lra_id_free, out)
    k, n = r.k, r.n
    sk = _view(_iptr(r.sk), (k,), np.int64, own)
    rd = _view(_iptr(r.rd), (n - k,), np.int64, own)
    T = _view(r.T, (k, n - k), M.np_dtype, own)
    return IDPackedV(sk, rd, T, r.nsteps)


def idfact_batched(mats, opts: LRAOptions | None = None, rands=None, ctx: "Context | None" = None):
    """idfact of many independent matrices of one element type
    (lra_idfact_batched): their work overlaps on the device; each result is
    identical to an idfact call on that matrix."""
    ctx = ctx or default_context()
    Ms = [_mat(A) for A in mats]
    if not Ms:
        return []
    if len({M.dtype for M in Ms}) != 1:
        raise ArgumentError(_ffi.LRA_EINVAL, "idfact_batched needs one element type")
    opts = opts or LRAOptions(Ms[0].np_dtype)
    lib = _ffi.load()
    arr = (_ffi.lra_matdesc * len(Ms))(*[_ffi.lra_matdesc(M.m, M.n, M.ld, M.ptr) for M in Ms])
    outs = (C.POINTER(_ffi.lra_id) * len(Ms))()
    rarr = None
    if rands is not None:
        rarr = (_ffi.lra_rand * len(Ms))(*[r.c for r in rands])
    co = opts.to_c()
    st = lib.lra_idfact_batched(ctx.handle, Ms[0].dtype, len(Ms), arr, C.byref(co), rarr, outs)
    _raise(st, ctx)
    res = []
    for M, p in zip(Ms, outs):
        r = p.contents
        own = _Result(lib.lra_id_free, p)
        k, n = r.k, r.n
        res.append(IDPackedV(_view(_iptr(r.sk), (k,), np.int64, own), _view(_iptr(r.rd), (n - k,), np.int64, own),
                             _view(r.T, (k, n - k), M.np_dtype, own), r.nsteps))
    return res


def id(*args, **kwargs):
    V = idfact(*args, **kwargs)
    return V.sk, V.rd, V.T


def _pqr_out(lib, out, np_dtype, want_pqr):
    r = out.contents
    try:
        m, n, k = r.m, r.n, r.k
        p = _host(_iptr(r.p), (n,), np.int64)
        Q = _host(r.Q, (m, k), np_dtype) if r.retval & _ffi.RET_Q else None
        R = _host(r.R, (k, n), np_dtype) if r.retval & _ffi.RET_R else None
        T = _host(r.T, (k, n - k), np_dtype) if r.retval & _ffi.RET_T else None
        if want_pqr and Q is not None and R is not None and T is None:
            return PartialQR(Q, R, p, k, None)
        return PartialQRFactors(Q, R, p, k, T)
    finally:
        lib.lra_pqr_free(out)


def pqrfact(*args, **kwargs):
    """pqrfact([trans,] A[, opts]) (src/pqr.jl:290-307)."""
    trans, M, opts, ctx, rand = _args(args, kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_pqr)()
    co = opts.to_c()
    st = _lcall(lib, "lra_pqrfact", ctx, M, (trans.encode(),), (C.byref(co), _rand(rand), C.byref(out)))
    _raise(st, ctx)
    return _pqr_out(lib, out, M.np_dtype, True)


def pqr(*args, **kwargs):
    kwargs.setdefault("pqrfact_retval", "qr")
    F = pqrfact(*args, **kwargs)
    return F.Q, F.R, F.p


def sketchfact(*args, **kwargs):
    """sketchfact([side, trans,] A[, opts]) (src/sketch.jl:52-66)."""
    args = list(args)
    side = "left"
    if len(args) >= 2 and isinstance(args[0], str) and isinstance(args[1], str):
        side = args.pop(0)
    trans, M, opts, ctx, rand = _args(args, kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_pqr)()
    co = opts.to_c()
    st = _lcall(lib, "lra_sketchfact", ctx, M, (side[0].encode(), trans.encode()),
                (C.byref(co), _rand(rand), C.byref(out)))
    _raise(st, ctx)
    return _pqr_out(lib, out, M.np_dtype, True)


def prange(*args, **kwargs) -> np.ndarray:
    """prange([trans,] A[, opts]) (src/prange.jl:14-61): an orthonormal basis
    (m' x k) of the range of op(A); trans "b" takes the ranges of A and A'
    together (A square)."""
    args = list(args)
    trans = "n"
    if args and isinstance(args[0], str):
        trans = args.pop(0)
    if trans not in ("n", "c", "t", "b"):
        raise ArgumentError(_ffi.LRA_EINVAL, "trans")  # prange_chktrans, src/prange.jl:79-80
    A = args.pop(0)
    opts = args.pop(0) if args else None
    ctx = kwargs.pop("ctx", None) or default_context()
    rand = kwargs.pop("rand", None)
    M = _mat(A)
    opts = (opts or LRAOptions(M.np_dtype)).copy(**kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_pqr)()
    co = opts.to_c()
    st = _lcall(lib, "lra_prange", ctx, M, (trans.encode(),), (C.byref(co), _rand(rand), C.byref(out)))
    _raise(st, ctx)
    return _pqr_out(lib, out, M.np_dtype, False).Q


def sketch(*args, **kwargs):
    """sketch([side, trans,] A, order[, opts]) (src/sketch.jl:35-50).  With
    out= a column-major CUDA tensor of the sketch's shape and element type,
    the sketch is written there (device to device) and out is returned;
    otherwise a new host array."""
    args = list(args)
    side, trans = "left", "n"
    if len(args) >= 2 and isinstance(args[0], str) and isinstance(args[1], str):
        side, trans = args.pop(0), args.pop(0)
    A = args.pop(0)
    order = int(args.pop(0))
    opts = args.pop(0) if args else None
    ctx = kwargs.pop("ctx", None) or default_context()
    rand = kwargs.pop("rand", None)
    out = kwargs.pop("out", None)
    M = _mat(A)
    opts = (opts or LRAOptions(M.np_dtype)).copy(**kwargs)
    Mop = M.m if trans == "n" else M.n
    Nop = M.n if trans == "n" else M.m
    shape = (order, Nop) if side == "left" else (Mop, order)
    if out is not None:
        O = _mat(out)
        if O.keep is not out or (O.m, O.n) != shape or O.dtype != M.dtype:
            raise ArgumentError(_ffi.LRA_EINVAL, "out must be a column-major CUDA tensor of the sketch's shape and type")
        B, ptr, ld = out, O.ptr, O.ld
    else:
        B = np.zeros(shape, dtype=M.np_dtype, order="F")
        ptr, ld = B.ctypes.data, max(shape[0], 1)
    lib = _ffi.load()
    co = opts.to_c()
    st = lib.lra_sketch(ctx.handle, M.dtype, side[0].encode(), trans.encode(), M.m, M.n, C.c_void_p(M.ptr),
                        M.ld, order, C.byref(co), _rand(rand), C.c_void_p(ptr), ld)
    _raise(st, ctx)
    return B


def geqp3_adap(B, opts: LRAOptions | None = None, ctx: Context | None = None, **kwargs):
    """geqp3_adap! (src/pqr.jl:348-359) in place on a column-major CUDA
    tensor; returns (jpvt, tau, k) as CUDA tensors / int."""
    import torch
    ctx = ctx or default_context()
    M = _mat(B)
    if M.keep is not B:
        raise ArgumentError(_ffi.LRA_EINVAL, "B must be a column-major CUDA tensor")
    opts = (opts or LRAOptions(M.np_dtype)).copy(**kwargs)
    jpvt = torch.empty(max(M.n, 1), dtype=torch.int64, device=B.device)
    tau = torch.empty(max(min(M.m, M.n), 1), dtype=B.dtype, device=B.device)
    k = C.c_int64()
    co = opts.to_c()
    st = _ffi.load().lra_geqp3_adap(ctx.handle, M.dtype, M.m, M.n, C.c_void_p(M.ptr), M.ld,
                                    C.c_void_p(jpvt.data_ptr()), C.c_void_p(tau.data_ptr()), C.byref(co),
                                    C.byref(k))
    _raise(st, ctx)
    return jpvt[:M.n], tau[:min(M.m, M.n)], int(k.value)


def _psvd(A, opts, kwargs, vals_only):
    trans, M, opts, ctx, rand = _args((A,) + ((opts,) if opts is not None else ()), kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_psvd)()
    co = opts.to_c()
    st = _lcall(lib, "lra_psvdfact", ctx, M, (), (C.byref(co), _rand(rand), 1 if vals_only else 0, C.byref(out)))
    _raise(st, ctx)
    r = out.contents
    own = _Result(lib.lra_psvd_free, out)
    k = r.k
    S = _view(r.S, (k,), _real_of(M.np_dtype), own)
    if vals_only:
        return S
    U = _view(r.U, (M.m, k), M.np_dtype, own)
    Vt = _view(r.Vt, (k, M.n), M.np_dtype, own)
    return PartialSVD(U, S, Vt)


class Server:
    """Serving loop (lra_server_*): continuous batching of idfact / psvdfact
    requests over `slots` worker streams under an HBM budget.  No
    counterpart in the reference.  submit() returns a ticket; result()
    waits for it and returns an IDPackedV or PartialSVD."""

    def __init__(self, slots: int = 4, hbm_budget_bytes: int = 64 << 30, device: int = 0):
        lib = _ffi.load()
        h = C.c_void_p()
        st = lib.lra_server_create(int(device), int(slots), int(hbm_budget_bytes), C.byref(h))
        if st != _ffi.LRA_OK:
            raise LRAError(st, f"lra_server_create: {lib.lra_status_string(st).decode()}")
        self.handle = h
        self._keep = {}

    def submit(self, kind: str, A, opts: LRAOptions | None = None, rand: "RandStream | None" = None,
               trans: str = "n") -> int:
        M = _mat(A)
        opts = opts or LRAOptions(M.np_dtype)
        req = _ffi.lra_request()
        req.kind = {"idfact": _ffi.LRA_REQ_IDFACT, "psvdfact": _ffi.LRA_REQ_PSVDFACT}[kind]
        req.dtype = M.dtype
        req.trans = trans.encode()
        req.m, req.n, req.lda = M.m, M.n, M.ld
        req.A = M.ptr
        req.opts = opts.to_c()
        if rand is not None:
            req.rand = C.pointer(rand.c)
        t = C.c_uint64()
        st = _ffi.load().lra_server_submit(self.handle, C.byref(req), C.byref(t))
        if st != _ffi.LRA_OK:
            raise LRAError(st, f"lra_server_submit: {_ffi.load().lra_status_string(st).decode()}")
        # the input and the random streams must outlive the request
        self._keep[t.value] = (M, rand, req, kind)
        return t.value

    def result(self, ticket: int, wait_ms: int = -1):
        """The factorization of `ticket` (None if not done within wait_ms),
        with .queue_ms / .run_ms / .total_ms / .slot attached."""
        lib = _ffi.load()
        res = _ffi.lra_result()
        st = lib.lra_server_poll(self.handle, C.c_uint64(ticket), int(wait_ms), C.byref(res))
        if st == _ffi.LRA_EBUSY:
            return None
        if st != _ffi.LRA_OK:
            raise LRAError(st, "lra_server_poll: unknown ticket")
        M, rand, req, kind = self._keep.pop(ticket)
        own_id = _Result(lib.lra_id_free, res.id) if res.id else None
        own_sv = _Result(lib.lra_psvd_free, res.psvd) if res.psvd else None
        if res.status != _ffi.LRA_OK:
            raise LRAError(res.status, f"{kind} in the server: {res.error.decode(errors='replace')}")
        if kind == "idfact":
            r = res.id.contents
            k, n = r.k, r.n
            out = IDPackedV(_view(_iptr(r.sk), (k,), np.int64, own_id), _view(_iptr(r.rd), (n - k,), np.int64, own_id),
                            _view(r.T, (k, n - k), M.np_dtype, own_id), r.nsteps)
        else:
            r = res.psvd.contents
            k = r.k
            out = PartialSVD(_view(r.U, (M.m, k), M.np_dtype, own_sv), _view(r.S, (k,), M.np_dtype, own_sv),
                             _view(r.Vt, (k, M.n), M.np_dtype, own_sv))
        out.queue_ms, out.run_ms, out.total_ms, out.slot = res.queue_ms, res.run_ms, res.total_ms, res.slot
        return out

    def stats(self) -> dict:
        s = _ffi.lra_server_stats()
        _ffi.load().lra_server_get_stats(self.handle, C.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if getattr(self, "handle", None):
            _ffi.load().lra_server_destroy(self.handle)
            self.handle = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def psvdfact(A, opts: LRAOptions | None = None, **kwargs) -> PartialSVD:
    """psvdfact(A[, opts]) (src/psvd.jl:238-272)."""
    return _psvd(A, opts, kwargs, False)


def psvdvals(A, opts: LRAOptions | None = None, **kwargs) -> np.ndarray:
    """psvdvals(A[, opts]) (src/psvd.jl:274-290)."""
    return _psvd(A, opts, kwargs, True)


def psvd(A, opts=None, **kwargs):
    F = psvdfact(A, opts, **kwargs)
    return F.U, F.S, F.Vt.T


def _pheig(A, opts, kwargs, vals_only):
    trans, M, opts, ctx, rand = _args((A,) + ((opts,) if opts is not None else ()), kwargs)
    if M.m != M.n:
        raise DimensionMismatch(_ffi.LRA_EDIM, "matrix is not square")
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_pheig)()
    co = opts.to_c()
    if M.lin is not None:
        st = lib.lra_pheigfact_linop(ctx.handle, C.byref(M.lin.c), C.byref(co), _rand(rand), 1 if vals_only else 0,
                                     C.byref(out))
    else:
        st = lib.lra_pheigfact(ctx.handle, M.dtype, M.n, C.c_void_p(M.ptr), M.ld, C.byref(co), _rand(rand),
                               1 if vals_only else 0, C.byref(out))
    _raise(st, ctx)
    r = out.contents
    try:
        k = r.k
        w = _host(r.values, (k,), _real_of(M.np_dtype))
        if vals_only:
            return w
        return PartialHermitianEigen(w, _host(r.vectors, (M.n, k), M.np_dtype))
    finally:
        lib.lra_pheig_free(out)


def pheigfact(A, opts: LRAOptions | None = None, **kwargs) -> PartialHermitianEigen:
    """pheigfact(A[, opts]) (src/pheig.jl:276-296)."""
    return _pheig(A, opts, kwargs, False)


def pheigvals(A, opts: LRAOptions | None = None, **kwargs) -> np.ndarray:
    """pheigvals(A[, opts]) (src/pheig.jl:298-311)."""
    return _pheig(A, opts, kwargs, True)


def pheig(A, opts=None, **kwargs):
    F = pheigfact(A, opts, **kwargs)
    return F.values, F.vectors


def curfact(A, opts: LRAOptions | None = None, **kwargs) -> CURPackedU:
    """curfact(A[, opts]) (src/cur.jl:532-564)."""
    trans, M, opts, ctx, rand = _args((A,) + ((opts,) if opts is not None else ()), kwargs)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_cur)()
    co = opts.to_c()
    st = _lcall(lib, "lra_curfact", ctx, M, (), (C.byref(co), _rand(rand), C.byref(out)))
    _raise(st, ctx)
    r = out.contents
    try:
        rows = _host(_iptr(r.rows), (r.kr,), np.int64)
        cols = _host(_iptr(r.cols), (r.kc,), np.int64)
        return CURPackedU(rows, cols, r.kind)
    finally:
        lib.lra_cur_free(out)


class CURFactor:
    """CUR / HermitianCUR / SymmetricCUR (src/cur.jl:60-80): A ~= C U R with
    U the pseudo-inverse of A[rows, cols] as a PartialSVD."""

    def __init__(self, rows, cols, C, U, R):
        self.rows, self.cols, self.C, self.U, self.R = rows, cols, C, U, R

    def matrix(self) -> np.ndarray:
        return self.C @ ((self.U.U * self.U.S) @ self.U.Vt) @ self.R


def CUR(A, U: CURPackedU, ctx: "Context | None" = None) -> CURFactor:
    """CUR(A, U::CURPackedU) (src/cur.jl:85-115): C = A[:, cols],
    R = A[rows, :] (A[cols, :] for the Hermitian and symmetric forms) and the
    middle factor computed on the device."""
    rows = np.ascontiguousarray(np.asarray(U.cols if U.kind else U.rows, np.int64))
    cols = np.ascontiguousarray(np.asarray(U.cols, np.int64))
    if len(rows) != len(cols):
        raise DimensionMismatch(_ffi.LRA_EDIM, "rows and cols differ in length")
    ctx = ctx or default_context()
    M = _mat(A)
    k = len(cols)
    lib = _ffi.load()
    out = C.POINTER(_ffi.lra_psvd)()
    ip = C.POINTER(C.c_int64)
    st = lib.lra_cur_middle(ctx.handle, M.dtype, M.m, M.n, C.c_void_p(M.ptr), M.ld, k,
                            rows.ctypes.data_as(ip), cols.ctypes.data_as(ip), C.byref(out))
    _raise(st, ctx)
    own = _Result(lib.lra_psvd_free, out)
    r = out.contents
    W = PartialSVD(_view(r.U, (k, k), M.np_dtype, own), _view(r.S, (k,), _real_of(M.np_dtype), own),
                   _view(r.Vt, (k, k), M.np_dtype, own))
    if _is_torch(A):
        import torch
        ci = torch.as_tensor(cols - 1, device=A.device)
        ri = torch.as_tensor(rows - 1, device=A.device)
        Cm = np.asfortranarray(A.index_select(1, ci).cpu().numpy())
        Rm = np.asfortranarray(A.index_select(0, ri).cpu().numpy())
    else:
        Ah = np.asarray(A)
        Cm = np.asfortranarray(Ah[:, cols - 1])
        Rm = np.asfortranarray(Ah[rows - 1, :])
    return CURFactor(rows, cols, Cm, W, Rm)


def cur(A, opts=None, **kwargs):
    U = curfact(A, opts, **kwargs)
    return U.rows, U.cols


def dgemm(transa: str, transb: str, A, B, alpha: float = 1.0, beta: float = 0.0, C_=None,
          precision: str = "mixed", ctx: "Context | None" = None):
    """C = alpha op(A) op(B) + beta C on CUDA Float64 tensors, as the
    factorizations compute their GEMMs ("mixed": tensor-core split product;
    "native": FP64 CUDA cores).  No counterpart in the reference."""
    import torch
    ctx = ctx or default_context()
    MA, MB = _mat(A), _mat(B)
    if MA.dtype != LRA_F64 or MB.dtype != LRA_F64 or not (_is_torch(A) and A.is_cuda and _is_torch(B) and B.is_cuda):
        raise ArgumentError(_ffi.LRA_EINVAL, "dgemm takes CUDA Float64 tensors")
    m = MA.n if transa == "t" else MA.m
    k = MA.m if transa == "t" else MA.n
    n = MB.m if transb == "t" else MB.n
    if (MB.n if transb == "t" else MB.m) != k:
        raise DimensionMismatch(_ffi.LRA_EDIM, "inner dimensions differ")
    if C_ is None:
        C_ = torch.zeros((n, m), dtype=torch.float64, device=A.device).t()
        beta = 0.0
    MC = _mat(C_)
    if MC.keep is not C_:
        raise ArgumentError(_ffi.LRA_EINVAL, "C must be a column-major CUDA tensor")
    st = _ffi.load().lra_dgemm(ctx.handle, _ffi.PREC[precision], transa.encode(), transb.encode(), m, n, k,
                               float(alpha), C.c_void_p(MA.ptr), MA.ld, C.c_void_p(MB.ptr), MB.ld, float(beta),
                               C.c_void_p(MC.ptr), MC.ld)
    _raise(st, ctx)
    return C_


def snorm(A, opts: LRAOptions | None = None, hermitian=None, **kwargs) -> float:
    """snorm(A[, opts]) (src/snorm.jl:14-45)."""
    trans, M, opts, ctx, rand = _args((A,) + ((opts,) if opts is not None else ()), kwargs)
    out = C.c_double()
    co = opts.to_c()
    herm = -1 if hermitian is None else (1 if hermitian else 0)
    if M.lin is not None:
        st = _ffi.load().lra_snorm_linop(ctx.handle, C.byref(M.lin.c), C.byref(co), _rand(rand), C.byref(out))
    else:
        st = _ffi.load().lra_snorm(ctx.handle, M.dtype, M.m, M.n, C.c_void_p(M.ptr), M.ld, herm, C.byref(co),
                                   _rand(rand), C.byref(out))
    _raise(st, ctx)
    return out.value


def snormdiff(A, B, opts: LRAOptions | None = None, trans: str = "n", **kwargs) -> float:
    """snormdiff(A, B[, opts]) (src/snorm.jl:50-53); B may be a dense matrix,
    an IDPackedV (F = A[:, sk] [I T] P') or a PartialSVD (factored form)."""
    _, M, opts, ctx, rand = _args((A,) + ((opts,) if opts is not None else ()), kwargs)
    lib = _ffi.load()
    out = C.c_double()
    co = opts.to_c()
    if isinstance(B, IDPackedV):
        keep = [np.ascontiguousarray(B.sk, np.int64), np.ascontiguousarray(B.rd, np.int64),
                np.asfortranarray(B.T.astype(M.np_dtype))]
        cid = _ffi.lra_id(M.dtype, B.nsteps, B.k, B.k + len(B.rd),
                          keep[0].ctypes.data_as(C.POINTER(C.c_int64)),
                          keep[1].ctypes.data_as(C.POINTER(C.c_int64)), keep[2].ctypes.data)
        st = lib.lra_snormdiff_id(ctx.handle, M.dtype, trans.encode(), M.m, M.n, C.c_void_p(M.ptr), M.ld,
                                  C.byref(cid), C.byref(co), _rand(rand), C.byref(out))
    elif isinstance(B, PartialSVD):
        keep = [np.asfortranarray(B.U.astype(M.np_dtype)), np.ascontiguousarray(B.S.astype(_real_of(M.np_dtype))),
                np.asfortranarray(B.Vt.astype(M.np_dtype))]
        cps = _ffi.lra_psvd(M.dtype, 0, M.m, M.n, B.k, keep[0].ctypes.data, keep[1].ctypes.data,
                            keep[2].ctypes.data)
        st = lib.lra_snormdiff_psvd(ctx.handle, M.dtype, M.m, M.n, C.c_void_p(M.ptr), M.ld, C.byref(cps),
                                    C.byref(co), _rand(rand), C.byref(out))
    else:
        MB = _mat(B)
        if MB.dtype != M.dtype or MB.m != M.m or MB.n != M.n:
            raise DimensionMismatch(_ffi.LRA_EDIM, "snormdiff operands differ")
        st = lib.lra_snormdiff(ctx.handle, M.dtype, M.m, M.n, C.c_void_p(M.ptr), M.ld, C.c_void_p(MB.ptr),
                               MB.ld, C.byref(co), _rand(rand), C.byref(out))
    _raise(st, ctx)
    return out.value


def matrixlib(name: str, *args, dtype=np.float64) -> np.ndarray:
    """matrixlib (src/matrixlib.jl:4-48): :hilb, :cauchy, :fourier."""
    if name == "hilb":
        m = args[0]
        n = args[1] if len(args) > 1 else m
        i = np.arange(1, m + 1)[:, None]
        j = np.arange(1, n + 1)[None, :]
        return np.asfortranarray((1.0 / (i + j - 1)).astype(dtype))
    if name == "cauchy":
        x, y = np.asarray(args[0]), np.asarray(args[1])
        return np.asfortranarray((1.0 / (x[:, None] - y[None, :])).astype(dtype))
    if name == "fourier":
        if len(args) == 2 and np.isscalar(args[0]):
            x = np.arange(args[0])
            y = np.arange(args[1]) / args[1]
        elif len(args) == 1:
            x = np.arange(args[0])
            y = np.arange(args[0]) / args[0]
        else:
            x, y = np.asarray(args[0]), np.asarray(args[1])
        return np.asfortranarray(np.exp(-2j * np.pi * np.outer(x, y)))
    raise ArgumentError(_ffi.LRA_EINVAL, "name")


LinOp = LinearOperator


def HermLinOp(n: int, mul, T=np.float64) -> LinearOperator:
    """HermitianLinearOperator (src/linop.jl:17-21, 33-39)."""
    return LinearOperator(n, n, mul, None, T, True)
