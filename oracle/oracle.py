"""CPU oracle for LowRankApprox.jl's sketch-then-factor path.

TEST INFRASTRUCTURE ONLY.  This module is the checker the CUDA library is
compared against; only tests/, the smoke check and bench.py's CPU-baseline
leg import it.  The product (liblra) never links, calls or falls back to it.

It restates, function by function, the reference's Julia code for real
element types (Float32 / Float64):

* the pivoted-QR core ``geqp3_adap!`` / ``pqrback_postproc`` / ``maxdet_*``
  (src/pqr.jl:343-501) on top of the C restatement of LAPACK xLAQPS in
  ``lra_oracle.c`` -- or, for pinning, on top of the real LAPACK xLAQPS
  exported by numpy's bundled OpenBLAS (the same routine the reference
  ``ccall``s, src/lapack.jl:117-139);
* the sketch operators and adaptive drivers of src/sketch.jl (Gaussian,
  subset, SRFT, sparse Gaussian; power iterations);
* ``idfact`` (src/id.jl:434-450), ``pqrfact`` (src/pqr.jl:290-307),
  ``psvdfact`` / ``psvdvals`` (src/psvd.jl:238-308), ``pheigfact`` /
  ``pheigvals`` (src/pheig.jl:276-364), ``curfact`` (src/cur.jl:532-564),
  ``snorm`` / ``snormdiff`` (src/snorm.jl:14-53);
* ``matrixlib`` (src/matrixlib.jl:4-48).

Random numbers are not drawn here: like the library, every sketch consumes
an injected stream (``RandStream``) in the documented order, so that the
oracle and the GPU see the same sketch.
"""
from __future__ import annotations

import ctypes
import glob
import os
from dataclasses import dataclass, field, replace

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LAPACK = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


def lib_path() -> str:
    return os.path.join(_HERE, "liblra_oracle.so")


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, a few seconds)."""
    out = lib_path()
    src = os.path.join(_HERE, "lra_oracle.c")
    hdr = os.path.join(_HERE, "lra_oracle_impl.h")
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return out
    import subprocess
    tmp = out + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)
    return out


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        for s in ("d", "s"):
            f = getattr(_LIB, f"ora_{s}laqps")
            f.argtypes = [_i64, _i64, _i64, _i64, _p, _p, _i64, _p, _p, _p, _p, _p, _p, _i64]
            f.restype = None
            g = getattr(_LIB, f"ora_{s}geqp3_adap")
            g.argtypes = [_i64, _i64, _p, _i64, _p, _p, ctypes.c_double, ctypes.c_double,
                          _i64, _i64, _p]
            g.restype = ctypes.c_int
            t = getattr(_LIB, f"ora_{s}maxdet_t")
            t.argtypes = [_i64, _i64, _p, _i64, _p, _i64]
            t.restype = ctypes.c_int
            r = getattr(_LIB, f"ora_{s}nrm2")
            r.argtypes = [_i64, _p, _i64]
            r.restype = ctypes.c_double if s == "d" else ctypes.c_float
    return _LIB


def lapack_available() -> bool:
    return _lapack() is not None


def _lapack():
    """numpy's bundled OpenBLAS (ILP64): the real LAPACK xLAQPS, for pinning."""
    global _LAPACK
    if _LAPACK is None:
        import numpy as _np
        root = os.path.dirname(os.path.dirname(_np.__file__))
        cands = glob.glob(os.path.join(root, "numpy.libs", "libscipy_openblas64_*.so"))
        _LAPACK = False
        for c in cands:
            try:
                lib = ctypes.CDLL(c)
                for s in ("d", "s", "z", "c"):
                    f = getattr(lib, f"scipy_{s}laqps_64_")
                    f.argtypes = [_p] * 14
                    f.restype = None
                _LAPACK = lib
                break
            except (OSError, AttributeError):
                continue
    return _LAPACK or None


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _sfx(dtype) -> str:
    return {np.dtype(np.float64): "d", np.dtype(np.float32): "s", np.dtype(np.complex128): "z",
            np.dtype(np.complex64): "c"}[np.dtype(dtype)]


def _H(X):
    """X' in the reference: the conjugate transpose."""
    return X.conj().T if np.iscomplexobj(X) else X.T


def _real(dtype):
    return np.float32 if np.dtype(dtype) in (np.float32, np.complex64) else np.float64


def crandn(rs: "RandStream", n: int, dtype) -> np.ndarray:
    """crandn(T, n) (src/util.jl:4-11) from the stream: real types take n
    values, complex types n pairs (re, im) of the reinterpreted real draw."""
    if np.iscomplexobj(np.zeros(0, dtype)):
        g = rs.take_gauss(2 * n)
        return (g[0::2] + 1j * g[1::2]).astype(dtype)
    return rs.take_gauss(n).astype(dtype)


# --------------------------------------------------------------------------
# options (src/LowRankApprox.jl:77-148)
# --------------------------------------------------------------------------

@dataclass
class Opts:
    """The LRAOptions fields the path reads, with LRAOptions(T) defaults."""
    atol: float = 0.0
    maxdet_niter: int = -1
    maxdet_tol: float = -1.0
    nb: int = 32
    pheig_orthtol: float | None = None
    pqrfact_retval: str = "qr"
    rank: int = -1
    rtol: float | None = None
    sketch: str = "randn"
    sketch_randn_niter: int = 0
    sketchfact_adap: bool = True
    randn_samp: tuple = (1, 8)
    srft_samp: tuple = (1, 8)
    sub_samp: tuple = (4, 8)
    snorm_niter: int = 32

    def for_dtype(self, dtype) -> "Opts":
        eps = float(np.finfo(np.dtype(dtype)).eps)
        o = replace(self)
        if o.rtol is None:
            o.rtol = 5 * eps
        if o.pheig_orthtol is None:
            o.pheig_orthtol = float(np.sqrt(eps))
        return o


# --------------------------------------------------------------------------
# injected randomness
# --------------------------------------------------------------------------

@dataclass
class RandStream:
    """Caller-supplied random numbers, consumed in the library's order:
    Gaussians as given; ints as indices 1 + (v - 1) mod M, or -- for the
    sparse sketch's permutation -- as sort keys ranked stably."""
    gauss: np.ndarray = field(default_factory=lambda: np.zeros(0))
    ints: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    g: int = 0
    q: int = 0

    def take_gauss(self, n: int) -> np.ndarray:
        if self.g + n > len(self.gauss):
            raise ValueError("gauss stream exhausted")
        out = self.gauss[self.g:self.g + n]
        self.g += n
        return out

    def take_ints(self, n: int) -> np.ndarray:
        if self.q + n > len(self.ints):
            raise ValueError("int stream exhausted")
        out = self.ints[self.q:self.q + n]
        self.q += n
        return out


# --------------------------------------------------------------------------
# pivoted QR core (src/pqr.jl:343-501)
# --------------------------------------------------------------------------

def laqps(m, n, offset, nb, a, lda, jpvt, tau, vn1, vn2, auxv, f, ldf, *, backend="oracle",
          a_off=0, v_off=0):
    """One xLAQPS block; arrays are numpy buffers, offsets in elements."""
    dt = a.dtype
    isz = dt.itemsize
    kb = np.zeros(1, np.int64)
    pa = _ptr(a) + a_off * lda * isz
    pj = _ptr(jpvt) + a_off * 8
    pt = _ptr(tau) + a_off * isz
    p1 = _ptr(vn1) + v_off * vn1.dtype.itemsize
    p2 = _ptr(vn2) + v_off * vn2.dtype.itemsize
    if backend == "oracle":
        getattr(_lib(), f"ora_{_sfx(dt)}laqps")(m, n, offset, nb, _ptr(kb), pa, lda, pj, pt, p1,
                                                 p2, _ptr(auxv), _ptr(f), ldf)
    else:
        lp = _lapack()
        if lp is None:
            raise RuntimeError("LAPACK xLAQPS not available")
        ints = [np.array([v], np.int64) for v in (m, n, offset, nb, lda, ldf)]
        getattr(lp, f"scipy_{_sfx(dt)}laqps_64_")(
            _ptr(ints[0]), _ptr(ints[1]), _ptr(ints[2]), _ptr(ints[3]), _ptr(kb), pa,
            _ptr(ints[4]), pj, pt, p1, p2, _ptr(auxv), _ptr(f), _ptr(ints[5]))
    return int(kb[0])


def colnorms(B: np.ndarray) -> np.ndarray:
    """`norm(view(A,:,j))` for every column (src/pqr.jl:376-386)."""
    return np.sqrt(np.einsum("ij,ij->j", B.astype(np.float64), B.astype(np.float64))).astype(B.dtype)


def geqp3_adap(B: np.ndarray, opts: Opts, backend: str = "oracle"):
    """geqp3_adap! (src/pqr.jl:348-418), in place on Fortran-ordered B.

    Returns (p, tau, k) with p 1-based (int64).  backend "c" runs the whole
    loop inside the C restatement; "oracle" / "lapack" run the block loop
    here around the C or the real LAPACK xLAQPS.
    """
    assert B.flags.f_contiguous
    m, n = B.shape
    lda = max(1, m)
    jpvt = np.arange(1, n + 1, dtype=np.int64)
    l = min(m, n)
    k = l if (opts.rank < 0 or opts.rank > l) else opts.rank
    tau = np.zeros(max(k, 1), B.dtype)
    if k <= 0:
        return jpvt, tau[:0], 0
    if np.iscomplexobj(B) and backend != "lapack":
        return _geqp3_complex(B, opts, k, jpvt, tau)
    if backend == "c":
        kout = np.zeros(1, np.int64)
        getattr(_lib(), f"ora_{_sfx(B.dtype)}geqp3_adap")(
            m, n, _ptr(B), lda, _ptr(jpvt), _ptr(tau), float(opts.atol), float(opts.rtol),
            int(opts.rank), int(opts.nb), _ptr(kout))
        return jpvt, tau[:k], int(kout[0])
    nb = min(opts.nb, k)
    vn1 = np.empty(n, _real(B.dtype))
    for j in range(n):
        vn1[j] = _nrm2(B[:, j]) if not np.iscomplexobj(B) else np.linalg.norm(B[:, j])
    vn2 = vn1.copy()
    maxnrm = float(vn1.max()) if n else 0.0
    ptol = max(opts.atol, opts.rtol * maxnrm)
    auxv = np.zeros(nb, B.dtype)
    f = np.zeros((n + 1) * nb, B.dtype)
    j = 1
    while j <= k:
        jb = min(nb, k - j + 1)
        kb = laqps(m, n - j + 1, j - 1, jb, B, lda, jpvt, tau, vn1, vn2, auxv, f,
                   max(1, n - j + 1), backend=backend, a_off=j - 1, v_off=j - 1)
        jn = j + kb
        if abs(B[jn - 2, jn - 2]) <= ptol:
            for i in range(j, jn):
                if abs(B[i - 1, i - 1]) <= ptol:
                    return jpvt, tau[:k], i - 1
        j = jn
    return jpvt, tau[:k], k


def _geqp3_complex(B, opts: Opts, kmax: int, jpvt, tau):
    """geqp3_adap! for complex types (src/pqr.jl:348-418) with the rules of
    ZLAQPS / CLAQPS (src/lapack.jl:117-139) column by column: IxAMAX pivots
    on the partial norms, the complex xLARFG reflector (beta real), H^H
    applied to the trailing columns, the tol3z downdate whose unreliable
    columns are recomputed and end the block, and the block-end rank test.
    Checked against the real LAPACK routine in the oracle's tests."""
    m, n = B.shape
    rdt = _real(B.dtype)
    eps = float(np.finfo(rdt).eps) / 2
    tol3z = np.sqrt(eps)
    vn1 = np.array([np.linalg.norm(B[:, j]) for j in range(n)], np.float64)
    vn2 = vn1.copy()
    ptol = max(opts.atol, opts.rtol * (vn1.max() if n else 0.0))
    lastrk = min(m, n)
    nb = max(1, min(opts.nb, kmax))
    c = 0
    while c < kmax:
        jb = min(nb, kmax - c)
        kk, first_small, last_small, flag = 0, -1, False, False
        while kk < jb and not flag:
            pvt = c + int(np.argmax(vn1[c:]))
            if pvt != c:
                B[:, [c, pvt]] = B[:, [pvt, c]]
                jpvt[c], jpvt[pvt] = jpvt[pvt], jpvt[c]
                vn1[pvt], vn2[pvt] = vn1[c], vn2[c]
            alpha = complex(B[c, c])
            x = B[c + 1:, c].astype(np.complex128)
            xnorm = float(np.linalg.norm(x))
            if xnorm == 0 and alpha.imag == 0:
                t, beta, scal = 0j, alpha.real, 1.0 + 0j
            else:
                r = float(np.sqrt(alpha.real ** 2 + alpha.imag ** 2 + xnorm ** 2))
                beta = -np.copysign(r, alpha.real)
                t = complex((beta - alpha.real) / beta, -alpha.imag / beta)
                scal = 1.0 / (alpha - beta)
            tau[c] = t
            v = np.concatenate([[1.0 + 0j], x * scal])
            if t != 0 and c + 1 < n:
                W = v.conj() @ B[c:, c + 1:].astype(np.complex128)
                B[c:, c + 1:] = (B[c:, c + 1:] - np.conj(t) * np.outer(v, W)).astype(B.dtype)
            B[c, c] = beta
            B[c + 1:, c] = (x * scal).astype(B.dtype)
            if c < lastrk - 1:
                for j in range(c + 1, n):
                    if vn1[j] != 0:
                        temp = abs(complex(B[c, j])) / vn1[j]
                        temp = max(0.0, (1 + temp) * (1 - temp))
                        temp2 = temp * (vn1[j] / vn2[j]) ** 2
                        if temp2 <= tol3z:
                            vn1[j] = vn2[j] = np.linalg.norm(B[c + 1:, j])
                            flag = True
                        else:
                            vn1[j] *= np.sqrt(temp)
            small = abs(beta) <= ptol
            if small and first_small < 0:
                first_small = c
            last_small = small
            c += 1
            kk += 1
        if last_small:
            return jpvt, tau[:kmax], first_small
    return jpvt, tau[:kmax], kmax


def _nrm2(x: np.ndarray):
    """xNRM2 of the C restatement."""
    x = np.ascontiguousarray(x)
    return x.dtype.type(getattr(_lib(), f"ora_{_sfx(x.dtype)}nrm2")(len(x), _ptr(x), 1))


def maxdet_t(R: np.ndarray) -> np.ndarray:
    """T = R11 \\ R12 (src/pqr.jl:438-442), back substitution like xTRSM."""
    k, n = R.shape
    R = np.asfortranarray(R)
    if np.iscomplexobj(R):
        import scipy.linalg
        if k == 0 or n == k:
            return np.zeros((k, n - k), R.dtype, order="F")
        return np.asfortranarray(scipy.linalg.solve_triangular(np.triu(R[:, :k]), R[:, k:]).astype(R.dtype))
    T = np.zeros((k, n - k), R.dtype, order="F")
    if k > 0 and n > k:
        getattr(_lib(), f"ora_{_sfx(R.dtype)}maxdet_t")(k, n, _ptr(R), max(1, k), _ptr(T), max(1, k))
    return T


def findmaxabs(x: np.ndarray):
    """findmaxabs (src/util.jl:13-23): ties go to the LAST index (1-based)."""
    flat = np.abs(x.reshape(-1, order="F"))
    if flat.size == 0:
        return 0.0, 0
    m = flat.max()
    idx = np.nonzero(flat == m)[0][-1]
    return float(m), int(idx) + 1


def maxdet_swapcols(Q, R, p, T, opts: Opts):
    """maxdet_swapcols! / maxdet_update! (src/pqr.jl:445-501), in place."""
    k, n = R.shape
    retq = "q" in opts.pqrfact_retval
    retr = "r" in opts.pqrfact_retval
    niter = 0
    while True:
        tmax, idx = findmaxabs(T)
        if tmax <= 1 + opts.maxdet_tol:
            break
        if niter == opts.maxdet_niter:
            break
        niter += 1
        i, j = (idx - 1) % k, (idx - 1) // k          # 0-based
        p[i], p[k + j] = p[k + j], p[i]
        w1 = T[:, j].copy()
        T[:, j] = 0
        w1[i] -= 1
        T[i, j] = 1
        w2 = T[i, :].copy()
        T -= (1.0 / (1 + w1[i])) * np.outer(w1, w2)
        if retr:
            R[:, i] += R[:, :k] @ w1
    if niter == 0:
        return Q, R
    qf, rf = np.linalg.qr(R[:, :k], mode="complete")
    if retq and Q is not None:
        Q = Q @ qf
    if retr:
        R[:, :k] = np.triu(rf)
        R[:, k:] = np.triu(rf) @ T
    return Q, R


def pqrback_postproc(B: np.ndarray, p, tau, k: int, opts: Opts) -> dict:
    """pqrback_postproc (src/pqr.jl:420-436)."""
    retq = "q" in opts.pqrfact_retval
    retr = "r" in opts.pqrfact_retval
    rett = "t" in opts.pqrfact_retval
    n = B.shape[1]
    maxdet = 0 < k < n and opts.maxdet_tol >= 0
    Q = _orgqr(B[:, :k], tau[:k]) if retq else None
    R = np.triu(B[:k, :]).astype(B.dtype) if (retr or rett or maxdet) else None
    T = maxdet_t(R) if (rett or maxdet) else None
    p = np.array(p, np.int64)
    if maxdet:
        Q, R = maxdet_swapcols(Q, R, p, T, opts)
        R = R if retr else None
    return {"Q": Q, "R": R, "T": T, "p": p, "k": int(k)}


def _orgqr(V: np.ndarray, tau: np.ndarray) -> np.ndarray:
    """Explicit Q from Householder vectors (LAPACK xORGQR semantics)."""
    m, k = V.shape
    Q = np.zeros((m, k), V.dtype, order="F")
    for c in range(k):
        Q[c, c] = 1
    for i in range(k - 1, -1, -1):
        v = np.zeros(m, V.dtype)
        v[i] = 1
        v[i + 1:] = V[i + 1:, i]
        w = v[i:].conj() @ Q[i:, :]
        Q[i:, :] -= tau[i] * np.outer(v[i:], w)
    return Q


def pqrfact_backend(B: np.ndarray, opts: Opts, backend: str = "oracle") -> dict:
    p, tau, k = geqp3_adap(B, opts, backend)
    return pqrback_postproc(B, p, tau, k, opts)


# --------------------------------------------------------------------------
# sketches (src/sketch.jl)
# --------------------------------------------------------------------------

def _op(A, trans):
    return A if trans == "n" else _H(A)


def orthrows(B):
    """orthrows!(thin=false) (src/util.jl:87-97): LQ, keep Q's rows."""
    m, n = B.shape
    k = min(m, n)
    q, _ = np.linalg.qr(_H(B))
    out = np.zeros_like(B)
    out[:k, :] = _H(q[:, :k])
    return out


def orthcols(B):
    m, n = B.shape
    k = min(m, n)
    q, _ = np.linalg.qr(B)
    out = np.zeros_like(B)
    out[:, :k] = q[:, :k]
    return out


def _ishermitian(A) -> bool:
    return A.shape[0] == A.shape[1] and np.array_equal(A, _H(A))


def sketch_randn(side, trans, A, order, opts: Opts, rs: RandStream):
    """sketch_randn_{ln,lc,rn,rc} (src/sketch.jl:129-220)."""
    dt = A.dtype
    isherm = _ishermitian(A)
    opA = _op(A, trans)
    if side == "left":
        M = opA.shape[0]
        S = crandn(rs, order * M, dt).reshape((order, M), order="F")
        Bp = S @ opA
        for _ in range(opts.sketch_randn_niter):
            Bp = orthrows(Bp)
            Bq = Bp @ _H(opA)
            if isherm:
                Bp = Bq
            else:
                Bq = orthrows(Bq)
                Bp = Bq @ opA
        return np.asfortranarray(Bp.astype(dt))
    N = opA.shape[1]
    S = crandn(rs, N * order, dt).reshape((N, order), order="F")
    Bp = opA @ S
    for _ in range(opts.sketch_randn_niter):
        Bp = orthcols(Bp)
        Bq = _H(opA) @ Bp
        if isherm:
            Bp = Bq
        else:
            Bq = orthcols(Bq)
            Bp = opA @ Bq
    return np.asfortranarray(Bp.astype(dt))


def sketch_sub(side, trans, A, order, rs: RandStream):
    """RandomSubset mul! (src/sketch.jl:248-293): rows/cols with replacement."""
    opA = _op(A, trans)
    if side == "left":
        r = (rs.take_ints(order) - 1) % opA.shape[0]
        return np.asfortranarray(opA[r, :])
    r = (rs.take_ints(order) - 1) % opA.shape[1]
    return np.asfortranarray(opA[:, r])


def _srft_apply_columns(Xin: np.ndarray, d: np.ndarray, idx: np.ndarray, k: int) -> np.ndarray:
    """srft_reshape! + srft_apply! (src/sketch.jl:378-450) for every column
    of Xin (M x c), real element types.  Returns k x c."""
    M, c = Xin.shape
    dt = Xin.dtype
    l = k
    while M % l > 0:
        l -= 1
    mm = M // l
    out = np.zeros((k, c), dt)
    n = l * mm
    wn = np.exp(-2j * np.pi / n)
    wm = np.exp(-2j * np.pi / mm)
    cnyq = l // 2
    for col in range(c):
        x = (d * Xin[:, col]).astype(dt)
        X = x.reshape((l, mm))                       # row-major fill, X[j,k]
        Y = np.fft.fft(X.astype(np.float64), axis=0)  # R2HC along dim 1
        R2 = np.empty((l, mm))
        R2[:cnyq + 1, :] = Y[:cnyq + 1, :].real
        for cc in range(1, (l + 1) // 2):
            R2[l - cc, :] = Y[cc, :].imag
        R2 = R2.astype(dt)
        y = np.zeros(k, np.float64)
        i = 0
        while i < k:
            idx_ = int(idx[i]) - 1
            row = idx_ // l
            cl = idx_ % l
            w = (wm ** row) * (wn ** cl)
            cswap = cl > cnyq
            ia = l - cl if cswap else cl
            ib = l - ia if cl > 0 else 0
            s = 1.0 + 0j
            if i == k - 1:
                acc = 0.0
                for j in range(mm):
                    a = float(R2[ia, j])
                    b = 0.0 if (ib == 0 or ib == ia) else float(R2[ib, j])
                    b = -b if cswap else b
                    acc += (s * complex(a, b)).real
                    s *= w
                y[i] = acc
            else:
                acc_r = 0.0
                acc_i = 0.0
                for j in range(mm):
                    a = float(R2[ia, j])
                    b = 0.0 if (ib == 0 or ib == ia) else float(R2[ib, j])
                    b = -b if cswap else b
                    z = s * complex(a, b)
                    acc_r += z.real
                    acc_i += z.imag
                    s *= w
                y[i] = acc_r
                y[i + 1] = acc_i
                i += 1
            i += 1
        out[:, col] = y.astype(dt)
    return out


def srft_exact(Xin: np.ndarray, d: np.ndarray, idx: np.ndarray, k: int) -> np.ndarray:
    """The same SRFT sample computed from a full-length FFT (for checking the
    restatement above): output pairs (Re, Im) of DFT(d * x)[idx[i]-1] for
    i = 1, 3, 5, ...; an odd last slot holds Re of DFT(d * x)[idx[k]-1]."""
    M, c = Xin.shape
    Z = np.fft.fft((d[:, None] * Xin.astype(np.float64)), axis=0)
    out = np.zeros((k, c))
    i = 0
    while i < k:
        f = int(idx[i]) - 1
        if i == k - 1:
            out[i] = Z[f].real
        else:
            out[i] = Z[f].real
            out[i + 1] = Z[f].imag
            i += 1
        i += 1
    return out.astype(Xin.dtype)


def srft_sampled_dft(Xin: np.ndarray, d: np.ndarray, idx: np.ndarray, k: int, chunk: int = 8192) -> np.ndarray:
    """srft_exact's output computed from the sampled DFT rows only: for the
    frequencies f = idx[i] - 1 it forms exp(-2 pi i f j / M) with the phase
    reduced exactly as (f * j) mod M, and multiplies by d * x (float64 GEMMs
    over row chunks).  Same values as the full FFT up to rounding, at a cost
    of 2 k M c flops, which keeps tall sketches (65536 rows) tractable."""
    M, c = Xin.shape
    pos = list(range(0, k, 2))
    freqs = np.array([int(idx[i]) - 1 for i in pos], np.int64)
    npos = len(pos)
    acc = np.zeros((2 * npos, c))           # rows: Re of each frequency, then Im
    for j0 in range(0, M, chunk):
        j = np.arange(j0, min(M, j0 + chunk), dtype=np.int64)
        ang = (2 * np.pi / M) * ((freqs[:, None] * j[None, :]) % M).astype(np.float64)
        E = np.concatenate([np.cos(ang), -np.sin(ang)])
        X = d[j0:j0 + len(j), None] * Xin[j0:j0 + len(j), :].astype(np.float64)
        acc += E @ X
    out = np.zeros((k, c))
    for r, i in enumerate(pos):
        out[i] = acc[r]
        if i + 1 < k:
            out[i + 1] = acc[npos + r]
    return out.astype(Xin.dtype)


def srft_sampled_dft_complex(Xin: np.ndarray, d: np.ndarray, idx: np.ndarray, k: int, chunk: int = 8192):
    """The complex SRFT (srft_apply! for complex types, src/sketch.jl:452-472):
    y_i = sum_t d_t x_t exp(-2 pi i f_i t / M), f_i = idx_i - 1, one
    complex value per index, the phase reduced exactly as (f t) mod M."""
    M, c = Xin.shape
    f = np.asarray(idx, np.int64) - 1
    out = np.zeros((k, c), np.complex128)
    for j0 in range(0, M, chunk):
        j = np.arange(j0, min(M, j0 + chunk), dtype=np.int64)
        E = np.exp(-2j * np.pi * (((f[:, None] * j[None, :]) % M).astype(np.float64) / M))
        out += E @ (d[j0:j0 + len(j), None] * Xin[j0:j0 + len(j), :].astype(np.complex128))
    return out.astype(Xin.dtype)


def sketch_srft(side, trans, A, order, rs: RandStream, fast: bool = False):
    """SRFT mul! (src/sketch.jl:474-522), real types, left side."""
    opA = _op(A, trans)
    if side != "left":
        return sketch_srft("left", "n", opA.T, order, rs, fast).T.copy(order="F")
    M = opA.shape[0]
    if np.iscomplexobj(opA):
        # random phases crandn / |crandn| (src/sketch.jl:345-351); the
        # sample is the DFT of d .* x at the frequencies idx (:452-472)
        z = crandn(rs, M, np.complex128)
        d = z / np.abs(z)
        idx = (rs.take_ints(order) - 1) % M + 1
        return np.asfortranarray(srft_sampled_dft_complex(opA, d, idx, order))
    d = np.where(rs.take_gauss(M) > 0, 1.0, -1.0)
    idx = (rs.take_ints(order) - 1) % M + 1
    if fast:
        return np.asfortranarray(srft_sampled_dft(opA, d, idx, order))
    return np.asfortranarray(_srft_apply_columns(opA, d, idx, order))


def sketch_sprn(side, trans, A, order, rs: RandStream):
    """SparseRandomGaussian mul! (src/sketch.jl:571-653), real types."""
    opA = _op(A, trans)
    if side != "left":
        return sketch_sprn("left", "n", opA.T, order, rs).T.copy(order="F")
    M, N = opA.shape
    r = np.argsort(rs.take_ints(M), kind="stable")      # randperm(m) from M keys
    g = crandn(rs, M, A.dtype)
    C = np.zeros((order, N), A.dtype, order="F")
    idx = 0
    for i in range(1, order + 1):
        p = (M - i) // order + 1
        s = g[idx:idx + p]
        C[i - 1, :] = s @ opA[r[idx:idx + p], :]
        idx += p
    return C


def sketch(side, trans, A, order, opts: Opts, rs: RandStream, fast_srft=False):
    """sketch(side, trans, A, order) (src/sketch.jl:35-46)."""
    s = opts.sketch
    if s == "randn":
        return sketch_randn(side, trans, A, order, opts, rs)
    if s == "sub":
        return sketch_sub(side, trans, A, order, rs)
    if s == "srft":
        return sketch_srft(side, trans, A, order, rs, fast_srft)
    if s == "sprn":
        return sketch_sprn(side, trans, A, order, rs)
    raise ValueError("sketch")


def _samp(opts: Opts, n: int) -> int:
    s = opts.sketch
    if s == "randn":
        a, b = opts.randn_samp
    elif s == "srft":
        a, b = opts.srft_samp
    elif s == "sub":
        a, b = opts.sub_samp
    else:
        return n                                    # sprn: order = n
    return a * n + b


def sketchfact(side, trans, A, opts: Opts, rs: RandStream, backend="oracle", fast_srft=False,
               trace=None) -> dict:
    """sketchfact_{randn,sub,srft,sprn} (src/sketch.jl:223-240 and twins)."""
    opts = opts.for_dtype(A.dtype)
    if opts.sketch == "none":
        opts = replace(opts, sketch="randn")
    if opts.sketchfact_adap or opts.rank < 0:
        n = opts.nb
        opts_ = replace(opts, maxdet_tol=-1.0)
        steps = 0
        while True:
            order = _samp(opts, n)
            B = sketch(side, trans, A, order, opts, rs, fast_srft)
            B0 = B.copy(order="F") if trace is not None else None
            p, tau, k = geqp3_adap(B, opts_, backend)
            steps += 1
            if trace is not None:
                trace.append({"order": order, "k": k, "B": B0})
            if k < n:
                F = pqrback_postproc(B, p, tau, k, opts)
                F["nsteps"] = steps
                return F
            n *= 2
    order = _samp(opts, opts.rank)
    B = sketch(side, trans, A, order, opts, rs, fast_srft)
    if trace is not None:
        trace.append({"order": order, "B": B.copy(order="F")})
    F = pqrfact_backend(B, opts, backend)
    F["nsteps"] = 1
    return F


# --------------------------------------------------------------------------
# factorizations
# --------------------------------------------------------------------------

def prange(trans, A, opts: Opts, rs: RandStream, backend="oracle") -> np.ndarray:
    """prange (src/prange.jl:14-77): an orthonormal basis of the range of
    op(A), or of A and A' together for trans "b"."""
    opts = opts.for_dtype(A.dtype)
    if trans == "b":
        m, n = A.shape
        if m != n:
            raise ValueError("prange(:b) needs a square matrix")
        if _ishermitian(A):
            return prange("n", A, opts, rs, backend)
        oq = replace(opts, pqrfact_retval="qr")
        if opts.sketch == "none":
            Fr = pqrfact("c", A, oq, rs, backend)
            Fc = pqrfact("n", A, oq, rs, backend)
        else:
            Fr = sketchfact("right", "c", A, oq, rs, backend)
            Fc = sketchfact("right", "n", A, oq, rs, backend)
        kr, kc = Fr["k"], Fc["k"]
        B = np.concatenate([Fr["Q"] @ np.triu(Fr["R"][:kr, :kr]), Fc["Q"] @ np.triu(Fc["R"][:kc, :kc])], axis=1)
        return pqrfact_backend(np.asfortranarray(B.astype(A.dtype)), replace(opts, pqrfact_retval="q"), backend)["Q"]
    oq = replace(opts, pqrfact_retval="q")
    if opts.sketch == "none":
        return pqrfact(trans, A, oq, rs, backend)["Q"]
    if opts.sketch == "sub":
        F = sketchfact("left", trans, A, opts, rs, backend)
        k = F["k"]
        B = np.asfortranarray(_op(A, trans)[:, np.asarray(F["p"][:k]) - 1])
        return orthcols(B)[:, :min(B.shape)]
    return sketchfact("right", trans, A, oq, rs, backend)["Q"]


def _getcols(trans, A, cols):
    """getcols (src/util.jl:25-29), cols 1-based."""
    c = np.asarray(cols, np.int64) - 1
    return np.asfortranarray(A[:, c] if trans == "n" else _H(A[c, :]))


def idfact(trans, A, opts: Opts, rs: RandStream, backend="oracle", fast_srft=False,
           trace=None) -> dict:
    """idfact (src/id.jl:434-447): returns sk, rd (1-based), T, k."""
    opts = replace(opts.for_dtype(A.dtype), pqrfact_retval="t")
    if opts.sketch == "none":
        B = np.asfortranarray(_op(A, trans).copy())
        if trace is not None:
            trace.append({"order": None, "B": B.copy(order="F")})
        F = pqrfact_backend(B, opts, backend)
        F["nsteps"] = 0
    else:
        F = sketchfact("left", trans, A, opts, rs, backend, fast_srft, trace)
    k = F["k"]
    return {"sk": F["p"][:k].copy(), "rd": F["p"][k:].copy(), "T": F["T"], "k": k,
            "nsteps": F["nsteps"]}


def id_matrix(trans, A, V) -> np.ndarray:
    """Dense ID(trans, A, V) = C * [I T] * P' (src/id.jl:212-215)."""
    C = _getcols(trans, A, V["sk"])
    n = len(V["sk"]) + len(V["rd"])
    k = V["k"]
    out = np.zeros((C.shape[0], n), A.dtype)
    out[:, V["sk"] - 1] = C
    if k > 0 and n > k:
        out[:, V["rd"] - 1] = C @ V["T"]
    return out


def pqrfact(trans, A, opts: Opts, rs: RandStream, backend="oracle", trace=None) -> dict:
    """pqrfact (src/pqr.jl:290-307)."""
    opts = opts.for_dtype(A.dtype)
    if opts.sketch == "none":
        B = np.asfortranarray(_op(A, trans).copy())
        if trace is not None:
            trace.append({"order": None, "B": B.copy(order="F")})
        return pqrfact_backend(B, opts, backend)
    V = idfact(trans, A, opts, rs, backend, trace=trace)
    Aq = _getcols(trans, A, V["sk"])
    q, r = np.linalg.qr(Aq)
    out = {"p": np.concatenate([V["sk"], V["rd"]]), "k": V["k"], "T": None, "Q": None, "R": None}
    if "q" in opts.pqrfact_retval:
        out["Q"] = q
    if "r" in opts.pqrfact_retval:
        out["R"] = np.concatenate([r, r @ V["T"]], axis=1) if V["T"] is not None else r
    if "t" in opts.pqrfact_retval:
        out["T"] = V["T"]
    return out


def psvdrank(s: np.ndarray, opts: Opts) -> int:
    """psvdrank (src/psvd.jl:301-308)."""
    k = len(s)
    if k == 0:
        return 0
    ptol = max(opts.atol, opts.rtol * s[0])
    for i in range(1, k):
        if s[i] <= ptol:
            return i
    return k


def _v_matrix(V, n, dtype):
    """IDPackedV as a dense k x n matrix [I T] P'."""
    k = V["k"]
    out = np.zeros((k, n), dtype)
    out[:, V["sk"] - 1] = np.eye(k, dtype=dtype)
    if n > k:
        out[:, V["rd"] - 1] = V["T"]
    return out


def psvdfact(A, opts: Opts, rs: RandStream, backend="oracle", vals_only=False, trace=None) -> dict:
    """psvdfact / psvdvals (src/psvd.jl:238-290)."""
    opts = opts.for_dtype(A.dtype)
    m, n = A.shape
    if m >= n:
        V = idfact("n", A, opts, rs, backend, trace=trace)
        q, r = np.linalg.qr(_getcols("n", A, V["sk"]))
        W = r @ _v_matrix(V, n, A.dtype)
        if vals_only:
            s = np.linalg.svd(W, compute_uv=False)
        else:
            u, s, vt = np.linalg.svd(W, full_matrices=False)
    else:
        V = idfact("c", A, opts, rs, backend, trace=trace)
        q, r = np.linalg.qr(_getcols("c", A, V["sk"]))
        W = _H(_v_matrix(V, m, A.dtype)) @ _H(r)
        if vals_only:
            s = np.linalg.svd(W, compute_uv=False)
        else:
            u, s, vt = np.linalg.svd(W, full_matrices=False)
    k = psvdrank(s, opts)
    if vals_only:
        return {"S": s[:k], "k": k}
    if m >= n:
        U = q @ u[:, :k]
        Vt = vt[:k, :]
    else:
        U = u[:, :k]
        Vt = vt[:k, :] @ _H(q)
    return {"U": U, "S": s[:k], "Vt": Vt, "k": k, "id_k": V["k"], "sk": V["sk"], "rd": V["rd"]}


def _pheigrank1(w, opts: Opts, wmax):
    k = len(w)
    k = min(opts.rank, k) if opts.rank >= 0 else k
    ptol = max(opts.atol, opts.rtol * wmax)
    for i in range(1, k):
        if abs(w[i]) <= ptol:
            return i
    return k


def pheigrank(w: np.ndarray, opts: Opts):
    """pheigrank (src/pheig.jl:322-339) -> (kn, kp)."""
    n = len(w)
    if n == 0:
        return 0, 0
    wmax = max(abs(w[0]), abs(w[-1]))
    lo = int(np.searchsorted(w, 0, side="left"))
    hi = int(np.searchsorted(w, 0, side="right"))
    kn = _pheigrank1(w[:lo], opts, wmax)
    kp = _pheigrank1(w[hi:][::-1], opts, wmax)
    return kn, kp


def pheigorth(values, vectors, opts: Opts):
    """pheigorth! (src/pheig.jl:342-364), in place."""
    n = len(values)
    a = 0
    while a < n:
        va = values[a]
        b = a + 1
        while b < n:
            vb = values[b]
            if 2 * abs((va - vb) / (va + vb)) > opts.pheig_orthtol:
                break
            b += 1
        b -= 1
        for i in range(a, b + 1):
            vi = vectors[:, i]
            for j in range(i + 1, b + 1):
                vectors[:, j] -= (vi @ vectors[:, j]) * vi
        a = b + 1


def pheigfact(A, opts: Opts, rs: RandStream, backend="oracle", vals_only=False, trace=None) -> dict:
    """pheigfact / pheigvals (src/pheig.jl:276-311)."""
    opts = opts.for_dtype(A.dtype)
    if not _ishermitian(A):
        raise ValueError("matrix must be Hermitian")
    n = A.shape[0]
    V = idfact("n", A, opts, rs, backend, trace=trace)
    q, r = np.linalg.qr(_H(_v_matrix(V, n, A.dtype)))
    sk = V["sk"] - 1
    B = r @ (A[np.ix_(sk, sk)] @ _H(r))
    # hermitianize!(B) (src/util.jl:31-45): the averaged upper triangle
    U = 0.5 * (B + _H(B))
    Bh = np.triu(U) + _H(np.triu(U, 1))
    if vals_only:
        w = np.linalg.eigvalsh(Bh)
    else:
        w, Z = np.linalg.eigh(Bh)
    kn, kp = pheigrank(w, opts)
    kk = len(w)
    idx = np.r_[0:kn, kk - kp:kk] if kn + kp < kk else np.arange(kk)
    w = w[idx]
    if vals_only:
        return {"values": w, "k": len(w)}
    Z = Z[:, idx].copy()
    pheigorth(w, Z, opts)
    return {"values": w, "vectors": q @ Z, "k": len(w), "id_k": V["k"], "sk": V["sk"], "rd": V["rd"]}


def curfact(A, opts: Opts, rs: RandStream, backend="oracle") -> dict:
    """curfact (src/cur.jl:532-564)."""
    opts = replace(opts.for_dtype(A.dtype), pqrfact_retval="")
    if opts.sketch == "none":
        return _curfact_none(A, opts, backend)
    if _ishermitian(A):
        F = sketchfact("left", "n", A, opts, rs, backend)
        cols = F["p"][:F["k"]]
        return {"kind": 1, "rows": cols.copy(), "cols": cols.copy()}
    m, n = A.shape
    if m >= n:
        F = sketchfact("left", "c", A, opts, rs, backend)
        rows = F["p"][:F["k"]]
        F = sketchfact("left", "n", np.asfortranarray(A[rows - 1, :]), opts, rs, backend)
        cols = F["p"][:F["k"]]
    else:
        F = sketchfact("left", "n", A, opts, rs, backend)
        cols = F["p"][:F["k"]]
        F = sketchfact("left", "c", np.asfortranarray(A[:, cols - 1]), opts, rs, backend)
        rows = F["p"][:F["k"]]
    k = min(len(rows), len(cols))
    return {"kind": 0, "rows": rows[:k].copy(), "cols": cols[:k].copy()}


def cur_build(A, U: dict) -> dict:
    """CUR(A, U) (src/cur.jl:85-115): C = A[:, cols], R = A[rows, :] and the
    pseudo-inverse of A[rows, cols] as (V, 1 ./ S, U') from its SVD."""
    rows = np.asarray(U["rows"], np.int64)
    cols = np.asarray(U["cols"], np.int64)
    C = np.asfortranarray(A[:, cols - 1])
    R = np.asfortranarray(A[rows - 1, :])
    Uw, s, Vt = np.linalg.svd(C[rows - 1, :].astype(np.complex128 if np.iscomplexobj(C) else np.float64))
    return {"rows": rows, "cols": cols, "C": C, "R": R, "U": (_H(Vt), 1.0 / s, _H(Uw))}


def _curfact_none(A, opts, backend):
    """curfact_none (src/cur.jl:574-606)."""
    if _ishermitian(A):
        F = pqrfact_backend(np.asfortranarray(A.copy()), opts, backend)
        cols = F["p"][:F["k"]]
        return {"kind": 1, "rows": cols.copy(), "cols": cols.copy()}
    m, n = A.shape
    if m >= n:
        F = pqrfact_backend(np.asfortranarray(_H(A).copy()), opts, backend)
        rows = F["p"][:F["k"]]
        F = pqrfact_backend(np.asfortranarray(A[rows - 1, :]), opts, backend)
        cols = F["p"][:F["k"]]
    else:
        F = pqrfact_backend(np.asfortranarray(A.copy()), opts, backend)
        cols = F["p"][:F["k"]]
        F = pqrfact_backend(np.asfortranarray(_H(A[:, cols - 1])), opts, backend)
        rows = F["p"][:F["k"]]
    k = min(len(rows), len(cols))
    return {"kind": 0, "rows": rows[:k].copy(), "cols": cols[:k].copy()}


def snorm(apply, applyc, n: int, dtype, opts: Opts, rs: RandStream, hermitian=False) -> float:
    """snorm (src/snorm.jl:14-45) for an operator given as matvec closures."""
    opts = opts.for_dtype(dtype)
    xn = rs.take_gauss(n).astype(dtype)
    xnrm = float(np.linalg.norm(xn))
    s, t, niter = 1.0, 0.0, 0
    while s > 0 and abs(s - t) > max(opts.atol, t * opts.rtol):
        if niter == opts.snorm_niter:
            break
        niter += 1
        xn = xn * dtype(1 / xnrm)
        if hermitian:
            xn = apply(xn)
        else:
            xn = applyc(apply(xn))
        xnrm = float(np.linalg.norm(xn))
        t = s
        s = xnrm if hermitian else float(np.sqrt(xnrm))
    return s


def snorm_dense(A, opts: Opts, rs: RandStream) -> float:
    herm = _ishermitian(A)
    return snorm(lambda x: A @ x, lambda y: _H(A) @ y, A.shape[1], A.dtype.type, opts, rs, herm)


def snormdiff_dense(A, B, opts: Opts, rs: RandStream) -> float:
    """snormdiff(A, B) = snorm(LinOp(A) - LinOp(B)) (src/snorm.jl:50-53);
    the difference is Hermitian only if both are (src/linop.jl:163-169)."""
    herm = _ishermitian(A) and _ishermitian(B)
    return snorm(lambda x: A @ x - B @ x, lambda y: _H(A) @ y - _H(B) @ y, A.shape[1],
                 A.dtype.type, opts, rs, herm)


# --------------------------------------------------------------------------
# matrixlib (src/matrixlib.jl:4-48)
# --------------------------------------------------------------------------

def hilb(m: int, n: int | None = None, dtype=np.float64) -> np.ndarray:
    n = m if n is None else n
    i = np.arange(1, m + 1)[:, None]
    j = np.arange(1, n + 1)[None, :]
    return np.asfortranarray((1.0 / (i + j - 1)).astype(dtype))


def cauchy(x, y, dtype=np.float64) -> np.ndarray:
    return np.asfortranarray((1.0 / (np.asarray(x)[:, None] - np.asarray(y)[None, :])).astype(dtype))


def fourier(x, y) -> np.ndarray:
    return np.asfortranarray(np.exp(-2j * np.pi * np.outer(x, y)))
