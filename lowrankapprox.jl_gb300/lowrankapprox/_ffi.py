"""ctypes binding of liblra's C ABI (include/lra.h).

This is the same boundary a Julia ``ccall`` shim binds; the structs below
mirror lra.h field for field.  Loading fails loudly when the CUDA library
is missing: there is no CPU path behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblra.so")

LRA_OK, LRA_EINVAL, LRA_EDIM, LRA_ENOMEM, LRA_ETIMEDOUT, LRA_ENONFINITE, LRA_ECUDA, LRA_ERAND, \
    LRA_ENOTSUP, LRA_ENOTHERM, LRA_EBUSY = range(11)
LRA_F32, LRA_F64, LRA_C32, LRA_C64 = 0, 1, 2, 3
SKETCH = {"none": 0, "randn": 1, "sprn": 2, "srft": 3, "sub": 4}
RET_Q, RET_R, RET_T = 1, 2, 4
PREC = {"native": 0, "mixed": 1}


class lra_opts(C.Structure):
    _fields_ = [
        ("atol", C.c_double),
        ("maxdet_niter", C.c_int64),
        ("maxdet_tol", C.c_double),
        ("nb", C.c_int64),
        ("pheig_orthtol", C.c_double),
        ("pqrfact_retval", C.c_int32),
        ("sketch", C.c_int32),
        ("rank", C.c_int64),
        ("rtol", C.c_double),
        ("sketch_randn_niter", C.c_int64),
        ("sketchfact_adap", C.c_int32),
        ("verb", C.c_int32),
        ("sketchfact_randn_samp", C.c_int64 * 2),
        ("sketchfact_srft_samp", C.c_int64 * 2),
        ("sketchfact_sub_samp", C.c_int64 * 2),
        ("snorm_niter", C.c_int64),
        ("precision", C.c_int32),
        ("check_finite", C.c_int32),
        ("seed", C.c_uint64),
    ]


class lra_rand(C.Structure):
    _fields_ = [("gauss", C.c_void_p), ("gauss_len", C.c_int64),
                ("ints", C.c_void_p), ("ints_len", C.c_int64)]


class lra_id(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("nsteps", C.c_int32), ("k", C.c_int64), ("n", C.c_int64),
                ("sk", C.POINTER(C.c_int64)), ("rd", C.POINTER(C.c_int64)), ("T", C.c_void_p)]


class lra_pqr(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("retval", C.c_int32), ("m", C.c_int64), ("n", C.c_int64),
                ("k", C.c_int64), ("p", C.POINTER(C.c_int64)), ("Q", C.c_void_p), ("R", C.c_void_p),
                ("T", C.c_void_p)]


class lra_psvd(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("_pad", C.c_int32), ("m", C.c_int64), ("n", C.c_int64),
                ("k", C.c_int64), ("U", C.c_void_p), ("S", C.c_void_p), ("Vt", C.c_void_p)]


class lra_pheig(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("_pad", C.c_int32), ("n", C.c_int64), ("k", C.c_int64),
                ("values", C.c_void_p), ("vectors", C.c_void_p)]


class lra_cur(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("kr", C.c_int64), ("kc", C.c_int64),
                ("rows", C.POINTER(C.c_int64)), ("cols", C.POINTER(C.c_int64))]


class lra_matdesc(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("lda", C.c_int64), ("A", C.c_void_p)]


LRA_REQ_IDFACT, LRA_REQ_PSVDFACT = 0, 1


class lra_request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("dtype", C.c_int32), ("trans", C.c_char), ("_pad", C.c_char * 7),
                ("m", C.c_int64), ("n", C.c_int64), ("lda", C.c_int64), ("A", C.c_void_p),
                ("opts", lra_opts), ("rand", C.POINTER(lra_rand))]


class lra_result(C.Structure):
    _fields_ = [("kind", C.c_int32), ("status", C.c_int32), ("id", C.POINTER(lra_id)),
                ("psvd", C.POINTER(lra_psvd)), ("queue_ms", C.c_double), ("run_ms", C.c_double),
                ("total_ms", C.c_double), ("slot", C.c_int32), ("_pad", C.c_int32),
                ("error", C.c_char * 160)]


class lra_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
                ("in_flight", C.c_int64), ("queued", C.c_int64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("matrices_per_s", C.c_double),
                ("hbm_budget", C.c_int64), ("hbm_in_use", C.c_int64)]


# the operator's product callback (lra_matmat_fn) and lra_linop
MATMAT = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                     C.c_void_p)


class lra_linop(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("dtype", C.c_int32), ("hermitian", C.c_int32),
                ("matmat", MATMAT), ("user", C.c_void_p)]


# every exported entry point: (name, restype, argtypes)
_vp, _i64, _i32, _d, _ch = C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_char
_P = C.POINTER
SIGNATURES = [
    ("lra_ctx_create", _i32, [_i32, _P(_vp)]),
    ("lra_ctx_destroy", None, [_vp]),
    ("lra_ctx_set_stream", _i32, [_vp, _vp]),
    ("lra_last_error", C.c_char_p, [_vp]),
    ("lra_status_string", C.c_char_p, [_i32]),
    ("lra_ctx_launches", _i64, [_vp]),
    ("lra_ctx_kernel_launches", _i64, [_vp, C.c_char_p]),
    ("lra_ctx_stage_ms", _i32, [_vp, _P(_d)]),
    ("lra_ctx_set_tuning", _i32, [_vp, C.c_char_p, _i64, _i64]),
    ("lra_ctx_get_tuning", _i32, [_vp, C.c_char_p, _i64]),
    ("lra_ctx_set_wait_limit", _i32, [_vp, _i64]),
    ("lra_ctx_probe_wait", _i32, [_vp]),
    ("lra_opts_init", _i32, [_P(lra_opts), _i32]),
    ("lra_chkopts", _i32, [_P(lra_opts)]),
    ("lra_sketch", _i32, [_vp, _i32, _ch, _ch, _i64, _i64, _vp, _i64, _i64, _P(lra_opts),
                          _P(lra_rand), _vp, _i64]),
    ("lra_sketchfact", _i32, [_vp, _i32, _ch, _ch, _i64, _i64, _vp, _i64, _P(lra_opts),
                              _P(lra_rand), _P(_P(lra_pqr))]),
    ("lra_prange", _i32, [_vp, _i32, _ch, _i64, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand), _P(_P(lra_pqr))]),
    ("lra_geqp3_adap", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _vp, _vp, _P(lra_opts), _P(_i64)]),
    ("lra_geqp3_adap_noalloc", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _vp, _vp, _P(lra_opts), _P(_i64)]),
    ("lra_idfact", _i32, [_vp, _i32, _ch, _i64, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand),
                          _P(_P(lra_id))]),
    ("lra_pqrfact", _i32, [_vp, _i32, _ch, _i64, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand),
                           _P(_P(lra_pqr))]),
    ("lra_psvdfact", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand), _i32,
                            _P(_P(lra_psvd))]),
    ("lra_pheigfact", _i32, [_vp, _i32, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand), _i32,
                             _P(_P(lra_pheig))]),
    ("lra_curfact", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _P(lra_opts), _P(lra_rand),
                           _P(_P(lra_cur))]),
    ("lra_cur_middle", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _i64, _P(_i64), _P(_i64), _P(_P(lra_psvd))]),
    ("lra_rand_gauss", _i32, [_vp, C.c_uint64, C.c_uint64, _i64, _vp]),
    ("lra_dgemm", _i32, [_vp, _i32, C.c_char, C.c_char, _i64, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d,
                         _vp, _i64]),
    ("lra_snorm", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _i32, _P(lra_opts), _P(lra_rand),
                         _P(_d)]),
    ("lra_snormdiff", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _vp, _i64, _P(lra_opts),
                             _P(lra_rand), _P(_d)]),
    ("lra_snormdiff_id", _i32, [_vp, _i32, _ch, _i64, _i64, _vp, _i64, _P(lra_id), _P(lra_opts),
                                _P(lra_rand), _P(_d)]),
    ("lra_snormdiff_psvd", _i32, [_vp, _i32, _i64, _i64, _vp, _i64, _P(lra_psvd), _P(lra_opts),
                                  _P(lra_rand), _P(_d)]),
    ("lra_sketchfact_linop", _i32, [_vp, _ch, _ch, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_P(lra_pqr))]),
    ("lra_idfact_linop", _i32, [_vp, _ch, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_P(lra_id))]),
    ("lra_pqrfact_linop", _i32, [_vp, _ch, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_P(lra_pqr))]),
    ("lra_prange_linop", _i32, [_vp, _ch, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_P(lra_pqr))]),
    ("lra_psvdfact_linop", _i32, [_vp, _P(lra_linop), _P(lra_opts), _P(lra_rand), _i32, _P(_P(lra_psvd))]),
    ("lra_pheigfact_linop", _i32, [_vp, _P(lra_linop), _P(lra_opts), _P(lra_rand), _i32, _P(_P(lra_pheig))]),
    ("lra_curfact_linop", _i32, [_vp, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_P(lra_cur))]),
    ("lra_snorm_linop", _i32, [_vp, _P(lra_linop), _P(lra_opts), _P(lra_rand), _P(_d)]),
    ("lra_idfact_batched", _i32, [_vp, _i32, _i64, _P(lra_matdesc), _P(lra_opts), _P(lra_rand),
                                  _P(_P(lra_id))]),
    ("lra_server_create", _i32, [_i32, _i32, _i64, _P(_vp)]),
    ("lra_server_submit", _i32, [_vp, _P(lra_request), _P(C.c_uint64)]),
    ("lra_server_poll", _i32, [_vp, C.c_uint64, _i64, _P(lra_result)]),
    ("lra_server_get_stats", _i32, [_vp, _P(lra_server_stats)]),
    ("lra_server_destroy", None, [_vp]),
    ("lra_id_free", None, [_P(lra_id)]),
    ("lra_pqr_free", None, [_P(lra_pqr)]),
    ("lra_psvd_free", None, [_P(lra_psvd)]),
    ("lra_pheig_free", None, [_P(lra_pheig)]),
    ("lra_cur_free", None, [_P(lra_cur)]),
]

_LIB = None


def load(path: str | None = None):
    """Load liblra.so and bind every entry point; raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"liblra.so not found at {p}: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib
