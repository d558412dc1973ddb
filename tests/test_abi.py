"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/lra.h declares, the ctypes structs match the C layout, and the
option defaults / validation mirror LRAOptions (src/LowRankApprox.jl:96-148)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "lra.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lra_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    import lowrankapprox._ffi as F
    if not os.path.exists(F.LIB_PATH):
        import __graft_entry__ as g
        g.build()
    return F.load()


def test_exports_every_declared_symbol(lib):
    import lowrankapprox._ffi as F
    syms = header_symbols()
    assert len(syms) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", F.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lra_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    bound = {name for name, _, _ in F.SIGNATURES}
    assert set(syms) <= bound | {"lra_geqp3_adap_noalloc"}


def test_struct_layout_matches_header(tmp_path):
    import lowrankapprox._ffi as F
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lra.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(lra_opts),'
                   'sizeof(lra_rand), sizeof(lra_id), sizeof(lra_pqr), sizeof(lra_psvd), sizeof(lra_pheig),'
                   'sizeof(lra_cur), sizeof(lra_matdesc), offsetof(lra_opts, seed), sizeof(lra_request),'
                   'offsetof(lra_request, opts), offsetof(lra_request, rand), sizeof(lra_result),'
                   'sizeof(lra_server_stats)); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = list(map(int, subprocess.check_output([str(exe)]).split()))
    want = [ctypes.sizeof(c) for c in (F.lra_opts, F.lra_rand, F.lra_id, F.lra_pqr, F.lra_psvd, F.lra_pheig,
                                       F.lra_cur, F.lra_matdesc)] + [F.lra_opts.seed.offset] + \
        [ctypes.sizeof(F.lra_request), F.lra_request.opts.offset, F.lra_request.rand.offset,
         ctypes.sizeof(F.lra_result), ctypes.sizeof(F.lra_server_stats)]
    assert got == want


@pytest.mark.parametrize("dtype,eps", [(1, np.finfo(np.float64).eps), (0, np.finfo(np.float32).eps)])
def test_opts_defaults(lib, dtype, eps):
    import lowrankapprox._ffi as F
    o = F.lra_opts()
    assert lib.lra_opts_init(ctypes.byref(o), dtype) == 0
    assert o.nb == 32 and o.rank == -1 and o.atol == 0 and o.maxdet_tol == -1 and o.maxdet_niter == -1
    assert o.rtol == pytest.approx(5 * eps) and o.pheig_orthtol == pytest.approx(np.sqrt(eps))
    assert o.sketch == F.SKETCH["randn"] and o.sketch_randn_niter == 0 and o.sketchfact_adap == 1
    assert list(o.sketchfact_randn_samp) == [1, 8] and list(o.sketchfact_sub_samp) == [4, 8]
    assert o.snorm_niter == 32 and o.pqrfact_retval == F.RET_Q | F.RET_R
    # python mirror agrees
    import lowrankapprox as L
    p = L.LRAOptions(np.float64 if dtype == 1 else np.float32).to_c()
    assert p.rtol == o.rtol and p.nb == o.nb and p.pqrfact_retval == o.pqrfact_retval


@pytest.mark.parametrize("field,value", [("atol", -1.0), ("nb", 0), ("rtol", -1e-3), ("pheig_orthtol", -1.0),
                                         ("sketch", 9), ("precision", 5)])
def test_chkopts_rejects(lib, field, value):
    import lowrankapprox._ffi as F
    o = F.lra_opts()
    lib.lra_opts_init(ctypes.byref(o), 1)
    assert lib.lra_chkopts(ctypes.byref(o)) == 0
    setattr(o, field, value)
    assert lib.lra_chkopts(ctypes.byref(o)) == F.LRA_EINVAL


def test_status_strings(lib):
    assert lib.lra_status_string(0) == b"ok"
    assert lib.lra_status_string(9) == b"matrix must be Hermitian"


def test_python_options_mirror():
    import lowrankapprox as L
    o = L.LRAOptions(sketch="subs", rank=5)   # the :subs spelling means :sub
    assert o.sketch == "sub" and o.rank == 5
    o2 = o.copy(rtol=1e-3)
    assert o2.rtol == 1e-3 and o.rtol != 1e-3
    with pytest.raises(ValueError):
        L.LRAOptions(bogus=1)


def test_python_argument_checks_before_the_device():
    # prange_chktrans (src/prange.jl:79-80) and CUR's row / column count are
    # checked on the host, before any context or device work
    import lowrankapprox as L
    A = np.zeros((4, 4))
    with pytest.raises(L.ArgumentError):
        L.prange("x", A)
    with pytest.raises(L.DimensionMismatch):
        L.CUR(A, L.CURPackedU(np.array([1, 2]), np.array([1])))


def test_tuning_table_syntax():
    """The committed tuning table (written by lowrankapprox/autotune.py)
    holds only keys and values the library accepts."""
    path = os.path.join(ROOT, "lowrankapprox.jl_gb300", "lowrankapprox", "tuning_gb300.txt")
    if not os.path.exists(path):
        pytest.skip("no tuning table committed")
    seen = set()
    for line in open(path):
        line = line.split("#", 1)[0].split()
        if not line:
            continue
        key = line[0]
        seen.add(key)
        if key == "tc_tile_n":
            assert line[1] in ("f32", "f64") and 0 <= int(line[2]) < 16 and int(line[3]) in (32, 64, 96)
        elif key == "qr_seq_len":
            assert 0 <= int(line[1]) <= 4096
        elif key == "srft_wide":
            assert 0 <= int(line[1]) <= 10 and int(line[2]) in (0, 1)
        else:
            raise AssertionError(f"unknown key {key}")
    assert {"tc_tile_n", "qr_seq_len", "srft_wide"} <= seen


def test_julia_shim_binds_exported_symbols(lib):
    """The Julia binding (julia/LowRankApproxGPU.jl) ccalls only entry points
    that the header declares and the library exports, and its mirrors of the
    header's structs list the same fields in the same order."""
    jl = open(os.path.join(ROOT, "lowrankapprox.jl_gb300", "julia", "LowRankApproxGPU.jl")).read()
    called = set(re.findall(r"\(:(lra_\w+), liblra\)", jl))
    called |= {f"lra_{n}_linop" for n in re.findall(r"\(:(pqrfact|prange), true\)", jl)}
    assert len(called) >= 30
    declared = set(header_symbols())
    assert called <= declared, sorted(called - declared)
    # field widths in order: the layout ccall sees
    csize = {"double": 8, "int64_t": 8, "uint64_t": 8, "int32_t": 4, "lra_matmat_fn": 8}
    hdr = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "lra.h")).read(), flags=re.S)
    for name in ("lra_opts", "lra_rand", "lra_id", "lra_pqr", "lra_psvd", "lra_pheig", "lra_cur", "lra_linop"):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), hdr, re.S).group(1)
        cw = []
        for decl in filter(str.strip, body.split(";")):
            typ, names = re.match(r"\s*(?:const\s+)?(\w+)\s*(.*)", decl).groups()
            for f in names.split(","):
                arr = re.search(r"\[(\d+)\]", f)
                w = 8 if "*" in f else csize[typ]
                cw.append(w * (int(arr.group(1)) if arr else 1))
        m = re.search(r"struct %s\b(.*?)\bend\b" % name, jl, re.S)
        jw = []
        for t in re.findall(r"\w+::([\w{},]+)", m.group(1)):
            tup = re.match(r"NTuple\{(\d+),(\w+)\}", t)
            base = tup.group(2) if tup else t
            w = 8 if base.startswith("Ptr") else {"Float64": 8, "Int64": 8, "UInt64": 8, "Int32": 4}[base]
            jw.append(w * (int(tup.group(1)) if tup else 1))
        assert jw == cw, (name, jw, cw)
