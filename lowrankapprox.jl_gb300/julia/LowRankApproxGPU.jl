#= LowRankApproxGPU.jl -- LowRankApprox.jl's sketch-then-factor entry points on
   liblra (GB300, sm_103a) through `ccall`.

   Drop-in for the path idfact / pqrfact / psvdfact / pheigfact / curfact /
   sketch / sketchfact / snorm / snormdiff of LowRankApprox.jl: same names,
   same LRAOptions fields, same result types (PartialQR, IDPackedV,
   PartialSVD, PartialHermitianEigen, CURPackedU) -- the LowRankApprox
   package provides the types and their algebra; this module only replaces
   the factorization routines.  Every call lands in one C entry point of
   include/lra.h; there is no Julia-side numerics and no CPU fallback.

   Usage:
     using LowRankApprox, LowRankApproxGPU
     V = LowRankApproxGPU.idfact(A; rtol=1e-10, precision=:mixed)
=#
module LowRankApproxGPU

using LinearAlgebra
import LowRankApprox
using LowRankApprox: LRAOptions, IDPackedV, PartialQR, PartialSVD, PartialHermitianEigen, CURPackedU,
                     HermitianCURPackedU, PartialQRFactors

const liblra = get(ENV, "LIBLRA", joinpath(@__DIR__, "..", "lowrankapprox", "liblra.so"))

# ---- C structs (include/lra.h) ------------------------------------------------
struct lra_opts
  atol::Float64; maxdet_niter::Int64; maxdet_tol::Float64; nb::Int64; pheig_orthtol::Float64
  pqrfact_retval::Int32; sketch::Int32; rank::Int64; rtol::Float64; sketch_randn_niter::Int64
  sketchfact_adap::Int32; verb::Int32
  randn_samp::NTuple{2,Int64}; srft_samp::NTuple{2,Int64}; sub_samp::NTuple{2,Int64}
  snorm_niter::Int64; precision::Int32; check_finite::Int32; seed::UInt64
end
struct lra_rand;  gauss::Ptr{Float64}; gauss_len::Int64; ints::Ptr{Int64}; ints_len::Int64; end
struct lra_id;    dtype::Int32; nsteps::Int32; k::Int64; n::Int64; sk::Ptr{Int64}; rd::Ptr{Int64}; T::Ptr{Cvoid}; end
struct lra_pqr;   dtype::Int32; retval::Int32; m::Int64; n::Int64; k::Int64; p::Ptr{Int64}
                  Q::Ptr{Cvoid}; R::Ptr{Cvoid}; T::Ptr{Cvoid}; end
struct lra_psvd;  dtype::Int32; pad::Int32; m::Int64; n::Int64; k::Int64; U::Ptr{Cvoid}; S::Ptr{Cvoid}; Vt::Ptr{Cvoid}; end
struct lra_pheig; dtype::Int32; pad::Int32; n::Int64; k::Int64; values::Ptr{Cvoid}; vectors::Ptr{Cvoid}; end
struct lra_cur;   kind::Int32; pad::Int32; kr::Int64; kc::Int64; rows::Ptr{Int64}; cols::Ptr{Int64}; end
struct lra_request
  kind::Int32; dtype::Int32; trans::UInt8; pad::NTuple{7,UInt8}
  m::Int64; n::Int64; lda::Int64; A::Ptr{Cvoid}; opts::lra_opts; rand::Ptr{lra_rand}
end
struct lra_result
  kind::Int32; status::Int32; id::Ptr{lra_id}; psvd::Ptr{lra_psvd}
  queue_ms::Float64; run_ms::Float64; total_ms::Float64; slot::Int32; pad::Int32; error::NTuple{160,UInt8}
end
struct lra_server_stats
  submitted::Int64; completed::Int64; rejected::Int64; in_flight::Int64; queued::Int64
  p50_ms::Float64; p99_ms::Float64; mean_ms::Float64; matrices_per_s::Float64; hbm_budget::Int64; hbm_in_use::Int64
end

const SKETCH = Dict(:none => 0, :randn => 1, :sprn => 2, :srft => 3, :sub => 4, :subs => 4)
dtype(::Type{Float64}) = Int32(1)
dtype(::Type{Float32}) = Int32(0)
dtype(::Type{ComplexF32}) = Int32(2)
dtype(::Type{ComplexF64}) = Int32(3)
# the element types the reference's tests sweep (test/id.jl:6: Float32, Float64, ComplexF32, ComplexF64)
const LRAType = Union{Float32,Float64,ComplexF32,ComplexF64}

# an affine n -> a n + b, read off the option's function (src/LowRankApprox.jl:109-111)
function affine(f)
  b = f(0); a = f(1) - b
  all(f(n) == a*n + b for n in (2, 7, 32, 1000)) || throw(ArgumentError("oversampling must be affine"))
  (Int64(a), Int64(b))
end

function c_opts(o::LRAOptions; precision::Symbol=:native, seed::Integer=0x4c5241)
  rv = lowercase(o.pqrfact_retval)
  bits = Int32((occursin('q', rv) ? 1 : 0) | (occursin('r', rv) ? 2 : 0) | (occursin('t', rv) ? 4 : 0))
  lra_opts(o.atol, o.maxdet_niter, o.maxdet_tol, o.nb, o.pheig_orthtol, bits, SKETCH[o.sketch], o.rank, o.rtol,
           o.sketch_randn_niter, Int32(o.sketchfact_adap), Int32(o.verb), affine(o.sketchfact_randn_samp),
           affine(o.sketchfact_srft_samp), affine(o.sketchfact_sub_samp), o.snorm_niter,
           Int32(precision == :mixed), Int32(1), UInt64(seed))
end

# ---- context and errors ---------------------------------------------------------
mutable struct Context
  h::Ptr{Cvoid}
  function Context(device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:lra_ctx_create, liblra), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r)
    st == 0 || error("lra_ctx_create: ", unsafe_string(ccall((:lra_status_string, liblra), Cstring, (Cint,), st)))
    c = new(r[])
    finalizer(c -> ccall((:lra_ctx_destroy, liblra), Cvoid, (Ptr{Cvoid},), c.h), c)
  end
end
const CTX = Ref{Context}()
ctx() = (isassigned(CTX) || (CTX[] = Context()); CTX[])

function check(st::Cint, c::Context)
  st == 0 && return
  msg = unsafe_string(ccall((:lra_last_error, liblra), Cstring, (Ptr{Cvoid},), c.h))
  st == 1 && throw(ArgumentError(msg))               # LRA_EINVAL  (chkopts!, src/LowRankApprox.jl:133-148)
  st == 2 && throw(DimensionMismatch(msg))           # LRA_EDIM
  st == 9 && error("matrix must be Hermitian")       # LRA_ENOTHERM (src/pheig.jl:279)
  error("liblra: ", msg, " (status ", st, ")")
end

opts_of(::Type{T}, opts, kw) where T = isempty(kw) ? (opts === nothing ? LRAOptions(T) : opts) :
                                      copy(opts === nothing ? LRAOptions(T) : opts; kw...)

take(ptr::Ptr{T}, n) where T = n == 0 ? T[] : copy(unsafe_wrap(Array, ptr, n))
takem(ptr::Ptr{Cvoid}, ::Type{T}, m, n) where T = (m*n == 0 ? zeros(T, m, n) :
                                                   copy(unsafe_wrap(Array, Ptr{T}(ptr), (m, n))))

# ---- entry points --------------------------------------------------------------
function pqr_result(ptr::Ptr{lra_pqr}, ::Type{T}) where T
  r = unsafe_load(ptr)
  try
    p = take(r.p, r.n)
    Q = (r.retval & 1) != 0 ? takem(r.Q, T, r.m, r.k) : nothing
    R = (r.retval & 2) != 0 ? takem(r.R, T, r.k, r.n) : nothing
    Tm = (r.retval & 4) != 0 ? takem(r.T, T, r.k, r.n - r.k) : nothing
    Q !== nothing && R !== nothing && Tm === nothing && return PartialQR(Q, R, p)
    PartialQRFactors(Q, R, p, r.k, Tm)
  finally
    ccall((:lra_pqr_free, liblra), Cvoid, (Ptr{lra_pqr},), ptr)
  end
end
function range_result(ptr::Ptr{lra_pqr}, ::Type{T}) where T
  r = unsafe_load(ptr)
  try
    takem(r.Q, T, r.m, r.k)
  finally
    ccall((:lra_pqr_free, liblra), Cvoid, (Ptr{lra_pqr},), ptr)
  end
end
"idfact(trans, A[, opts]; precision=:native) -- src/id.jl:434-450 on the GPU."
function idfact(trans::Symbol, A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                precision::Symbol=:native, kw...) where T<:LRAType
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_id}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_idfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Cchar, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_id}}),
             c.h, dtype(T), trans == :n ? 'n' : 'c', size(A,1), size(A,2), A, stride(A,2), co, C_NULL, out)
  check(st, c)
  r = unsafe_load(out[])
  try
    IDPackedV(take(r.sk, r.k), take(r.rd, r.n - r.k), takem(r.T, T, r.k, r.n - r.k))
  finally
    ccall((:lra_id_free, liblra), Cvoid, (Ptr{lra_id},), out[])
  end
end
idfact(A::StridedMatrix, args...; kw...) = idfact(:n, A, args...; kw...)

"pqrfact(trans, A[, opts]) -- src/pqr.jl:290-307 on the GPU."
function pqrfact(trans::Symbol, A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                 precision::Symbol=:native, kw...) where T<:LRAType
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pqr}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_pqrfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Cchar, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_pqr}}),
             c.h, dtype(T), trans == :n ? 'n' : 'c', size(A,1), size(A,2), A, stride(A,2), co, C_NULL, out)
  check(st, c)
  pqr_result(out[], T)
end
pqrfact(A::StridedMatrix, args...; kw...) = pqrfact(:n, A, args...; kw...)

"prange(trans, A[, opts]) -- src/prange.jl:14-61 on the GPU: an orthonormal basis of the range (:n, :c, :b)."
function prange(trans::Symbol, A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                precision::Symbol=:native, kw...) where T<:LRAType
  trans in (:n, :c, :b) || throw(ArgumentError("trans"))
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pqr}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_prange, liblra), Cint,
             (Ptr{Cvoid}, Cint, Cchar, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_pqr}}),
             c.h, dtype(T), trans == :n ? 'n' : (trans == :c ? 'c' : 'b'), size(A,1), size(A,2), A, stride(A,2), co,
             C_NULL, out)
  check(st, c)
  range_result(out[], T)
end
prange(A::StridedMatrix, args...; kw...) = prange(:n, A, args...; kw...)

function _psvd(A::StridedMatrix{T}, opts, vals::Bool; precision::Symbol=:native, kw...) where T
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_psvd}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_psvdfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Cint, Ref{Ptr{lra_psvd}}),
             c.h, dtype(T), size(A,1), size(A,2), A, stride(A,2), co, C_NULL, Cint(vals), out)
  check(st, c)
  r = unsafe_load(out[])
  try
    S = take(Ptr{real(T)}(r.S), r.k)
    vals && return S
    PartialSVD(takem(r.U, T, r.m, r.k), S, takem(r.Vt, T, r.k, r.n))
  finally
    ccall((:lra_psvd_free, liblra), Cvoid, (Ptr{lra_psvd},), out[])
  end
end
"psvdfact(A[, opts]) -- src/psvd.jl:238-272 on the GPU."
psvdfact(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; kw...) where T = _psvd(A, opts, false; kw...)
"psvdvals(A[, opts]) -- src/psvd.jl:274-290 on the GPU."
psvdvals(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; kw...) where T = _psvd(A, opts, true; kw...)
psvd(A, args...; kw...) = (F = psvdfact(A, args...; kw...); (F.U, F.S, F.Vt'))

function _pheig(A::StridedMatrix{T}, opts, vals::Bool; precision::Symbol=:native, kw...) where T
  LinearAlgebra.checksquare(A)
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pheig}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_pheigfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Cint, Ref{Ptr{lra_pheig}}),
             c.h, dtype(T), size(A,1), A, stride(A,2), co, C_NULL, Cint(vals), out)
  check(st, c)
  r = unsafe_load(out[])
  try
    w = take(Ptr{real(T)}(r.values), r.k)
    vals && return w
    PartialHermitianEigen(w, takem(r.vectors, T, r.n, r.k))
  finally
    ccall((:lra_pheig_free, liblra), Cvoid, (Ptr{lra_pheig},), out[])
  end
end
"pheigfact(A[, opts]) -- src/pheig.jl:276-296 on the GPU."
pheigfact(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; kw...) where T = _pheig(A, opts, false; kw...)
pheigvals(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; kw...) where T = _pheig(A, opts, true; kw...)
pheig(A, args...; kw...) = (F = pheigfact(A, args...; kw...); (F.values, F.vectors))

"curfact(A[, opts]) -- src/cur.jl:532-564 on the GPU."
function curfact(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; precision::Symbol=:native,
                 kw...) where T<:LRAType
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_cur}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_curfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_cur}}),
             c.h, dtype(T), size(A,1), size(A,2), A, stride(A,2), co, C_NULL, out)
  check(st, c)
  r = unsafe_load(out[])
  try
    rows = take(r.rows, r.kr); cols = take(r.cols, r.kc)
    r.kind == 1 ? HermitianCURPackedU(cols) : CURPackedU(rows, cols)
  finally
    ccall((:lra_cur_free, liblra), Cvoid, (Ptr{lra_cur},), out[])
  end
end

"""CUR(A, U) -- src/cur.jl:85-115: C = A[:, cols], R = A[rows, :] and the
pseudo-inverse of A[rows, cols] computed on the GPU (lra_cur_middle).  The
reference's own CUR / HermitianCUR types are built from the three parts."""
function CUR(A::StridedMatrix{T}, U::Union{CURPackedU,HermitianCURPackedU}) where T<:LRAType
  rows = Int64.(U[:rows]); cols = Int64.(U[:cols])
  length(rows) == length(cols) || throw(DimensionMismatch("rows and cols differ in length"))
  c = ctx(); out = Ref{Ptr{lra_psvd}}(C_NULL); k = length(cols)
  st = ccall((:lra_cur_middle, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Int64, Ptr{T}, Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ref{Ptr{lra_psvd}}),
             c.h, dtype(T), size(A,1), size(A,2), A, stride(A,2), k, rows, cols, out)
  check(st, c)
  p = unsafe_load(out[])
  try
    W = PartialSVD(takem(p.U, T, p.m, p.k), take(Ptr{real(T)}(p.S), p.k), takem(p.Vt, T, p.k, p.n))
    U isa HermitianCURPackedU ? LowRankApprox.HermitianCUR(cols, A[:, cols], W) :
                                LowRankApprox.CUR(rows, cols, A[:, cols], W, A[rows, :])
  finally
    ccall((:lra_psvd_free, liblra), Cvoid, (Ptr{lra_psvd},), out[])
  end
end

"snorm(A[, opts]) -- src/snorm.jl:14-45 on the GPU."
function snorm(A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing; kw...) where T<:LRAType
  o = opts_of(T, opts, kw); c = ctx(); s = Ref{Float64}(0)
  co = Ref(c_opts(o))
  st = ccall((:lra_snorm, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Int64, Ptr{T}, Int64, Cint, Ref{lra_opts}, Ptr{lra_rand}, Ref{Float64}),
             c.h, dtype(T), size(A,1), size(A,2), A, stride(A,2), Cint(-1), co, C_NULL, s)
  check(st, c)
  s[]
end

"snormdiff(A, B[, opts]) -- src/snorm.jl:50-53 on the GPU."
function snormdiff(A::StridedMatrix{T}, B::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                   kw...) where T<:LRAType
  o = opts_of(T, opts, kw); c = ctx(); s = Ref{Float64}(0)
  co = Ref(c_opts(o))
  st = ccall((:lra_snormdiff, liblra), Cint,
             (Ptr{Cvoid}, Cint, Int64, Int64, Ptr{T}, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand}, Ref{Float64}),
             c.h, dtype(T), size(A,1), size(A,2), A, stride(A,2), B, stride(B,2), co, C_NULL, s)
  check(st, c)
  s[]
end

"sketch(side, trans, A, order[, opts]) -- src/sketch.jl:35-50 on the GPU."
function sketch(side::Symbol, trans::Symbol, A::StridedMatrix{T}, order::Integer,
                opts::Union{LRAOptions,Nothing}=nothing; kw...) where T<:LRAType
  side in (:left, :right) && trans in (:n, :c) || throw(ArgumentError("side / trans"))   # src/sketch.jl:76-79
  o = opts_of(T, opts, kw); c = ctx(); co = Ref(c_opts(o))
  mo, no = trans == :n ? size(A) : reverse(size(A))
  B = side == :left ? Matrix{T}(undef, order, no) : Matrix{T}(undef, mo, order)
  st = ccall((:lra_sketch, liblra), Cint,
             (Ptr{Cvoid}, Cint, Cchar, Cchar, Int64, Int64, Ptr{T}, Int64, Int64, Ref{lra_opts}, Ptr{lra_rand},
              Ptr{T}, Int64),
             c.h, dtype(T), side == :left ? 'l' : 'r', trans == :n ? 'n' : 'c', size(A,1), size(A,2), A,
             stride(A,2), order, co, C_NULL, B, max(size(B,1), 1))
  check(st, c)
  B
end
sketch(A::StridedMatrix, order::Integer, args...; kw...) = sketch(:left, :n, A, order, args...; kw...)

"sketchfact(side, trans, A[, opts]) -- src/sketch.jl:52-66 on the GPU (PartialQRFactors of the sketch)."
function sketchfact(side::Symbol, trans::Symbol, A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                    precision::Symbol=:native, kw...) where T<:LRAType
  side in (:left, :right) && trans in (:n, :c) || throw(ArgumentError("side / trans"))   # src/sketch.jl:80-83
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pqr}}(C_NULL)
  co = Ref(c_opts(o; precision))
  st = ccall((:lra_sketchfact, liblra), Cint,
             (Ptr{Cvoid}, Cint, Cchar, Cchar, Int64, Int64, Ptr{T}, Int64, Ref{lra_opts}, Ptr{lra_rand},
              Ref{Ptr{lra_pqr}}),
             c.h, dtype(T), side == :left ? 'l' : 'r', trans == :n ? 'n' : 'c', size(A,1), size(A,2), A,
             stride(A,2), co, C_NULL, out)
  check(st, c)
  pqr_result(out[], T)
end
sketchfact(A::StridedMatrix, args...; kw...) = sketchfact(:left, :n, A, args...; kw...)

# ---- matrix-free operators (src/linop.jl:9-40) ------------------------------------
#= A LinearOperator / HermitianLinearOperator reaches the engine as a lra_linop
   whose matmat callback applies the operator's own mul! (src/linop.jl:105-110)
   to the engine's block of vectors: the block comes to the host, the Julia
   product runs there, and the result goes back to the device on the call's
   stream.  One callback serves every element type: `user` points at a Ref
   holding the operator, and the product dispatches on its type.  A product
   that throws makes the library call fail (LRA_ECUDA); the exception is
   rethrown here.  Real element types only, as the engine's operator entry
   points accept. =#
struct lra_linop; m::Int64; n::Int64; dtype::Int32; hermitian::Int32; matmat::Ptr{Cvoid}; user::Ptr{Cvoid}; end

const libcudart = get(ENV, "LIBCUDART", "libcudart.so")
const D2H, H2D = Cint(2), Cint(1)      # cudaMemcpyDeviceToHost / HostToDevice

cudacheck(e::Cint, what) = e == 0 || error(what, " failed with CUDA error ", e)
function copy2d!(dst, dpitch, src, spitch, width, height, kind, stream)
  cudacheck(ccall((:cudaMemcpy2DAsync, libcudart), Cint,
                  (Ptr{Cvoid}, Csize_t, Ptr{Cvoid}, Csize_t, Csize_t, Csize_t, Cint, Ptr{Cvoid}),
                  dst, dpitch, src, spitch, width, height, kind, stream), "cudaMemcpy2DAsync")
  cudacheck(ccall((:cudaStreamSynchronize, libcudart), Cint, (Ptr{Cvoid},), stream), "cudaStreamSynchronize")
end

mutable struct OpBox
  A::LowRankApprox.AbstractLinOp
  err::Any
end

function apply_op!(A::LowRankApprox.AbstractLinOp{T}, adj::Bool, ncols, X, ldx, Y, ldy, stream) where T
  m, n = size(A)
  rx, ry = adj ? (m, n) : (n, m)
  Xh = Matrix{T}(undef, rx, ncols); Yh = Matrix{T}(undef, ry, ncols)
  s = sizeof(T)
  copy2d!(pointer(Xh), rx*s, X, ldx*s, rx*s, ncols, D2H, stream)
  adj ? mul!(Yh, A', Xh) : mul!(Yh, A, Xh)
  copy2d!(Y, ldy*s, pointer(Yh), ry*s, ry*s, ncols, H2D, stream)
end

function matmat_cb(user::Ptr{Cvoid}, trans::Cchar, ncols::Int64, X::Ptr{Cvoid}, ldx::Int64, Y::Ptr{Cvoid},
                   ldy::Int64, stream::Ptr{Cvoid})::Cint
  box = unsafe_pointer_to_objref(user)::OpBox
  try
    ncols > 0 && apply_op!(box.A, trans != Cchar('n'), ncols, X, ldx, Y, ldy, stream)
    Cint(0)
  catch e
    box.err = e
    Cint(1)
  end
end

function with_op(f, A::LowRankApprox.AbstractLinOp{T}) where T<:Union{Float32,Float64}
  box = OpBox(A, nothing)
  cb = @cfunction(matmat_cb, Cint, (Ptr{Cvoid}, Cchar, Int64, Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64, Ptr{Cvoid}))
  m, n = size(A)
  L = Ref(lra_linop(m, n, dtype(T), Int32(A isa LowRankApprox.HermLinOp), cb, pointer_from_objref(box)))
  GC.@preserve box begin
    st, res = f(L)
    box.err === nothing || throw(box.err)
    st, res
  end
end

opfn(name) = Symbol("lra_", name, "_linop")

"idfact / pqrfact / prange / psvdfact / pheigfact / curfact / snorm of a LinearOperator (Gaussian sketch, src/LowRankApprox.jl:142-148)."
function idfact(trans::Symbol, A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
                kw...) where T<:Union{Float32,Float64}
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_id}}(C_NULL); co = Ref(c_opts(o))
  st, _ = with_op(A) do L
    (ccall((:lra_idfact_linop, liblra), Cint,
           (Ptr{Cvoid}, Cchar, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_id}}),
           c.h, trans == :n ? 'n' : 'c', L, co, C_NULL, out), nothing)
  end
  check(st, c)
  r = unsafe_load(out[])
  try
    IDPackedV(take(r.sk, r.k), take(r.rd, r.n - r.k), takem(r.T, T, r.k, r.n - r.k))
  finally
    ccall((:lra_id_free, liblra), Cvoid, (Ptr{lra_id},), out[])
  end
end
idfact(A::LowRankApprox.AbstractLinOp, args...; kw...) = idfact(:n, A, args...; kw...)

for (name, hastrans) in ((:pqrfact, true), (:prange, true))
  @eval function $name(trans::Symbol, A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
                       kw...) where T<:Union{Float32,Float64}
    o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pqr}}(C_NULL); co = Ref(c_opts(o))
    tc = trans == :n ? 'n' : (trans == :c ? 'c' : 'b')
    st, _ = with_op(A) do L
      (ccall(($(QuoteNode(opfn(name))), liblra), Cint,
             (Ptr{Cvoid}, Cchar, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_pqr}}),
             c.h, tc, L, co, C_NULL, out), nothing)
    end
    check(st, c)
    $(name == :prange ? :(range_result(out[], T)) : :(pqr_result(out[], T)))
  end
  @eval $name(A::LowRankApprox.AbstractLinOp, args...; kw...) = $name(:n, A, args...; kw...)
end

function psvdfact(A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
                  vals::Bool=false, kw...) where T<:Union{Float32,Float64}
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_psvd}}(C_NULL); co = Ref(c_opts(o))
  st, _ = with_op(A) do L
    (ccall((:lra_psvdfact_linop, liblra), Cint,
           (Ptr{Cvoid}, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Cint, Ref{Ptr{lra_psvd}}),
           c.h, L, co, C_NULL, Cint(vals), out), nothing)
  end
  check(st, c)
  r = unsafe_load(out[])
  try
    S = take(Ptr{T}(r.S), r.k)
    vals && return S
    PartialSVD(takem(r.U, T, r.m, r.k), S, takem(r.Vt, T, r.k, r.n))
  finally
    ccall((:lra_psvd_free, liblra), Cvoid, (Ptr{lra_psvd},), out[])
  end
end
psvdvals(A::LowRankApprox.AbstractLinOp, args...; kw...) = psvdfact(A, args...; vals=true, kw...)

function pheigfact(A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
                   vals::Bool=false, kw...) where T<:Union{Float32,Float64}
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_pheig}}(C_NULL); co = Ref(c_opts(o))
  st, _ = with_op(A) do L
    (ccall((:lra_pheigfact_linop, liblra), Cint,
           (Ptr{Cvoid}, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Cint, Ref{Ptr{lra_pheig}}),
           c.h, L, co, C_NULL, Cint(vals), out), nothing)
  end
  check(st, c)
  r = unsafe_load(out[])
  try
    w = take(Ptr{T}(r.values), r.k)
    vals && return w
    PartialHermitianEigen(w, takem(r.vectors, T, r.n, r.k))
  finally
    ccall((:lra_pheig_free, liblra), Cvoid, (Ptr{lra_pheig},), out[])
  end
end
pheigvals(A::LowRankApprox.AbstractLinOp, args...; kw...) = pheigfact(A, args...; vals=true, kw...)

function curfact(A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
                 kw...) where T<:Union{Float32,Float64}
  o = opts_of(T, opts, kw); c = ctx(); out = Ref{Ptr{lra_cur}}(C_NULL); co = Ref(c_opts(o))
  st, _ = with_op(A) do L
    (ccall((:lra_curfact_linop, liblra), Cint,
           (Ptr{Cvoid}, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Ref{Ptr{lra_cur}}),
           c.h, L, co, C_NULL, out), nothing)
  end
  check(st, c)
  r = unsafe_load(out[])
  try
    rows = take(r.rows, r.kr); cols = take(r.cols, r.kc)
    r.kind == 1 ? HermitianCURPackedU(cols) : CURPackedU(rows, cols)
  finally
    ccall((:lra_cur_free, liblra), Cvoid, (Ptr{lra_cur},), out[])
  end
end

function snorm(A::LowRankApprox.AbstractLinOp{T}, opts::Union{LRAOptions,Nothing}=nothing;
               kw...) where T<:Union{Float32,Float64}
  o = opts_of(T, opts, kw); c = ctx(); s = Ref{Float64}(0); co = Ref(c_opts(o))
  st, _ = with_op(A) do L
    (ccall((:lra_snorm_linop, liblra), Cint,
           (Ptr{Cvoid}, Ref{lra_linop}, Ref{lra_opts}, Ptr{lra_rand}, Ref{Float64}), c.h, L, co, C_NULL, s), nothing)
  end
  check(st, c)
  s[]
end

# ---- engine settings (no counterpart in LowRankApprox.jl) -------------------------
"The autotuned shape table in force on the default context, as text."
function tuning()
  c = ctx(); n = ccall((:lra_ctx_get_tuning, liblra), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), c.h, C_NULL, 0)
  buf = Vector{UInt8}(undef, n)
  ccall((:lra_ctx_get_tuning, liblra), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), c.h, buf, n)
  unsafe_string(pointer(buf))
end
"Override one tuning entry (\"tc_tile_n\", \"qr_seq_len\", \"srft_wide\") on the default context."
set_tuning!(key::AbstractString, index::Integer, value::Integer) =
  check(ccall((:lra_ctx_set_tuning, liblra), Cint, (Ptr{Cvoid}, Cstring, Int64, Int64), ctx().h, key, index, value), ctx())
"Limit of every bounded device-side wait, in ns (0 = the default 4 s); a wait that runs out fails its call."
set_wait_limit!(ns::Integer) =
  check(ccall((:lra_ctx_set_wait_limit, liblra), Cint, (Ptr{Cvoid}, Int64), ctx().h, ns), ctx())
"Self-test of the bounded waits: true when a barrier nothing completes timed out and the context stayed usable."
probe_wait() = ccall((:lra_ctx_probe_wait, liblra), Cint, (Ptr{Cvoid},), ctx().h) == 4   # LRA_ETIMEDOUT

"""gauss(n; seed, counter=0) -- the engine's Gaussian stream (Philox-4x32-10, Box-Muller,
rounded to the 1/32 lattice): the values a call on a fresh context draws for its
Gaussian sketches, so that a caller can reproduce them on the CPU."""
function gauss(n::Integer; seed::Integer=0x4c5241, counter::Integer=0)
  out = Vector{Float64}(undef, n)
  check(ccall((:lra_rand_gauss, liblra), Cint, (Ptr{Cvoid}, UInt64, UInt64, Int64, Ptr{Float64}),
              ctx().h, seed, counter, n, out), ctx())
  out
end

# ---- serving loop (lra_server_*; no counterpart in LowRankApprox.jl) ----------------
"""
    Server(; slots=8, hbm_budget=150 << 30, device=0)

Continuous batching of idfact / psvdfact requests on one GPU: `submit` returns
a ticket, `fetch(srv, t)` waits and returns the factorization.  Inputs stay
referenced by the server until their result is fetched.
"""
mutable struct Server
  h::Ptr{Cvoid}
  keep::Dict{UInt64,Any}
  function Server(; slots::Integer=8, hbm_budget::Integer=150 << 30, device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:lra_server_create, liblra), Cint, (Cint, Cint, Int64, Ref{Ptr{Cvoid}}), device, slots,
               hbm_budget, r)
    st == 0 || error("lra_server_create failed with status $st")
    s = new(r[], Dict{UInt64,Any}())
    finalizer(x -> ccall((:lra_server_destroy, liblra), Cvoid, (Ptr{Cvoid},), x.h), s)
  end
end

function submit(s::Server, kind::Symbol, A::StridedMatrix{T}, opts::Union{LRAOptions,Nothing}=nothing;
                precision::Symbol=:native, trans::Symbol=:n, kw...) where T<:Union{Float32,Float64}  # real only
  o = c_opts(opts_of(T, opts, kw); precision)
  req = lra_request(kind == :psvdfact ? 1 : 0, dtype(T), UInt8(trans == :n ? 'n' : 'c'), ntuple(_ -> 0x0, 7),
                    size(A,1), size(A,2), stride(A,2), Ptr{Cvoid}(pointer(A)), o, C_NULL)
  t = Ref{UInt64}(0)
  st = ccall((:lra_server_submit, liblra), Cint, (Ptr{Cvoid}, Ref{lra_request}, Ref{UInt64}), s.h, req, t)
  st == 0 || error("lra_server_submit failed with status $st")
  s.keep[t[]] = (A, T, kind)
  t[]
end

function Base.fetch(s::Server, t::UInt64)
  res = Ref{lra_result}()
  st = ccall((:lra_server_poll, liblra), Cint, (Ptr{Cvoid}, UInt64, Int64, Ref{lra_result}), s.h, t, -1, res)
  st == 0 || error("lra_server_poll failed with status $st")
  A, T, kind = pop!(s.keep, t)
  r = res[]
  r.status == 0 || error(unsafe_string(pointer(collect(r.error))))
  if kind == :psvdfact
    p = unsafe_load(r.psvd)
    try
      return PartialSVD(takem(p.U, T, p.m, p.k), take(Ptr{T}(p.S), p.k), takem(p.Vt, T, p.k, p.n))
    finally
      ccall((:lra_psvd_free, liblra), Cvoid, (Ptr{lra_psvd},), r.psvd)
    end
  else
    v = unsafe_load(r.id)
    try
      return IDPackedV(take(v.sk, v.k), take(v.rd, v.n - v.k), takem(v.T, T, v.k, v.n - v.k))
    finally
      ccall((:lra_id_free, liblra), Cvoid, (Ptr{lra_id},), r.id)
    end
  end
end

function stats(s::Server)
  r = Ref{lra_server_stats}()
  ccall((:lra_server_get_stats, liblra), Cint, (Ptr{Cvoid}, Ref{lra_server_stats}), s.h, r)
  r[]
end

end # module
