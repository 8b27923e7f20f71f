"""
    TNRKitGB300

Julia binding of the GB300 coarse-graining engine (`libtnr_gb300.so`, C ABI in
`include/tnr_gb300.h`).  It keeps TNRKit's user interface for the hot path:

    using TNRKit, TensorKit, TNRKitGB300
    T = classical_ising(ising_βc)
    scheme = GPU(BTRG(T))                       # tensors move to the GPU once
    data = run!(scheme, truncrank(16), maxiter(25))
    f = free_energy(data, ising_βc)

`GPU(scheme)` wraps a TNRKit `TRG`, `BTRG`, `HOTRG` or `HOTRG_3D` whose tensor is a
dense or abelian (Z_N) TensorMap; `run!`, `step!` and `finalize!` on the wrapper
call the library, which keeps the tensor resident on the device.  `run_batch!` runs
many wrapped schemes at once, and `Server` is the request loop that admits `run!`
requests by their HBM footprint:

    srv = Server(; precision = TNR_PREC_SPLIT)
    id = submit!(srv, BTRG(T), 32, 30)
    norms, latency_ms, queue_ms = result(srv, id)
"""
module TNRKitGB300

using TensorKit
import TNRKit
import TNRKit: run!, step!, finalize!, free_energy, maxiter, TNRScheme

export GPU, run_batch!, Server, submit!, result, TNR_PREC_F64, TNR_PREC_SPLIT

const libtnr = get(ENV, "TNR_GB300_LIB", joinpath(@__DIR__, "..", "libtnr_gb300.so"))

const TNR_TRG, TNR_BTRG, TNR_HOTRG, TNR_HOTRG_3D = 1, 2, 3, 4
const TNR_PREC_F64, TNR_PREC_SPLIT = 0, 1

# mirrors `tnr_options` (include/tnr_gb300.h)
struct Options
    precision::Cint
    btrg_k::Cdouble
    symmetry_n::Cint
    leg_charges::Ptr{Int32}
    seed::UInt64
    stream::Ptr{Cvoid}
end

struct TNRError <: Exception
    status::Int
    msg::String
end

function lasterror(h::Ptr{Cvoid})
    buf = Vector{UInt8}(undef, 1024)
    ccall((:tnr_last_error, libtnr), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf))
    return unsafe_string(pointer(buf))
end

check(st, h = C_NULL) = st == 0 || throw(TNRError(st, lasterror(h)))

scheme_kind(scheme) = scheme isa TNRKit.TRG ? TNR_TRG : scheme isa TNRKit.BTRG ? TNR_BTRG :
    scheme isa TNRKit.HOTRG ? TNR_HOTRG : scheme isa TNRKit.HOTRG_3D ? TNR_HOTRG_3D :
    throw(ArgumentError("scheme $(typeof(scheme)) has no GPU path"))

function dense_tensor(scheme)
    arr = convert(Array, scheme.T)                     # dense column-major T[i1, i2, ...]
    eltype(arr) <: Real || throw(ArgumentError("the GPU path takes real tensors"))
    return Array{Float64}(arr)
end

btrg_k(scheme) = scheme isa TNRKit.BTRG ? scheme.k : -0.5

mutable struct GPU{S <: TNRScheme} <: TNRScheme{Float64, Any}
    scheme::S
    handle::Ptr{Cvoid}
    function GPU(scheme::S; precision = TNR_PREC_F64, seed = 0) where {S <: TNRScheme}
        kind = scheme_kind(scheme)
        arr = dense_tensor(scheme)
        dims = Int64[size(arr)...]
        k = btrg_k(scheme)
        opts = Ref(Options(precision, k, 1, Ptr{Int32}(C_NULL), UInt64(seed), C_NULL))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:tnr_create, libtnr), Cint,
            (Ptr{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Ref{Options}),
            h, kind, length(dims), dims, arr, opts)
        check(st)
        g = new{S}(scheme, h[])
        finalizer(x -> ccall((:tnr_destroy, libtnr), Cint, (Ptr{Cvoid},), x.handle), g)
        return g
    end
end

function step!(g::GPU, trunc::TensorKit.MatrixAlgebraKit.TruncationByOrder)
    check(ccall((:tnr_step, libtnr), Cint, (Ptr{Cvoid}, Cint), g.handle, trunc.howmany), g.handle)
    return g
end

function finalize!(g::GPU)
    n = Ref{Float64}(0)
    check(ccall((:tnr_finalize, libtnr), Cint, (Ptr{Cvoid}, Ref{Float64}), g.handle, n), g.handle)
    return n[]
end

# run!(scheme, truncrank(chi), maxiter(n); finalize_beginning) with the default Finalizer
function run!(g::GPU, trunc, crit::maxiter; finalize_beginning = true, verbosity = 1)
    cap = max(crit.n, 1) + 1
    out = Vector{Float64}(undef, cap)
    n = Ref{Csize_t}(0)
    check(ccall((:tnr_run, libtnr), Cint,
        (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Float64}, Csize_t, Ref{Csize_t}),
        g.handle, trunc.howmany, crit.n, finalize_beginning, out, cap, n), g.handle)
    return out[1:n[]]
end

"""
    run_batch!(gs, chis, maxiters; finalize_beginning = true)

`run!` on many wrapped schemes at once (`tnr_run_batch`); returns one norm vector per
scheme.  Fresh TRG/BTRG schemes with equal kind, precision, k, legs, χ and maxiter step
together in lockstep (one batched GEMM per contraction, one CTA per member in the small
solvers); the others run concurrently, one stream each.
"""
function run_batch!(gs::AbstractVector{<:GPU}, chis::AbstractVector{<:Integer},
                    maxiters::AbstractVector{<:Integer}; finalize_beginning = true)
    n = length(gs)
    (length(chis) == n && length(maxiters) == n) || throw(ArgumentError("one χ and one maxiter per scheme"))
    stride = maximum(max.(maxiters, 1)) + 1
    norms = Vector{Float64}(undef, n * stride)
    counts = Vector{Csize_t}(undef, n)
    hs = Ptr{Cvoid}[g.handle for g in gs]
    check(ccall((:tnr_run_batch, libtnr), Cint,
        (Ptr{Ptr{Cvoid}}, Cint, Ptr{Cint}, Ptr{Cint}, Cint, Ptr{Float64}, Csize_t, Ptr{Csize_t}, Ptr{Float64},
         Ptr{Float64}),
        hs, n, Cint.(chis), Cint.(maxiters), finalize_beginning, norms, stride, counts, C_NULL, C_NULL))
    return [norms[(i - 1) * stride + 1:(i - 1) * stride + counts[i]] for i in 1:n]
end

"""
    Server(; hbm_budget_bytes = 200 * 2^30, max_active = 48, precision = TNR_PREC_SPLIT)

The `run!` request loop (`tnr_server_*`): a request is admitted when a slot is free and
its estimated HBM footprint fits the unused budget; admitted requests stay resident and
iterate concurrently, one CUDA stream each, and later arrivals are admitted as slots and
memory free up.  A request that can never fit is refused at `submit!`.
"""
mutable struct Server
    ptr::Ptr{Cvoid}
    function Server(; hbm_budget_bytes = 200 * 2^30, max_active = 48, precision = TNR_PREC_SPLIT)
        p = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:tnr_server_create, libtnr), Cint, (Ptr{Ptr{Cvoid}}, Csize_t, Cint, Cint),
            p, hbm_budget_bytes, max_active, precision))
        s = new(p[])
        finalizer(x -> ccall((:tnr_server_destroy, libtnr), Cint, (Ptr{Cvoid},), x.ptr), s)
        return s
    end
end

"""submit!(srv, scheme, χ, maxiter) -> request id (`run!(scheme, truncrank(χ), maxiter(maxiter))`)"""
function submit!(s::Server, scheme::TNRScheme, chi::Integer, maxiter::Integer)
    arr = dense_tensor(scheme)
    dims = Int64[size(arr)...]
    id = Ref{UInt64}(0)
    check(ccall((:tnr_server_submit, libtnr), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Cint, Cint, Cdouble, Ref{UInt64}),
        s.ptr, scheme_kind(scheme), length(dims), dims, arr, chi, maxiter, btrg_k(scheme), id))
    return id[]
end

"""result(srv, id) -> (norms, latency_ms, queue_ms); blocks until the request finishes"""
function result(s::Server, id::UInt64; cap = 4096)
    done = Ref{Cint}(0)
    n = Ref{Csize_t}(0)
    lat = Ref{Cdouble}(0)
    queue = Ref{Cdouble}(0)
    norms = Vector{Float64}(undef, cap)
    check(ccall((:tnr_server_poll, libtnr), Cint,
        (Ptr{Cvoid}, UInt64, Cint, Ref{Cint}, Ptr{Float64}, Csize_t, Ref{Csize_t}, Ref{Cdouble}, Ref{Cdouble}),
        s.ptr, id, 1, done, norms, cap, n, lat, queue))
    return norms[1:n[]], lat[], queue[]
end

end # module
