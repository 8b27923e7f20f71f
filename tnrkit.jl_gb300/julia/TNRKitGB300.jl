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
call the library, which keeps the tensor resident on the device.
"""
module TNRKitGB300

using TensorKit
import TNRKit
import TNRKit: run!, step!, finalize!, free_energy, maxiter, TNRScheme

export GPU

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

mutable struct GPU{S <: TNRScheme} <: TNRScheme{Float64, Any}
    scheme::S
    handle::Ptr{Cvoid}
    function GPU(scheme::S; precision = TNR_PREC_F64, seed = 0) where {S <: TNRScheme}
        kind = scheme isa TNRKit.TRG ? TNR_TRG : scheme isa TNRKit.BTRG ? TNR_BTRG :
            scheme isa TNRKit.HOTRG ? TNR_HOTRG : scheme isa TNRKit.HOTRG_3D ? TNR_HOTRG_3D :
            throw(ArgumentError("scheme $(typeof(scheme)) has no GPU path"))
        arr = convert(Array, scheme.T)                 # dense column-major T[i1, i2, ...]
        eltype(arr) <: Real || throw(ArgumentError("the GPU path takes real tensors"))
        dims = Int64[size(arr)...]
        k = scheme isa TNRKit.BTRG ? scheme.k : -0.5
        opts = Ref(Options(precision, k, 1, Ptr{Int32}(C_NULL), UInt64(seed), C_NULL))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:tnr_create, libtnr), Cint,
            (Ptr{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Ref{Options}),
            h, kind, length(dims), dims, Array{Float64}(arr), opts)
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

end # module
