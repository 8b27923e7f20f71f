"""
    TNRKitGB300

Julia binding of the GB300 coarse-graining engine (`libtnr_gb300.so`, C ABI in
`include/tnr_gb300.h`).  It keeps TNRKit's user interface for the hot path:

    using TNRKit, TensorKit, TNRKitGB300
    T = classical_ising(ising_βc)
    scheme = GPU(BTRG(T))                       # tensors move to the GPU once
    data = run!(scheme, truncrank(16), maxiter(25))
    f = free_energy(data, ising_βc)

`GPU(scheme)` wraps a TNRKit `TRG`, `BTRG`, `HOTRG`, `HOTRG_3D`, `ATRG`, `ATRG_3D`,
`ImpurityHOTRG`, `ImpurityTRG` or `CorrelationHOTRG` whose tensors are dense or abelian
(Z_N) TensorMaps; `run!`, `step!` and `finalize!` on the wrapper call the library, which
keeps the tensors resident on the device.  `run!(g, trunc, crit, two_by_two_Finalizer)`
selects the 2 x 2 finalizer; `cft_data`, `ground_state_degeneracy`, `gu_wen_ratio` and
`central_charge` read the fixed-point tensor on the device.  `run_batch!` runs
many wrapped schemes at once, and `Server` is the request loop that admits `run!`
requests by their HBM footprint:

    srv = Server(; precision = TNR_PREC_SPLIT)
    id = submit!(srv, BTRG(T), 32, 30)
    norms, latency_ms, queue_ms = result(srv, id)
"""
module TNRKitGB300

using TensorKit
import TNRKit
import TNRKit: run!, step!, finalize!, free_energy, maxiter, TNRScheme, cft_data, ground_state_degeneracy,
    gu_wen_ratio, central_charge

export GPU, run_batch!, Server, submit!, result, decomposition_stats, TNR_PREC_F64, TNR_PREC_SPLIT

const libtnr = get(ENV, "TNR_GB300_LIB", joinpath(@__DIR__, "..", "libtnr_gb300.so"))

const TNR_TRG, TNR_BTRG, TNR_HOTRG, TNR_HOTRG_3D = 1, 2, 3, 4
const TNR_IMPURITY_HOTRG, TNR_IMPURITY_TRG, TNR_CORRELATION_HOTRG, TNR_ATRG, TNR_ATRG_3D = 5, 6, 7, 8, 9
const TNR_FINALIZER_DEFAULT, TNR_FINALIZER_TWO_BY_TWO = 0, 1
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
    scheme isa TNRKit.ATRG ? TNR_ATRG : scheme isa TNRKit.ATRG_3D ? TNR_ATRG_3D :
    scheme isa TNRKit.ImpurityHOTRG ? TNR_IMPURITY_HOTRG : scheme isa TNRKit.ImpurityTRG ? TNR_IMPURITY_TRG :
    scheme isa TNRKit.CorrelationHOTRG ? TNR_CORRELATION_HOTRG :
    throw(ArgumentError("scheme $(typeof(scheme)) has no GPU path"))

function dense_array(t)
    arr = convert(Array, t)                            # dense column-major t[i1, i2, ...]
    eltype(arr) <: Real || throw(ArgumentError("the GPU path takes real tensors"))
    return Array{Float64}(arr)
end
dense_tensor(scheme) = dense_array(scheme isa TNRKit.CorrelationHOTRG ? scheme.Tpure : scheme.T)

# the impurity tensors in the order of the library's create call
impurity_tensors(s) = s isa TNRKit.ImpurityHOTRG ? (s.T_imp_order1_1, s.T_imp_order1_2, s.T_imp_order2) :
    s isa TNRKit.ImpurityTRG ? (s.T_imp1, s.T_imp2, s.T_imp3, s.T_imp4) : (s.Timp1, s.Timp2)
norms_per_entry(g) = g.kind == TNR_IMPURITY_HOTRG ? 4 : g.kind == TNR_IMPURITY_TRG ? 2 :
    g.kind == TNR_CORRELATION_HOTRG ? 3 : 1

btrg_k(scheme) = scheme isa TNRKit.BTRG ? scheme.k : -0.5

# Z_N charges of a symmetric tensor for the block-sparse path: the charge of every basis
# index of every leg (codomain legs, then domain legs), in the order of the dense embedding
# `convert(Array, t)` (sector by sector, each repeated dim(V, c) times).  A Trivial tensor
# gives (nothing, 1).
zn_order(::Type{TensorKit.ZNIrrep{N}}) where {N} = N
zn_order(::Type) = 1
function leg_charges(t)
    N = zn_order(TensorKit.sectortype(t))
    N > 1 || return nothing, 1
    qs = Int32[]
    for V in (TensorKit.codomain(t)..., TensorKit.domain(t)...)
        for c in TensorKit.sectors(V)
            append!(qs, fill(Int32(mod(c.n, N)), TensorKit.dim(V, c)))
        end
    end
    return qs, N
end

mutable struct GPU{S} <: TNRScheme{Float64, Any}
    scheme::S
    handle::Ptr{Cvoid}
    kind::Int
    function GPU(scheme::S; precision = TNR_PREC_F64, seed = 0) where {S}
        kind = scheme_kind(scheme)
        arr = dense_tensor(scheme)
        dims = Int64[size(arr)...]
        k = btrg_k(scheme)
        opts = Ref(Options(precision, k, 1, Ptr{Int32}(C_NULL), UInt64(seed), C_NULL))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        if kind <= TNR_HOTRG_3D || kind >= TNR_ATRG
            qs, N = leg_charges(scheme isa TNRKit.CorrelationHOTRG ? scheme.Tpure : scheme.T)
            st = GC.@preserve qs begin
                if qs !== nothing
                    opts = Ref(Options(precision, k, N, pointer(qs), UInt64(seed), C_NULL))
                end
                ccall((:tnr_create, libtnr), Cint,
                    (Ptr{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Ref{Options}),
                    h, kind, length(dims), dims, arr, opts)
            end
        else
            imps = map(dense_array, impurity_tensors(scheme))
            if kind == TNR_IMPURITY_HOTRG
                st = ccall((:tnr_create_impurity_hotrg, libtnr), Cint,
                    (Ptr{Ptr{Cvoid}}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Options}),
                    h, dims, arr, imps[1], imps[2], imps[3], opts)
            elseif kind == TNR_IMPURITY_TRG
                st = ccall((:tnr_create_impurity_trg, libtnr), Cint,
                    (Ptr{Ptr{Cvoid}}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                     Ptr{Float64}, Ref{Options}),
                    h, dims, arr, imps[1], imps[2], imps[3], imps[4], opts)
            else
                st = ccall((:tnr_create_correlation_hotrg, libtnr), Cint,
                    (Ptr{Ptr{Cvoid}}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint, Ref{Options}),
                    h, dims, arr, imps[1], imps[2], scheme.dist, opts)
            end
        end
        check(st)
        g = new{S}(scheme, h[], kind)
        finalizer(x -> ccall((:tnr_destroy, libtnr), Cint, (Ptr{Cvoid},), x.handle), g)
        return g
    end
end

function step!(g::GPU, trunc::TensorKit.MatrixAlgebraKit.TruncationByOrder)
    check(ccall((:tnr_step, libtnr), Cint, (Ptr{Cvoid}, Cint), g.handle, trunc.howmany), g.handle)
    return g
end

function finalize!(g::GPU)
    np = norms_per_entry(g)
    if np > 1
        out = Vector{Float64}(undef, 4)
        check(ccall((:tnr_finalize_impurity, libtnr), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.handle, out), g.handle)
        return Tuple(out[1:np])
    end
    n = Ref{Float64}(0)
    check(ccall((:tnr_finalize, libtnr), Cint, (Ptr{Cvoid}, Ref{Float64}), g.handle, n), g.handle)
    return n[]
end

# run!(scheme, truncrank(chi), maxiter(n); finalize_beginning) with the scheme's Finalizer;
# impurity schemes return tuples, CorrelationHOTRG its own run! (no finalize at the beginning)
function run!(g::GPU, trunc, crit::maxiter; finalize_beginning = true, verbosity = 1)
    np = norms_per_entry(g)
    n = Ref{Csize_t}(0)
    if g.kind == TNR_CORRELATION_HOTRG
        out = Vector{Float64}(undef, 3 * crit.n)
        check(ccall((:tnr_run_correlation, libtnr), Cint,
            (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Csize_t, Ref{Csize_t}),
            g.handle, trunc.howmany, crit.n, out, length(out), n), g.handle)
        return [Tuple(out[3i - 2:3i]) for i in 1:n[]]
    end
    cap = max(crit.n, 1) + 1
    out = Vector{Float64}(undef, np * cap)
    if np > 1
        st = ccall((:tnr_run_impurity, libtnr), Cint,
            (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Float64}, Csize_t, Ref{Csize_t}),
            g.handle, trunc.howmany, crit.n, finalize_beginning, out, length(out), n)
    else
        st = ccall((:tnr_run, libtnr), Cint,
            (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Float64}, Csize_t, Ref{Csize_t}),
            g.handle, trunc.howmany, crit.n, finalize_beginning, out, length(out), n)
    end
    check(st, g.handle)
    return np == 1 ? out[1:n[]] : [Tuple(out[np * (i - 1) + 1:np * i]) for i in 1:n[]]
end

# run! with any other stopping criterion (convcrit, a & b): the loop of tnrscheme.jl:39-52 on
# the host, each step and finalize! on the device
function run!(g::GPU, trunc, crit; finalize_beginning = true, verbosity = 1)
    g.kind == TNR_CORRELATION_HOTRG && throw(ArgumentError("CorrelationHOTRG's run! takes maxiter(n)"))
    data = finalize_beginning ? Any[finalize!(g)] : Any[]
    steps = 0
    while true
        step!(g, trunc)
        push!(data, finalize!(g))
        steps += 1
        crit(steps, data) || break
    end
    return [d for d in data]
end

# run! with a Finalizer object: the 2 x 2 finalizer (finalize.jl:151) or the default one
function run!(g::GPU, trunc, crit::maxiter, fin; finalize_beginning = true, verbosity = 1)
    code = fin === TNRKit.two_by_two_Finalizer ? TNR_FINALIZER_TWO_BY_TWO : TNR_FINALIZER_DEFAULT
    check(ccall((:tnr_set_finalizer, libtnr), Cint, (Ptr{Cvoid}, Cint), g.handle, code), g.handle)
    return run!(g, trunc, crit; finalize_beginning, verbosity)
end

# the fixed-point finalizers (cft.jl): eigenvalues of the transfer matrix on the device, the
# sorting and filtering of cft.jl:17-36 and 296-309 on the host
function transfer_eigvals(g::GPU; unitcell = 1)
    n = size(dense_tensor(g.scheme), 2)^unitcell
    re, im = Vector{Float64}(undef, n), Vector{Float64}(undef, n)
    k = Ref{Csize_t}(0)
    check(ccall((:tnr_transfer_eigvals, libtnr), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Csize_t, Ref{Csize_t}), g.handle, unitcell, re, im, n, k),
        g.handle)
    return complex.(re[1:k[]], im[1:k[]])
end

function cft_data(g::GPU; v = 1, unitcell = 1, is_real = true)
    data = sort(transfer_eigvals(g; unitcell); by = x -> abs(x), rev = true)
    data = filter(x -> real(x) > 0 && abs(x) > 1.0e-12, data)
    is_real && (data = real(data))
    return unitcell * (1 / (2π * v)) * log.(data[1] ./ data)
end

function ground_state_degeneracy(g::GPU; unitcell = 1)
    D = transfer_eigvals(g; unitcell)
    p = filter(!iszero, abs.(D ./ sum(D)))
    return exp(-sum(p .* log.(p)))
end

function gu_wen_ratio(g::GPU)
    x1, x2 = Ref{Float64}(0), Ref{Float64}(0)
    check(ccall((:tnr_gu_wen_ratio, libtnr), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Float64}), g.handle, x1, x2),
        g.handle)
    return x1[], x2[]
end

function central_charge(g::GPU, n::Number)
    c = Ref{Float64}(0)
    check(ccall((:tnr_central_charge, libtnr), Cint, (Ptr{Cvoid}, Cdouble, Ref{Float64}), g.handle, n, c), g.handle)
    return c[]
end

"""
    decomposition_stats(g) -> (decompositions, gap_fallbacks, max_iters)

Diagnostic (`tnr_decomposition_stats`, no reference counterpart): truncated decompositions run on
the handle, how many of them the spectral-gap fallback decomposed in full FP64, and the largest
subspace-iteration count.
"""
function decomposition_stats(g::GPU)
    nd, nf, mi = Ref{UInt64}(0), Ref{UInt64}(0), Ref{Cint}(0)
    check(ccall((:tnr_decomposition_stats, libtnr), Cint, (Ptr{Cvoid}, Ref{UInt64}, Ref{UInt64}, Ref{Cint}),
        g.handle, nd, nf, mi), g.handle)
    return Int(nd[]), Int(nf[]), Int(mi[])
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
    qs, N = leg_charges(scheme.T)
    if qs === nothing
        check(ccall((:tnr_server_submit, libtnr), Cint,
            (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Cint, Cint, Cdouble, Ref{UInt64}),
            s.ptr, scheme_kind(scheme), length(dims), dims, arr, chi, maxiter, btrg_k(scheme), id))
    else
        # a Z_N request runs block by block over its charge sectors
        check(ccall((:tnr_server_submit_sym, libtnr), Cint,
            (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Float64}, Cint, Ptr{Int32}, Cint, Cint, Cdouble, Ref{UInt64}),
            s.ptr, scheme_kind(scheme), length(dims), dims, arr, N, qs, chi, maxiter, btrg_k(scheme), id))
    end
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
